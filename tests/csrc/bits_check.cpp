// Checks the bisection bit arithmetic of mc_internal.h against IEEE
// arithmetic on this CPU: mid_bits == (f + t) * 0.5 and float_bits_of ==
// (float)x for doubles that pass bisect_bits_ok, on random and adversarial
// inputs (ties, carries, binade edges, both signs).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "../../model3d_gb300/csrc/mc_internal.h"

using namespace mcgpu;

static unsigned long long bits(double x) {
    unsigned long long b;
    std::memcpy(&b, &x, 8);
    return b;
}
static double dbl(unsigned long long b) {
    double x;
    std::memcpy(&x, &b, 8);
    return x;
}
static uint32_t fbits(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    return b;
}

int main() {
    std::mt19937_64 rng(12345);
    long long checked = 0, bad = 0;
    auto check = [&](double f, double t) {
        const unsigned long long a = bits(f), b = bits(t);
        if (!bisect_bits_ok(a, b)) return;
        checked++;
        volatile double s = f + t;
        const double ref = s * 0.5;
        const unsigned long long m = mid_bits(a, b);
        if (m != bits(ref)) {
            if (bad++ < 5) std::printf("mid %.17g %.17g -> %.17g want %.17g\n", f, t, dbl(m), ref);
        }
        if (float_bits_of(a) != fbits((float)f)) {
            if (bad++ < 5) std::printf("float %.17g -> %08x want %08x\n", f, float_bits_of(a), fbits((float)f));
        }
        if (float_bits_of(m) != fbits((float)dbl(m))) {
            if (bad++ < 5) std::printf("float(mid) %.17g\n", dbl(m));
        }
    };
    std::uniform_int_distribution<int> ex(897, 1150);
    for (int i = 0; i < 4000000; i++) {
        const unsigned long long e = (unsigned long long)ex(rng), sgn = rng() & 1ull;
        const unsigned long long m1 = rng() & kFrac52;
        unsigned long long m2;
        switch (i % 4) {
            case 0: m2 = rng() & kFrac52; break;                          // random
            case 1: m2 = (m1 + (rng() % 7)) & kFrac52; break;             // close: ties
            case 2: m2 = kFrac52 - (rng() % 5); break;                    // top of the binade
            default: m2 = (m1 & ~((1ull << 29) - 1)) | (1ull << 28); break;  // float ties
        }
        check(dbl(sgn << 63 | e << 52 | m1), dbl(sgn << 63 | e << 52 | m2));
    }
    // bisection walks from grid values like a real edge
    for (int i = 0; i < 200000; i++) {
        double lo = std::ldexp((double)(rng() % 2000000) - 1000000.0, -(int)(rng() % 30)) + 0.1;
        double hi = lo + 0.004;
        unsigned long long f = bits(lo), t = bits(hi);
        for (int k = 0; k < 8 && bisect_bits_ok(f, t); k++) {
            check(dbl(f), dbl(t));
            const unsigned long long m = mid_bits(f, t);
            if (rng() & 1) f = m; else t = m;
        }
    }
    std::printf("checked %lld bad %lld\n", checked, bad);
    return bad != 0;
}
