// mc_lower.cpp — host side of the library: lowers the mc_node serialisation
// of a Solid tree into the device program of mc_internal.h, builds the
// marching-cubes case table and the spacer.
//
// Compiled with -ffp-contract=off: every float64 constant precomputed here
// (cylinder direction, capsule segment order, torus basis, inverse
// transforms, per-triangle Moller-Trumbore terms) must equal what the
// reference computes on each call, operation for operation.

#include "mc_lower.h"

#include <algorithm>
#include <atomic>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <stdexcept>
#include <system_error>
#include <thread>

namespace mcgpu {
namespace {

// ---- Go float64 helpers (math.Min / math.Max, model3d/coords.go:440-448).
double gmin(double x, double y) {
    if (std::isinf(x) && x < 0) return x;
    if (std::isinf(y) && y < 0) return y;
    if (std::isnan(x) || std::isnan(y)) return std::numeric_limits<double>::quiet_NaN();
    if (x == 0 && x == y) return std::signbit(x) ? x : y;
    return x < y ? x : y;
}
double gmax(double x, double y) {
    if (std::isinf(x) && x > 0) return x;
    if (std::isinf(y) && y > 0) return y;
    if (std::isnan(x) || std::isnan(y)) return std::numeric_limits<double>::quiet_NaN();
    if (x == 0 && x == y) return std::signbit(x) ? y : x;
    return x > y ? x : y;
}

struct D3 {
    double v[3];
};
D3 d3(double a, double b, double c) { return D3{{a, b, c}}; }
D3 vadd(D3 a, D3 b) { return d3(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
D3 vscale(D3 a, double s) { return d3(a.v[0] * s, a.v[1] * s, a.v[2] * s); }
D3 vsub(D3 a, D3 b) { return vadd(a, vscale(b, -1)); }
D3 vmin3(D3 a, D3 b) { return d3(gmin(a.v[0], b.v[0]), gmin(a.v[1], b.v[1]), gmin(a.v[2], b.v[2])); }
D3 vmax3(D3 a, D3 b) { return d3(gmax(a.v[0], b.v[0]), gmax(a.v[1], b.v[1]), gmax(a.v[2], b.v[2])); }
double vdot(D3 a, D3 b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
D3 vcross(D3 a, D3 b) {
    return d3(a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2],
              a.v[0] * b.v[1] - a.v[1] * b.v[0]);
}
double vnorm(D3 a) { return std::sqrt(a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2]); }
D3 vnormalize(D3 a) { return vscale(a, 1 / vnorm(a)); }
bool veq(D3 a, D3 b) { return a.v[0] == b.v[0] && a.v[1] == b.v[1] && a.v[2] == b.v[2]; }

// Largest double S with sqrt_rn(S) <= R: the predicate sqrt(S) <= R of
// Coord3D.Dist comparisons (model3d/coords.go:272-277) is then S <= TR,
// because sqrt_rn is monotone.  R < 0 or NaN: nothing qualifies (-1).
double sqrt_threshold(double R) {
    if (!(R >= 0)) return -1.0;
    if (std::isinf(R)) return std::numeric_limits<double>::infinity();
    double s = R * R;
    if (std::isinf(s)) s = DBL_MAX;
    while (s > 0 && std::sqrt(s) > R) s = std::nextafter(s, -1.0);
    for (;;) {
        double t = std::nextafter(s, std::numeric_limits<double>::infinity());
        if (std::isinf(t) || std::sqrt(t) > R) break;
        s = t;
    }
    return s;
}

float f_down(double x) {  // largest float <= x
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
    return f;
}
float f_up(double x) {  // smallest float >= x
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}

// OrthoBasis (model3d/coords.go:388-422).
void ortho_basis(D3 c, D3* o1, D3* o2) {
    double ax = std::fabs(c.v[0]), ay = std::fabs(c.v[1]), az = std::fabs(c.v[2]);
    D3 b1 = d3(0, 0, 0);
    if (ax > ay && ax > az) {
        b1.v[0] = c.v[1] / ax;
        b1.v[1] = -c.v[0] / ax;
    } else {
        b1.v[1] = c.v[2];
        b1.v[2] = -c.v[1];
        if (ay > az) {
            b1.v[1] /= ay;
            b1.v[2] /= ay;
        } else {
            b1.v[1] /= az;
            b1.v[2] /= az;
        }
    }
    D3 b2 = d3(b1.v[1] * c.v[2] - b1.v[2] * c.v[1], b1.v[2] * c.v[0] - b1.v[0] * c.v[2],
               b1.v[0] * c.v[1] - b1.v[1] * c.v[0]);
    *o1 = vnormalize(b1);
    *o2 = vnormalize(b2);
}

// math.Ldexp (Go math/ldexp.go): exact for normal results; a subnormal
// result is scaled into range and multiplied by 2^-53 (one rounding).
double go_ldexp(double frac, long exp) {
    if (frac == 0 || std::isinf(frac) || std::isnan(frac)) return frac;
    if (std::fabs(frac) < DBL_MIN) {  // normalize
        frac *= 4503599627370496.0;
        exp -= 52;
    }
    uint64_t x;
    std::memcpy(&x, &frac, 8);
    exp += (long)((x >> 52) & 0x7ff) - 1023;
    if (exp < -1075) return std::copysign(0.0, frac);
    if (exp > 1023) return frac < 0 ? -HUGE_VAL : HUGE_VAL;
    double m = 1;
    if (exp < -1022) {
        exp += 53;
        m = 1.0 / 9007199254740992.0;
    }
    x &= ~(0x7ffull << 52);
    x |= (uint64_t)(exp + 1023) << 52;
    double f;
    std::memcpy(&f, &x, 8);
    return m * f;
}

// Matrix3 inverse (model3d/matrix.go:56-92).
void inverse3(const double* m, double* r) {
    double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                 m[2] * (m[3] * m[7] - m[4] * m[6]);
    double t[9] = {m[4] * m[8] - m[5] * m[7], m[2] * m[7] - m[1] * m[8], m[1] * m[5] - m[2] * m[4],
                   m[5] * m[6] - m[3] * m[8], m[0] * m[8] - m[2] * m[6], m[2] * m[3] - m[0] * m[5],
                   m[3] * m[7] - m[4] * m[6], m[1] * m[6] - m[0] * m[7], m[0] * m[4] - m[1] * m[3]};
    double s = 1 / det;
    for (int i = 0; i < 9; i++) r[i] = t[i] * s;
}

// Widen a culling box: any rounding in a leaf predicate moves its accepted
// set by a few ulps of the coordinates involved; 1e-7 relative is far more.
void widen(double lo[3], double hi[3]) {
    double mag = 0;
    for (int i = 0; i < 3; i++) {
        mag = std::max(mag, std::fabs(lo[i]));
        mag = std::max(mag, std::fabs(hi[i]));
    }
    double m = 1e-9 + 1e-7 * mag;
    for (int i = 0; i < 3; i++) {
        lo[i] -= m;
        hi[i] += m;
    }
}

const D3 kRay = {{0.5224892708603626, 0.10494477243214506, 0.43558938446126527}};  // collisions.go:124

// ---------------------------------------------------------------- colliders

struct Tri {
    D3 p[3];
    D3 mn, mx;
};

struct GItem {
    D3 mn, mx;
    int idx;
};

double bounds_area(D3 mn, D3 mx) {  // bvh.go:289-292
    D3 d = vsub(mx, mn);
    return 2 * (d.v[0] * (d.v[1] + d.v[2]) + d.v[1] * d.v[2]);
}

double multi_area(const GItem* b, size_t n) {  // bvh.go:257-287
    D3 mn = b[0].mn, mx = b[0].mx;
    for (size_t i = 1; i < n; i++)
        for (int a = 0; a < 3; a++) {
            if (b[i].mn.v[a] < mn.v[a]) mn.v[a] = b[i].mn.v[a];
            if (b[i].mx.v[a] > mx.v[a]) mx.v[a] = b[i].mx.v[a];
        }
    return bounds_area(mn, mx);
}

// groupBounders (model3d/bvh.go:135-217).  s[a] holds every item sorted by
// its midpoint along axis a (ties keep input order); a call on the range
// [lo, lo + n) picks the split axis, then stably partitions the two other
// axes' ranges into the lower and upper halves, so that each half's range
// stays sorted along every axis.  No allocation per call.  The two halves
// touch disjoint ranges of s, tmp and out and disjoint items of `lower`, so
// the upper levels run them on two threads; the result does not depend on it.
struct Grouper {
    std::vector<GItem> s[3];
    std::vector<uint8_t> lower;  // by item index: in the lower half of the split being made
    std::vector<GItem> tmp;      // partition scratch, indexed like s

    void rec(size_t lo, size_t n, int* out, int spawn_depth) {
        if (n <= 2) {
            for (size_t i = 0; i < n; i++) out[i] = s[0][lo + i].idx;
            return;
        }
        const size_t mid = n / 2;
        int axis = 0;
        double best = multi_area(&s[0][lo], mid) + multi_area(&s[0][lo + mid], n - mid);
        for (int a = 1; a < 3; a++) {
            double v = multi_area(&s[a][lo], mid) + multi_area(&s[a][lo + mid], n - mid);
            if (v < best) {
                best = v;
                axis = a;
            }
        }
        for (size_t i = 0; i < n; i++) lower[s[axis][lo + i].idx] = i < mid;
        for (int a = 0; a < 3; a++) {
            if (a == axis) continue;
            GItem* v = &s[a][lo];
            GItem* w = &tmp[lo];
            size_t k = 0, m = 0;
            for (size_t i = 0; i < n; i++) {
                if (lower[v[i].idx]) v[k++] = v[i];
                else w[m++] = v[i];
            }
            std::copy(w, w + m, v + k);
        }
        std::thread upper;
        if (spawn_depth > 0 && n >= kParallelGroup) {
            try {
                upper = std::thread([=] { rec(lo + mid, n - mid, out + mid, spawn_depth - 1); });
            } catch (const std::system_error&) {
                // no thread to be had: the caller's thread does both halves
            }
        }
        rec(lo, mid, out, upper.joinable() ? spawn_depth - 1 : 0);
        if (upper.joinable()) upper.join();
        else rec(lo + mid, n - mid, out + mid, 0);
    }
    static constexpr size_t kParallelGroup = 1 << 16;
};

std::vector<int> group_triangles(const bulk_vector<Tri>& t) {  // GroupTriangles, bvh.go:118-133
    const size_t n = t.size();
    std::vector<int> out(n);
    if (n == 0) return out;
    Grouper g;
    // The three axes' orders are independent: one thread each for large sets.
    auto sort_axis = [&](int a) {
        std::vector<std::pair<double, int>> key(n);
        for (size_t i = 0; i < n; i++) key[i] = {vscale(vadd(t[i].mn, t[i].mx), 0.5).v[a], (int)i};
        std::stable_sort(key.begin(), key.end(),
                         [](const std::pair<double, int>& x, const std::pair<double, int>& y) { return x.first < y.first; });
        g.s[a].reserve(n);
        for (size_t i = 0; i < n; i++) {
            const Tri& tr = t[key[i].second];
            g.s[a].push_back(GItem{tr.mn, tr.mx, key[i].second});
        }
    };
    std::thread th[2];
    for (int a = 1; a < 3 && n >= Grouper::kParallelGroup; a++) {
        try {
            th[a - 1] = std::thread(sort_axis, a);
        } catch (const std::system_error&) {
        }
    }
    sort_axis(0);
    for (int a = 1; a < 3; a++) {
        if (th[a - 1].joinable()) th[a - 1].join();
        else sort_axis(a);
    }
    g.lower.assign(n, 0);
    g.tmp.resize(n);
    const unsigned hw = std::thread::hardware_concurrency();
    int depth = 0;  // 2^depth threads at the deepest split level, up to the host's threads
    while (depth < 5 && (2u << depth) <= std::max(1u, hw)) depth++;
    g.rec(0, n, out.data(), depth);
    return out;
}

// GroupedTrianglesToCollider (collisions.go:169-181) over a grouped order:
// the halving tree of the order, where NewJoinedCollider
// (collisions.go:217-253) absorbs a child whose bounds equal its parent's
// (its children take its place, in order).  Internal node k of the
// recursion (post-order numbering, as the recursion creates them) has
// children ch1[k], ch2[k] (>= 0 node, < 0 triangle -(t+1)) and bounds
// mn[k], mx[k]; absorbed[k] marks a node whose bounds equal its parent's.
// Flat arrays instead of a child vector per node; the bounds are computed
// bottom up with the upper levels' halves on two threads.
struct FlatTree {
    const bulk_vector<Tri>& tris;
    const int* order;
    std::vector<D3> mn, mx;
    std::vector<int> ch1, ch2;
    std::vector<uint8_t> absorbed;
    static constexpr size_t kParallel = 1 << 15;

    FlatTree(const bulk_vector<Tri>& t, const int* o, size_t n)
        : tris(t), order(o), mn(n - 1), mx(n - 1), ch1(n - 1), ch2(n - 1), absorbed(n - 1, 0) {}

    D3 bmin(int c) const { return c >= 0 ? mn[c] : tris[-c - 1].mn; }
    D3 bmax(int c) const { return c >= 0 ? mx[c] : tris[-c - 1].mx; }

    // The subtree of positions [lo, lo + n) whose internal nodes take the
    // post-order numbers start .. start + n - 2; returns its reference.
    int build(size_t lo, size_t n, int start, int spawn_depth) {
        if (n == 1) return -(order[lo] + 1);
        const size_t mid = n / 2;
        int c1 = 0, c2 = 0;
        std::thread right;
        if (spawn_depth > 0 && n >= kParallel) {
            try {
                right = std::thread([&] { c2 = build(lo + mid, n - mid, start + (int)mid - 1, spawn_depth - 1); });
            } catch (const std::system_error&) {
            }
        }
        c1 = build(lo, mid, start, right.joinable() ? spawn_depth - 1 : 0);
        if (right.joinable()) right.join();
        else c2 = build(lo + mid, n - mid, start + (int)mid - 1, 0);
        const int k = start + (int)n - 2;
        D3 a = bmin(c1), b = bmax(c1);
        a = vmin3(a, bmin(c2));
        b = vmax3(b, bmax(c2));
        mn[k] = a;
        mx[k] = b;
        ch1[k] = c1;
        ch2[k] = c2;
        for (int c : {c1, c2})
            if (c >= 0 && veq(mn[c], a) && veq(mx[c], b)) absorbed[c] = 1;
        return k;
    }
};

// f(lo, hi) over contiguous chunks of [0, n) on up to 16 host threads, at
// least min_per_thread items a chunk; the caller's thread takes the first
// chunk, and runs any chunk whose thread cannot be created.  Chunks must
// touch disjoint data.
template <class F>
void parallel_chunks(size_t n, size_t min_per_thread, F&& f) {
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t T = std::min<size_t>({hw, 16, n / std::max<size_t>(min_per_thread, 1)});
    if (T <= 1) {
        f((size_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(T);
    for (size_t k = 1; k < T; k++) {
        const size_t lo = n * k / T, hi = n * (k + 1) / T;
        try {
            th.emplace_back([&f, lo, hi] { f(lo, hi); });
        } catch (const std::system_error&) {
            f(lo, hi);
        }
    }
    f((size_t)0, n / T);
    for (std::thread& x : th) x.join();
}

// Runs f(k) for every k in [0, n) on up to 16 host threads, each thread
// taking the next k from a shared counter (tasks of uneven size balance).
// Tasks must touch disjoint data.
template <class F>
void parallel_tasks(size_t n, F&& f) {
    std::atomic<size_t> next{0};
    auto worker = [&] {
        for (size_t k; (k = next.fetch_add(1)) < n;) f(k);
    };
    const size_t T = std::min<size_t>({(size_t)std::max(1u, std::thread::hardware_concurrency()), 16, n});
    std::vector<std::thread> th;
    for (size_t k = 1; k < T; k++) {
        try {
            th.emplace_back(worker);
        } catch (const std::system_error&) {
            break;  // the caller's thread takes what is left
        }
    }
    worker();
    for (std::thread& x : th) x.join();
}

// Sort of distinct 64-bit keys: chunks sorted on host threads, then merged
// pairwise, each round's merges on host threads.  The result is the sorted
// sequence whatever the split.
void parallel_sort_u64(std::vector<uint64_t>& v) {
    const size_t n = v.size();
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    size_t parts = 1;
    while (parts * 2 <= std::min<size_t>(hw, 16) && n / (parts * 2) >= 65536) parts *= 2;
    if (parts == 1) {
        std::sort(v.begin(), v.end());
        return;
    }
    std::vector<size_t> cut(parts + 1);
    for (size_t k = 0; k <= parts; k++) cut[k] = n * k / parts;
    auto run = [&](size_t count, const std::function<void(size_t)>& f) {
        std::vector<std::thread> th;
        for (size_t k = 1; k < count; k++) {
            try {
                th.emplace_back(f, k);
            } catch (const std::system_error&) {
                f(k);
            }
        }
        f(0);
        for (auto& t : th) t.join();
    };
    run(parts, [&](size_t k) { std::sort(v.begin() + cut[k], v.begin() + cut[k + 1]); });
    std::vector<uint64_t> tmp(n);
    std::vector<uint64_t>* src = &v;
    std::vector<uint64_t>* dst = &tmp;
    for (size_t width = 1; width < parts; width *= 2) {
        const size_t merges = (parts + 2 * width - 1) / (2 * width);
        run(merges, [&](size_t m) {
            const size_t a = cut[std::min(parts, 2 * width * m)], b = cut[std::min(parts, 2 * width * m + width)],
                         c = cut[std::min(parts, 2 * width * m + 2 * width)];
            std::merge(src->begin() + a, src->begin() + b, src->begin() + b, src->begin() + c, dst->begin() + a);
        });
        std::swap(src, dst);
    }
    if (src != &v) v.swap(*src);
}

// ---------------------------------------------------------------- ray grid

// Cells and entries of one tree's ray grid (layout and exactness argument at
// RayEnt in mc_internal.h).  Pads: the float projection of a ray origin inside
// the tree's bounds (|coordinate| <= R) errs by less than 5e-7 (R + 1) in a,
// b and t.  The reference's float64 Moller-Trumbore test reports a hit only
// within 50 eps (R + 1)(kappa1 + kappa2) of the triangle, in the projected
// plane and in t, where kappa1 = |v1||v2||D| / |det| bounds the relative
// error of det and kappa2 = max |e| / |e projected| over the edges; the pads
// below are 8 and 20 times larger.  Triangles with 7 eps kappa1 > 1e-3,
// whose det sign the float64 test may get wrong, are tested by every ray.
void build_ray_grid(const bulk_vector<Tri>& t, const std::vector<int>& order, int tri_base, double R,
                    HostProgram* P, TreeD* tree) {
    const double eps = DBL_EPSILON / 2;
    const D3 dh = vnormalize(kRay);
    const double dlen = vnorm(kRay);
    struct Box {
        double alo, ahi, blo, bhi;
        float maxt;
        int tri;
    };
    // Per triangle (position i of the grouped order), on host threads: 0 never
    // hit, 1 a box, 2 tested by every ray, 3 tested by every ray but its
    // extent still counts towards the cell size.  Then boxes, `all` and the
    // extents are collected in triangle order.
    const size_t n = order.size();
    bulk_vector<Box> cand(n);       // read only where kind is 1
    std::vector<uint8_t> kind(n, 0);
    bulk_vector<double> extent(n);  // read only where kind is 1 or 3
    parallel_chunks(n, 16384, [&](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; i++) {
            if (!P->tris[tri_base + i].valid) continue;  // parallel or det == 0: never hit
            const Tri& tr = t[order[i]];
            const D3 v1 = vsub(tr.p[1], tr.p[0]), v2 = vsub(tr.p[2], tr.p[0]);
            const double det = std::fabs(vdot(vcross(kRay, v2), v1));
            const double k1 = vnorm(v1) * vnorm(v2) * dlen / det;
            double k2 = 0;
            for (int e = 0; e < 3; e++) {
                const D3 ev = vsub(tr.p[(e + 1) % 3], tr.p[e]);
                const D3 perp = vsub(ev, vscale(dh, vdot(ev, dh)));
                const double nv = vnorm(ev), np = vnorm(perp);
                if (nv > 0) k2 = std::max(k2, nv / np);
            }
            if (!(7 * eps * k1 <= 1e-3) || !std::isfinite(k2)) {
                kind[i] = 2;
                continue;
            }
            const double pad = (R + 1) * (4e-6 + 1e3 * eps * (k1 + k2));
            Box b{DBL_MAX, -DBL_MAX, DBL_MAX, -DBL_MAX, 0.f, tri_base + (int)i};
            double mt = -DBL_MAX;
            for (int k = 0; k < 3; k++) {
                const D3& v = tr.p[k];
                const double a = v.v[1] - RAYGRID_KY * v.v[0], bb = v.v[2] - RAYGRID_KZ * v.v[0];
                b.alo = std::min(b.alo, a);
                b.ahi = std::max(b.ahi, a);
                b.blo = std::min(b.blo, bb);
                b.bhi = std::max(b.bhi, bb);
                mt = std::max(mt, v.v[0] * RAYGRID_INV_DX);
            }
            extent[i] = std::max(b.ahi - b.alo, b.bhi - b.blo);
            b.alo -= pad;
            b.ahi += pad;
            b.blo -= pad;
            b.bhi += pad;
            b.maxt = f_up(mt + pad * (1 + RAYGRID_INV_DX));
            if (!std::isfinite(b.alo + b.ahi + b.blo + b.bhi)) {
                kind[i] = 3;
                continue;
            }
            cand[i] = b;
            kind[i] = 1;
        }
    });
    // Boxes, the every-ray list and the extents collected in triangle order,
    // with the boxes' bounds: per-chunk counts, offsets, then each chunk
    // writes its own stretch.  The chunks' bounds are combined in chunk
    // order, so each bound is the first of its equal values, as in one pass.
    const size_t nck = n >= 65536 ? std::min<size_t>(16, std::max(1u, std::thread::hardware_concurrency())) : 1;
    std::vector<size_t> nb(nck + 1, 0), na(nck + 1, 0), ns(nck + 1, 0);
    parallel_tasks(nck, [&](size_t c) {
        size_t b = 0, a = 0, z = 0;
        for (size_t i = n * c / nck; i < n * (c + 1) / nck; i++) {
            b += kind[i] == 1;
            a += kind[i] == 2 || kind[i] == 3;
            z += kind[i] == 1 || kind[i] == 3;
        }
        nb[c + 1] = b;
        na[c + 1] = a;
        ns[c + 1] = z;
    });
    for (size_t c = 0; c < nck; c++) {
        nb[c + 1] += nb[c];
        na[c + 1] += na[c];
        ns[c + 1] += ns[c];
    }
    bulk_vector<Box> boxes(nb[nck]);
    std::vector<int> all(na[nck]);
    std::vector<double> sizes(ns[nck]);
    std::vector<std::array<double, 4>> part(nck, std::array<double, 4>{DBL_MAX, -DBL_MAX, DBL_MAX, -DBL_MAX});
    parallel_tasks(nck, [&](size_t c) {
        size_t b = nb[c], a = na[c], z = ns[c];
        std::array<double, 4>& m = part[c];
        for (size_t i = n * c / nck; i < n * (c + 1) / nck; i++) {
            if (kind[i] == 1 || kind[i] == 3) sizes[z++] = extent[i];
            if (kind[i] == 1) {
                const Box& x = cand[i];
                boxes[b++] = x;
                m[0] = std::min(m[0], x.alo);
                m[1] = std::max(m[1], x.ahi);
                m[2] = std::min(m[2], x.blo);
                m[3] = std::max(m[3], x.bhi);
            }
            if (kind[i] == 2 || kind[i] == 3) all[a++] = tri_base + (int)i;
        }
    });
    bulk_vector<Box>().swap(cand);
    double amin = 0, amax = 0, bmin = 0, bmax = 0;
    if (!boxes.empty()) {
        amin = bmin = DBL_MAX;
        amax = bmax = -DBL_MAX;
        for (const auto& m : part) {
            amin = std::min(amin, m[0]);
            amax = std::max(amax, m[1]);
            bmin = std::min(bmin, m[2]);
            bmax = std::max(bmax, m[3]);
        }
    }
    // Cell edge: a quarter of the median triangle extent (measured fastest
    // of 0.25 / 0.35 / 0.5 / 0.7 on a 1M-triangle mesh: ~7 candidate tests
    // per ray), at most 32000 cells per axis and 2^24 cells.
    double cs = 0;
    if (!sizes.empty()) {
        std::nth_element(sizes.begin(), sizes.begin() + sizes.size() / 2, sizes.end());
        cs = 0.25 * sizes[sizes.size() / 2];
    }
    const double ea = amax - amin, eb = bmax - bmin;
    cs = std::max({cs, ea / 32000, eb / 32000, std::sqrt(ea * eb / (double)(1 << 24)), 1e-300});
    if (!(cs > 0) || !std::isfinite(cs)) cs = 1;
    const float inv_f = (float)(1 / cs);
    const double inv = inv_f;
    const float amin_f = f_down(amin), bmin_f = f_down(bmin);
    const int ga = boxes.empty() ? 1 : (int)std::floor((amax - amin_f) * inv) + 1;
    const int gb = boxes.empty() ? 1 : (int)std::floor((bmax - bmin_f) * inv) + 1;
    // The device's float cell index errs by far less than 0.05 cells.
    auto cell_range = [&](double lo, double hi, float org, int n, int* c0, int* c1) {
        *c0 = std::max(0, (int)std::floor((lo - org) * inv - 0.05));
        *c1 = std::min(n - 1, (int)std::floor((hi - org) * inv + 0.05));
    };
    const size_t ncell = (size_t)ga * gb;
    // Each cell lists its boxes by (maxt, triangle), a strict order (a box
    // enters a cell once).  Filling the cells from the boxes in that order
    // leaves every cell sorted without a sort per cell.  The order is sorted
    // as 64-bit keys (order-preserving float bits of maxt, -0 folded into
    // +0, then the triangle), in chunks on host threads merged pairwise.
    {
        std::vector<uint64_t> key(boxes.size());
        parallel_chunks(boxes.size(), 65536, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; i++) {
                uint32_t u;
                const float m = boxes[i].maxt + 0.0f;
                std::memcpy(&u, &m, 4);
                u = (u >> 31) ? ~u : (u | 0x80000000u);
                key[i] = ((uint64_t)u << 32) | (uint32_t)i;  // box index: triangles are in box order
            }
        });
        parallel_sort_u64(key);
        bulk_vector<Box> sorted(boxes.size());
        parallel_chunks(boxes.size(), 65536, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; i++) sorted[i] = boxes[(uint32_t)key[i]];
        });
        boxes.swap(sorted);
    }
    // Counting and filling run on bands of cell rows, each band on one thread.
    // The boxes meeting a band are listed per band first (in the sorted
    // order), so a band walks only its own boxes and writes only its own,
    // contiguous, stretch of the entries.
    const int64_t base = (int64_t)P->ents.size();
    const size_t nband = std::min<size_t>((size_t)gb, boxes.size() >= 65536 ? 256 : 1);
    auto band_of = [&](int row) { return (size_t)row * nband / (size_t)gb; };
    auto band_rows = [&](size_t k, int* r0, int* r1) {
        *r0 = (int)((k * (size_t)gb + nband - 1) / nband);  // first row r with band_of(r) == k
        *r1 = (int)(((k + 1) * (size_t)gb + nband - 1) / nband) - 1;
    };
    // Per band, the indices of its boxes: counts per (chunk, band), offsets,
    // then each chunk writes its boxes at its offsets (order kept).
    const size_t nchunk = boxes.size() >= 65536 ? std::min<size_t>(16, std::max(1u, std::thread::hardware_concurrency())) : 1;
    std::vector<size_t> ccount(nchunk * nband, 0);
    auto box_bands = [&](const Box& b, size_t* k0, size_t* k1) {
        int b0, b1;
        cell_range(b.blo, b.bhi, bmin_f, gb, &b0, &b1);
        if (b0 > b1) return false;
        *k0 = band_of(b0);
        *k1 = band_of(b1);
        return true;
    };
    parallel_tasks(nchunk, [&](size_t c) {
        const size_t lo = boxes.size() * c / nchunk, hi = boxes.size() * (c + 1) / nchunk;
        for (size_t i = lo; i < hi; i++) {
            size_t k0, k1;
            if (box_bands(boxes[i], &k0, &k1))
                for (size_t k = k0; k <= k1; k++) ccount[c * nband + k]++;
        }
    });
    std::vector<size_t> band_start(nband + 1, 0), coff(nchunk * nband);
    {
        size_t at = 0;
        for (size_t k = 0; k < nband; k++) {
            band_start[k] = at;
            for (size_t c = 0; c < nchunk; c++) {
                coff[c * nband + k] = at;
                at += ccount[c * nband + k];
            }
        }
        band_start[nband] = at;
    }
    bulk_vector<uint32_t> band_box(band_start[nband]);
    parallel_tasks(nchunk, [&](size_t c) {
        const size_t lo = boxes.size() * c / nchunk, hi = boxes.size() * (c + 1) / nchunk;
        std::vector<size_t> at(coff.begin() + c * nband, coff.begin() + (c + 1) * nband);
        for (size_t i = lo; i < hi; i++) {
            size_t k0, k1;
            if (box_bands(boxes[i], &k0, &k1))
                for (size_t k = k0; k <= k1; k++) band_box[at[k]++] = (uint32_t)i;
        }
    });
    // Walks the cells of band k that box j (an index into band_box) covers.
    auto band_cells = [&](size_t k, size_t j, auto&& visit) {
        int y_lo, y_hi, a0, a1, b0, b1;
        band_rows(k, &y_lo, &y_hi);
        const Box& b = boxes[band_box[j]];
        cell_range(b.alo, b.ahi, amin_f, ga, &a0, &a1);
        cell_range(b.blo, b.bhi, bmin_f, gb, &b0, &b1);
        b0 = std::max(b0, y_lo);
        b1 = std::min(b1, y_hi);
        for (int y = b0; y <= b1; y++)
            for (int x = a0; x <= a1; x++) visit((size_t)y * ga + x, b);
    };
    // A band's cells are its rows, contiguous: each band zeroes and counts
    // its own cells and sums them.
    bulk_vector<uint32_t> cnt(ncell);
    std::vector<int64_t> band_total(nband + 1, 0);
    parallel_tasks(nband, [&](size_t k) {
        int y_lo, y_hi;
        band_rows(k, &y_lo, &y_hi);
        const size_t c_lo = (size_t)y_lo * ga, c_hi = (size_t)(y_hi + 1) * ga;
        std::fill(cnt.begin() + c_lo, cnt.begin() + c_hi, 0u);
        for (size_t j = band_start[k]; j < band_start[k + 1]; j++)
            band_cells(k, j, [&](size_t c, const Box&) { cnt[c]++; });
        int64_t sum = 0;
        for (size_t c = c_lo; c < c_hi; c++) sum += cnt[c];
        band_total[k] = sum;
    });
    int64_t total = 0;
    for (size_t k = 0; k < nband; k++) {
        const int64_t t = band_total[k];
        band_total[k] = total;
        total += t;
    }
    if (base + total + (int64_t)all.size() >= ((int64_t)1 << 31))
        throw LowerError(MC_ERR_LIMIT, "collider ray grid exceeds 2^31 entries");
    P->ents.resize(base + total);
    tree->cell_base = (int32_t)P->cell_start.size();
    tree->n_cells = (int32_t)ncell;
    const size_t cs0 = P->cell_start.size();
    P->cell_start.resize(cs0 + ncell + 1);
    P->cell_start[cs0 + ncell] = (int32_t)(base + total);
    // Each band turns its counts into cell offsets (from the band's own
    // offset), records them, and fills its cells using the offsets as cursors.
    parallel_tasks(nband, [&](size_t k) {
        int y_lo, y_hi;
        band_rows(k, &y_lo, &y_hi);
        const size_t c_lo = (size_t)y_lo * ga, c_hi = (size_t)(y_hi + 1) * ga;
        uint32_t at = (uint32_t)band_total[k];
        for (size_t c = c_lo; c < c_hi; c++) {
            const uint32_t n_c = cnt[c];
            cnt[c] = at;
            P->cell_start[cs0 + c] = (int32_t)(base + at);
            at += n_c;
        }
        for (size_t j = band_start[k]; j < band_start[k + 1]; j++)
            band_cells(k, j, [&](size_t c, const Box& b) { P->ents[base + cnt[c]++] = RayEnt{b.maxt, b.tri}; });
    });
    tree->all_first = (int32_t)P->ents.size();
    tree->all_count = (int32_t)all.size();
    for (int i : all) P->ents.push_back(RayEnt{INFINITY, i});
    tree->amin = amin_f;
    tree->bmin = bmin_f;
    tree->inv_cs = inv_f;
    tree->ga = ga;
    tree->gb = gb;
}

}  // namespace

// math.Pow(x, y) for integer y (Go math/pow.go): special cases for x = 1,
// NaN and +Inf, then x = x1 * 2^xe by Frexp, the product of x1 powers over
// the bits of |y| by repeated squaring renormalised to [0.5, 1), one
// reciprocal for y < 0, and Ldexp.
double go_pow_int(double x, long y) {
    if (y == 0 || x == 1) return 1;
    if (y == 1) return x;
    if (std::isnan(x)) return x;
    if (std::isinf(x) && x > 0) return y < 0 ? 0.0 : HUGE_VAL;
    if (!(x > 0)) throw LowerError(MC_ERR_BAD_PROGRAM, "go_pow_int: x must be positive");
    double a1 = 1;
    long ae = 0;
    int xe_i;
    double x1 = std::frexp(x, &xe_i);
    long xe = xe_i;
    for (long i = y < 0 ? -y : y; i != 0; i >>= 1) {
        if (xe < -(1 << 12) || (1 << 12) < xe) {
            ae += xe;
            break;
        }
        if (i & 1) {
            a1 *= x1;
            ae += xe;
        }
        x1 *= x1;
        xe <<= 1;
        if (x1 < .5) {
            x1 += x1;
            xe--;
        }
    }
    if (y < 0) {
        a1 = 1 / a1;
        ae = -ae;
    }
    return go_ldexp(a1, ae);
}

namespace {

// ---------------------------------------------------------------- lowering

struct Lowerer {
    const mc_node* nodes;
    size_t n;
    const mc_tri_set* sets;
    size_t n_sets;
    HostProgram* P;
    size_t pos = 0;
    int depth = 0, xdepth = 0;
    std::map<int, int> tree_of_set;

    void fail(const std::string& m) { throw LowerError(MC_ERR_BAD_PROGRAM, m); }

    void emit(uint32_t op) {
        if ((int)P->ops.size() >= MAX_OPS) throw LowerError(MC_ERR_LIMIT, "program too long");
        P->ops.push_back(op);
    }
    void leaf_out(int id) {
        last_leaf = id;
        if (emit_leaves) {
            emit(make_op(OP_LEAF, id));
            push_bool();
        }
    }
    void push_bool() {
        depth++;
        P->max_stack = std::max(P->max_stack, depth);
        if (depth > MAX_STACK) throw LowerError(MC_ERR_LIMIT, "solid tree too deep");
    }

    int add_leaf(int kind, const double* d, int nd, const float* f, int nf, const double cull[6]) {
        int id = (int)P->leaf_kind.size();
        P->leaf_kind.push_back(kind);
        size_t bd = P->leaf_d.size(), bf = P->leaf_f.size();
        P->leaf_d.resize(bd + LEAF_D, 0.0);
        P->leaf_f.resize(bf + LEAF_F, 0.0f);
        for (int i = 0; i < nd; i++) P->leaf_d[bd + i] = d[i];
        for (int i = 0; i < nf; i++) P->leaf_f[bf + i] = f[i];
        for (int i = 0; i < 6; i++) {
            P->cull.push_back(cull[i]);
            P->cull_f.push_back(i < 3 ? f_down(cull[i]) : f_up(cull[i]));
        }
        return id;
    }

    // WeightedMetaballSolid: one LK_METABALL leaf over the ball records.
    template <class SetCull>
    void lower_metaball(const mc_node& nd, SetCull& set_cull, double* cull) {
        if (nd.n_children < 0) fail("negative ball count");
        if (nd.n_children > MAX_BALLS) throw LowerError(MC_ERR_LIMIT, "more than 4096 metaballs");
        const int falloff = (int)nd.p[1];
        const double param = nd.p[2];
        if (falloff == MC_FALLOFF_POWER) {
            if (!(param >= 1 && param < (1 << 20)) || param != std::floor(param))
                throw LowerError(MC_ERR_NOT_LOWERABLE, "falloff power must be an integer in [1, 2^20)");
        } else if (falloff == MC_FALLOFF_WYVILL) {
            if (!(param > 0)) fail("WyvillMetaballFalloffFunc needs d > 0");
        } else {
            throw LowerError(MC_ERR_NOT_LOWERABLE, "metaball falloff has no device lowering");
        }
        MetaD md{};
        MetaF mf{};
        md.falloff = falloff;
        md.param = param;
        md.d2 = param * param;
        // threshold := f(radiusThreshold) (metaball.go:180)
        const double rt = nd.p[0];
        double thr;
        if (falloff == MC_FALLOFF_POWER) {
            thr = rt <= 0 ? HUGE_VAL : go_pow_int(rt, -(long)param);
        } else if (rt < 0) {
            thr = HUGE_VAL;
        } else if (rt >= param) {
            thr = 0;
        } else {
            double ratio2 = (rt * rt) / md.d2;
            double value = 1 - ratio2;
            thr = value * value;
        }
        md.thr = thr;
        md.never = thr < HUGE_VAL ? 0 : 1;  // +Inf or NaN
        for (int i = 0; i < 3; i++) {
            md.lo[i] = nd.min[i];
            md.hi[i] = nd.max[i];
            mf.lo_dn[i] = f_down(nd.min[i]);
            mf.lo_up[i] = f_up(nd.min[i]);
            mf.hi_dn[i] = f_down(nd.max[i]);
            mf.hi_up[i] = f_up(nd.max[i]);
        }
        mf.thr_lo = f_down(thr);
        mf.thr_hi = f_up(thr);
        mf.d_lo = f_down(param);
        mf.d_hi = f_up(param);
        {  // 1 / d2 rounded in float64 (relative error 2^-53), then widened and rounded outward
            const double inv = 1 / md.d2;
            mf.inv_d2_lo = f_down(inv * (1 - 0x1p-50));
            mf.inv_d2_hi = f_up(inv * (1 + 0x1p-50));
        }
        mf.k = falloff == MC_FALLOFF_POWER ? (int32_t)param : 0;
        // r^k by binary powering: squarings double the relative error, so at
        // most (k + popcount(k)) u <= 2k u, then 2 ulp (4u) for __fdividef.
        mf.eps_pow = (float)((2.0 * mf.k + 6.0) * 0x1p-24 * 1.5);
        mf.esc_all = falloff == MC_FALLOFF_WYVILL && !(md.d2 > 1e-30 && md.d2 < 1e30) ? 1 : 0;
        md.first_ball = (int32_t)P->balls.size();
        md.n_balls = nd.n_children;
        bool any_pos = false;
        for (int i = 0; i < nd.n_children; i++) {
            if (pos >= n || nodes[pos].kind != MC_NODE_BALL) fail("metaball child is not a MC_NODE_BALL");
            const mc_node& bn = nodes[pos++];
            if (bn.n_children != 1) fail("MC_NODE_BALL needs one primitive child");
            const int ns = std::max(bn.n_steps, 0);
            if (pos + (size_t)ns > n) fail("truncated ball transform steps");
            const std::vector<XStepD> inv = transform_steps(nodes + pos, ns, true);
            pos += ns;
            if (pos >= n) fail("truncated ball");
            const mc_node& pr = nodes[pos++];
            BallD bd{};
            BallF bf{};
            bd.w = bn.p[0];
            any_pos = any_pos || bd.w > 0;
            bd.first_step = (int32_t)P->xstep.size();
            bd.n_steps = (int32_t)inv.size();
            P->xstep.insert(P->xstep.end(), inv.begin(), inv.end());
            auto pp = [&](int o) { return d3(pr.p[o], pr.p[o + 1], pr.p[o + 2]); };
            auto put = [&](int o, D3 v) {
                for (int k = 0; k < 3; k++) bd.c[o + k] = v.v[k];
            };
            int nc = 0, nf = 0;  // double and float constant counts
            double fc[BALL_C] = {0};  // float constants before rounding
            D3 A = d3(0, 0, 0);
            // kint: the kind's own rounding error bound in units of u times
            // (|q| + mag + |r|) (see ball_field_32): sphere 2.5 n + R + |r| with
            // n <= |r| + R; rect 1.74 mag + 4.24 |r|; capsule 3.74 norm + 8.3 |q| +
            // 5.24 (R + |r|); the cylinder's caps add projections on rounded
            // bases; the torus adds the ring direction (<= 11.4 e_xy beyond
            // outer/64 of its axis).
            double kint = 5;
            switch (pr.kind) {
                case MC_NODE_SPHERE:
                    put(0, pp(0));
                    bd.c[3] = pr.p[3];
                    nc = 4;
                    A = pp(0);
                    fc[0] = pr.p[3];
                    nf = 1;
                    break;
                case MC_NODE_RECT: {
                    put(0, pp(0));
                    put(3, pp(3));
                    nc = 6;
                    A = vscale(vadd(pp(0), pp(3)), 0.5);
                    for (int k = 0; k < 3; k++) {
                        fc[k] = pr.p[k] - A.v[k];
                        fc[3 + k] = pr.p[3 + k] - A.v[k];
                    }
                    nf = 6;
                    kint = 6;
                    break;
                }
                case MC_NODE_CAPSULE:
                case MC_NODE_CYLINDER: {  // shapes.go:481-484, :747-749
                    D3 p1 = pp(0), p2 = pp(3);
                    D3 v = vsub(p2, p1);
                    double nrm = vnorm(v);
                    D3 axis = vscale(v, 1 / nrm);
                    put(0, p1);
                    put(3, p2);
                    put(6, axis);
                    bd.c[9] = nrm;
                    bd.c[10] = pr.p[6];
                    nc = 11;
                    A = p1;
                    for (int k = 0; k < 3; k++) {
                        fc[k] = p2.v[k] - p1.v[k];
                        fc[3 + k] = axis.v[k];
                    }
                    fc[6] = nrm;
                    fc[7] = pr.p[6];
                    nf = 8;
                    kint = 10;
                    if (pr.kind == MC_NODE_CYLINDER) {  // filledCircleDist bases, shapes.go:775-776
                        D3 b1, b2;
                        ortho_basis(vscale(axis, -1), &b1, &b2);
                        put(11, b1);
                        put(14, b2);
                        for (int k = 0; k < 3; k++) fc[8 + k] = b1.v[k], fc[11 + k] = b2.v[k];
                        ortho_basis(axis, &b1, &b2);
                        put(17, b1);
                        put(20, b2);
                        for (int k = 0; k < 3; k++) fc[14 + k] = b1.v[k], fc[17 + k] = b2.v[k];
                        nc = 23;
                        nf = 20;
                        kint = 40;
                    }
                    break;
                }
                case MC_NODE_TORUS: {  // shapes.go:1451-1487
                    D3 b1, b2;
                    ortho_basis(pp(3), &b1, &b2);
                    put(0, pp(0));
                    put(3, b1);
                    put(6, b2);
                    bd.c[9] = pr.p[6];
                    bd.c[10] = pr.p[7];
                    nc = 11;
                    A = pp(0);
                    for (int k = 0; k < 3; k++) fc[k] = b1.v[k], fc[3 + k] = b2.v[k];
                    fc[6] = pr.p[6];
                    fc[7] = pr.p[7];
                    nf = 8;
                    kint = 128;
                    break;
                }
                default: fail("a ball's primitive must be a sphere, rect, cylinder, capsule or torus");
            }
            (void)nc;
            double mag = 0;
            for (int k = 0; k < nf; k++) {
                bf.c[k] = (float)fc[k];
                mag = std::max(mag, std::fabs(fc[k]));
            }
            bf.mag = f_up(mag);
            bf.kint = (float)(kint * 0x1p-24);
            float am = 0;
            for (int k = 0; k < 3; k++) {
                bf.a[k] = (float)A.v[k];
                am = std::max(am, std::fabs(bf.a[k]));
            }
            bf.amag = am;
            bd.kind = pr.kind;
            bf.kind = pr.kind;
            bf.n_steps = bd.n_steps;
            bf.w_lo = f_down(bd.w);
            bf.w_hi = f_up(bd.w);
            P->balls.push_back(bd);
            P->balls_f.push_back(bf);
        }
        if (!any_pos) {  // NewRect(Origin, Origin) (metaball.go:186-188)
            P->balls.resize(md.first_ball);
            P->balls_f.resize(md.first_ball);
            double d[6] = {0, 0, 0, 0, 0, 0};
            float f[6] = {0, 0, 0, 0, 0, 0};
            set_cull(d3(0, 0, 0), d3(0, 0, 0));
            leaf_out(add_leaf(LK_RECT, d, 6, f, 6, cull));
            return;
        }
        double d[1] = {(double)P->metas.size()};
        float f[1] = {0};
        P->metas.push_back(md);
        P->metas_f.push_back(mf);
        set_cull(d3(nd.min[0], nd.min[1], nd.min[2]), d3(nd.max[0], nd.max[1], nd.max[2]));
        leaf_out(add_leaf(LK_METABALL, d, 1, f, 1, cull));
    }

    int lower_collider(int set) {
        auto it = tree_of_set.find(set);
        if (it != tree_of_set.end()) return it->second;
        const mc_tri_set& ts = sets[set];
        if (ts.n < 0 || (ts.n > 0 && !ts.tris)) fail("bad triangle set");
        bulk_vector<Tri> t(ts.n);
        parallel_chunks(t.size(), 65536, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; i++) {
                for (int k = 0; k < 3; k++)
                    t[i].p[k] = d3(ts.tris[i * 9 + 3 * k], ts.tris[i * 9 + 3 * k + 1], ts.tris[i * 9 + 3 * k + 2]);
                t[i].mn = vmin3(vmin3(t[i].p[0], t[i].p[1]), t[i].p[2]);  // Triangle.Min, primitives.go:36-38
                t[i].mx = vmax3(vmax3(t[i].p[0], t[i].p[1]), t[i].p[2]);
            }
        });
        std::vector<int> order;
        if (ts.grouped) {
            order.resize(ts.n);
            for (int64_t i = 0; i < ts.n; i++) order[i] = (int)i;
        } else {
            order = group_triangles(t);
        }
        TreeD tree{};
        int tri_base = (int)P->tris.size();
        std::vector<int> pos_of(ts.n);
        for (size_t i = 0; i < order.size(); i++) pos_of[order[i]] = (int)i;
        // Triangle records in grouped order (traversal locality), on host threads.
        P->tris.resize(tri_base + order.size());
        P->tris_f.resize(tri_base + order.size());
        D3 dn = vnormalize(kRay);
        parallel_chunks(order.size(), 16384, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; i++) {
                const Tri& tr = t[order[i]];
                TriD d{};
                TriF f{};
                D3 v1 = vsub(tr.p[1], tr.p[0]);
                D3 v2 = vsub(tr.p[2], tr.p[0]);
                D3 nrm = vnormalize(vcross(v1, v2));      // Triangle.Normal, primitives.go:27-33
                double dd = vdot(nrm, dn);                 // primitives.go:208
                bool parallel = dd < 1e-8 && dd > -1e-8;
                D3 c1 = vcross(kRay, v2);                  // primitives.go:219
                double det = vdot(c1, v1);                 // primitives.go:220
                double inv = 1 / det;                      // primitives.go:227
                for (int k = 0; k < 3; k++) {
                    d.t0[k] = tr.p[0].v[k];
                    d.v1[k] = v1.v[k];
                    d.v2[k] = v2.v[k];
                    d.c1[k] = c1.v[k];
                    f.t0[k] = (float)d.t0[k];
                    f.v1[k] = (float)d.v1[k];
                    f.v2[k] = (float)d.v2[k];
                    f.c1[k] = (float)d.c1[k];
                }
                d.inv_det = inv;
                d.valid = (!parallel && det != 0) ? 1 : 0;
                f.inv_det = (float)inv;
                f.valid = d.valid;
                P->tris[tri_base + i] = d;
                P->tris_f[tri_base + i] = f;
            }
        });
        P->tri_parent.resize(P->tris.size(), -1);
        if (ts.n > 1) {
            FlatTree ft(t, order.data(), order.size());
            const unsigned hw = std::thread::hardware_concurrency();
            int depth = 0;  // 2^depth threads at the deepest split, up to the host's threads
            while (depth < 4 && (2u << depth) <= std::max(1u, hw)) depth++;
            const int root = ft.build(0, order.size(), 0, depth);
            int node_base = (int)P->nodes.size();
            // Breadth first over the surviving nodes; a node's children are its
            // two subtrees' references, an absorbed node replaced by its own
            // children, in order (a stack of pending references).
            std::vector<int> queue = {root};
            queue.reserve(order.size());
            std::vector<int> stack;
            for (size_t qi = 0; qi < queue.size(); qi++) {
                const int u = queue[qi];
                stack.assign({ft.ch2[u], ft.ch1[u]});
                while (!stack.empty()) {
                    const int c = stack.back();
                    stack.pop_back();
                    if (c < 0) {
                        P->tri_parent[tri_base + pos_of[-c - 1]] = node_base + (int)qi;
                    } else if (ft.absorbed[c]) {
                        stack.push_back(ft.ch2[c]);
                        stack.push_back(ft.ch1[c]);
                    } else {
                        queue.push_back(c);
                    }
                }
            }
            P->nodes.resize(node_base + queue.size());
            P->nodes_f.resize(node_base + queue.size());
            parallel_chunks(queue.size(), 65536, [&](size_t lo, size_t hi) {
                for (size_t qi = lo; qi < hi; qi++) {
                    const int u = queue[qi];
                    BvhNodeD nd{};
                    BvhNodeF nf{};
                    for (int k = 0; k < 3; k++) {
                        nd.lo[k] = ft.mn[u].v[k];
                        nd.hi[k] = ft.mx[u].v[k];
                        nf.lo[k] = f_down(ft.mn[u].v[k]);
                        nf.hi[k] = f_up(ft.mx[u].v[k]);
                    }
                    P->nodes[node_base + qi] = nd;
                    P->nodes_f[node_base + qi] = nf;
                }
            });
        }
        tree.kind = ts.n > 0 ? 1 : 0;
        // Coordinate magnitude bound for the FP32 ray-box filter and the pads.
        double R = 0;
        {
            // Per-axis maxima of |coordinate| over every box, in chunks on
            // host threads (max is exact in any order).
            std::vector<std::array<double, 3>> part(16, std::array<double, 3>{0, 0, 0});
            std::atomic<int> next{0};
            parallel_chunks(t.size(), 65536, [&](size_t lo, size_t hi) {
                std::array<double, 3> m{0, 0, 0};
                for (size_t i = lo; i < hi; i++)
                    for (int a = 0; a < 3; a++)
                        m[a] = std::max(m[a], std::max(std::fabs(t[i].mn.v[a]), std::fabs(t[i].mx.v[a])));
                part[next++] = m;
            });
            for (int a = 0; a < 3; a++) {
                double m = 0;
                for (const auto& q : part) m = std::max(m, q[a]);
                tree.mbox[a] = f_up(m);
                R = std::max(R, m);
            }
        }
        build_ray_grid(t, order, tri_base, R, P, &tree);
        int id = (int)P->trees.size();
        P->trees.push_back(tree);
        tree_of_set[set] = id;
        return id;
    }

    // Lower one node (and its subtree); outer = index of the outermost
    // enclosing TRANSFORM box (-1 if none) for culling.
    // End (exclusive) of the serialised subtree starting at record p.
    size_t subtree_end(size_t p) {
        if (p >= n) fail("truncated node array");
        const mc_node& nd = nodes[p];
        size_t q = p + 1 + ((nd.kind == MC_NODE_TRANSFORM || nd.kind == MC_NODE_BALL)
                                ? (size_t)std::max(0, nd.n_steps) : 0);
        int nc = (nd.kind >= MC_NODE_JOIN && nd.kind <= MC_NODE_CHECKED) || nd.kind == MC_NODE_METABALL ||
                         nd.kind == MC_NODE_BALL
                     ? nd.n_children : 0;
        if (nc < 0) fail("negative child count");
        for (int i = 0; i < nc; i++) q = subtree_end(q);
        return q;
    }
    static bool is_leaf_kind(int k) { return k >= MC_NODE_SPHERE && k <= MC_NODE_METABALL; }

    int last_leaf = -1;
    bool emit_leaves = true;

    void lower(int outer) {
        if (pos >= n) fail("truncated node array");
        const mc_node& nd = nodes[pos++];
        auto pv = [&](int o) { return d3(nd.p[o], nd.p[o + 1], nd.p[o + 2]); };
        double cull[6];
        auto set_cull = [&](D3 lo, D3 hi) {
            if (outer >= 0) {
                for (int i = 0; i < 3; i++) {
                    cull[i] = P->xbox[outer].lo[i];
                    cull[3 + i] = P->xbox[outer].hi[i];
                }
            } else {
                for (int i = 0; i < 3; i++) {
                    cull[i] = lo.v[i];
                    cull[3 + i] = hi.v[i];
                }
            }
            widen(cull, cull + 3);
        };
        switch (nd.kind) {
            case MC_NODE_SPHERE: {  // shapes.go:29-31
                D3 c = pv(0);
                double R = nd.p[3];
                double d[4] = {c.v[0], c.v[1], c.v[2], sqrt_threshold(R)};
                float f[6] = {(float)c.v[0], (float)c.v[1], (float)c.v[2], 0, f_down(d[3]), f_up(d[3])};
                set_cull(vsub(c, d3(R, R, R)), vadd(c, d3(R, R, R)));
                if (!(R >= 0)) for (double& x : cull) x = 0;  // contains nothing: any box
                int id = add_leaf(LK_SPHERE, d, 4, f, 6, cull);
                leaf_out(id);
                return;
            }
            case MC_NODE_RECT: {  // shapes.go:171-173
                D3 lo = pv(0), hi = pv(3);
                double d[6] = {lo.v[0], lo.v[1], lo.v[2], hi.v[0], hi.v[1], hi.v[2]};
                float f[6];
                for (int i = 0; i < 6; i++) f[i] = (float)d[i];
                set_cull(lo, hi);
                int id = add_leaf(LK_RECT, d, 6, f, 6, cull);
                leaf_out(id);
                return;
            }
            case MC_NODE_CYLINDER: {  // shapes.go:588-598
                D3 p1 = pv(0), p2 = pv(3);
                double R = nd.p[6];
                D3 diff = vsub(p1, p2);
                D3 dir = vnormalize(diff);
                double nrm = vnorm(diff);
                double TR = sqrt_threshold(R);
                double d[8] = {p2.v[0], p2.v[1], p2.v[2], dir.v[0], dir.v[1], dir.v[2], nrm, TR};
                float f[12] = {(float)p2.v[0], (float)p2.v[1], (float)p2.v[2], (float)dir.v[0],
                               (float)dir.v[1], (float)dir.v[2], f_down(nrm), f_up(nrm),
                               f_down(TR), f_up(TR), 0, 0};
                set_cull(vsub(vmin3(p1, p2), d3(R, R, R)), vadd(vmax3(p1, p2), d3(R, R, R)));
                int id = add_leaf(LK_CYLINDER, d, 8, f, 12, cull);
                leaf_out(id);
                return;
            }
            case MC_NODE_CAPSULE: {  // shapes.go:365-368, primitives.go:547-594
                D3 p1 = pv(0), p2 = pv(3);
                double R = nd.p[6];
                bool keep = p1.v[0] < p2.v[0] || (p1.v[0] == p2.v[0] && p1.v[1] < p2.v[1]) ||
                            (p1.v[0] == p2.v[0] && p1.v[1] == p2.v[1] && p1.v[2] < p2.v[2]);
                D3 s0 = keep ? p1 : p2, s1 = keep ? p2 : p1;
                D3 v1 = vsub(s1, s0);
                double nrm = vnorm(v1);
                D3 v = vscale(v1, 1 / nrm);
                double TR = sqrt_threshold(R);
                double d[11] = {s0.v[0], s0.v[1], s0.v[2], s1.v[0], s1.v[1], s1.v[2],
                                v.v[0],  v.v[1],  v.v[2],  nrm,     TR};
                float f[15];
                for (int i = 0; i < 9; i++) f[i] = (float)d[i];
                f[9] = f_down(nrm);
                f[10] = f_up(nrm);
                f[11] = f_down(TR);
                f[12] = f_up(TR);
                f[13] = f[14] = 0;
                set_cull(vsub(vmin3(p1, p2), d3(R, R, R)), vadd(vmax3(p1, p2), d3(R, R, R)));
                int id = add_leaf(LK_CAPSULE, d, 11, f, 15, cull);
                leaf_out(id);
                return;
            }
            case MC_NODE_TORUS: {  // shapes.go:1363-1365, :1451-1487
                D3 c = pv(0), axis = pv(3);
                double outer_r = nd.p[6], inner = nd.p[7];
                D3 b1, b2;
                ortho_basis(axis, &b1, &b2);
                double Ti = std::isinf(inner) && inner > 0 ? DBL_MAX : sqrt_threshold(inner);
                double d[11] = {c.v[0],  c.v[1],  c.v[2],  b1.v[0], b1.v[1], b1.v[2],
                                b2.v[0], b2.v[1], b2.v[2], outer_r, Ti};
                float f[13];
                for (int i = 0; i < 11; i++) f[i] = (float)d[i];
                f[11] = f_down(Ti);  // threshold bounds of the FP32 filter
                f[12] = f_up(Ti);
                double ext = std::fabs(outer_r) + std::fabs(inner);
                set_cull(vsub(c, d3(ext, ext, ext)), vadd(c, d3(ext, ext, ext)));
                int id = add_leaf(LK_TORUS, d, 11, f, 13, cull);
                leaf_out(id);
                return;
            }
            case MC_NODE_COLLIDER: {  // solid.go:292-305
                if (nd.mesh < 0 || (size_t)nd.mesh >= n_sets) fail("bad mesh index");
                int tree = lower_collider(nd.mesh);
                double d[7] = {nd.min[0], nd.min[1], nd.min[2], nd.max[0], nd.max[1], nd.max[2], (double)tree};
                float f[1] = {0};
                set_cull(d3(nd.min[0], nd.min[1], nd.min[2]), d3(nd.max[0], nd.max[1], nd.max[2]));
                int id = add_leaf(LK_COLLIDER, d, 7, f, 1, cull);
                P->has_collider = true;
                leaf_out(id);
                return;
            }
            case MC_NODE_METABALL: {  // metaball.go:165-242
                lower_metaball(nd, set_cull, cull);
                return;
            }
            case MC_NODE_JOIN:
            case MC_NODE_INTERSECT: {  // solid.go:89-98, :165-172
                if (nd.n_children < 1) fail("JoinedSolid/IntersectedSolid without children");
                // OR / AND are commutative: the leaf children get consecutive
                // ids and one range op, then the other children follow.
                const uint32_t op = nd.kind == MC_NODE_JOIN ? OP_OR : OP_AND;
                const uint32_t rop = nd.kind == MC_NODE_JOIN ? OP_JLEAVES : OP_ALEAVES;
                std::vector<size_t> starts;
                size_t q = pos;
                for (int i = 0; i < nd.n_children; i++) {
                    starts.push_back(q);
                    q = subtree_end(q);
                }
                const size_t end = q;
                int first = -1, count = 0, have = 0;
                for (size_t st : starts) {
                    if (!is_leaf_kind(nodes[st].kind)) continue;
                    pos = st;
                    bool saved = emit_leaves;
                    emit_leaves = false;
                    lower(outer);
                    emit_leaves = saved;
                    if (first < 0) first = last_leaf;
                    count++;
                }
                if (count > 0) {
                    if (first >= (1 << 14) || count >= (1 << 14))
                        throw LowerError(MC_ERR_LIMIT, "more than 16383 leaves");
                    emit(make_op(rop, ((uint32_t)first << 14) | (uint32_t)count));
                    push_bool();
                    have = 1;
                }
                for (size_t st : starts) {
                    if (is_leaf_kind(nodes[st].kind)) continue;
                    pos = st;
                    lower(outer);
                    if (have) {
                        emit(make_op(op, 0));
                        depth--;
                    }
                    have = 1;
                }
                pos = end;
                return;
            }
            case MC_NODE_SUBTRACT: {  // solid.go:138-141
                if (nd.n_children != 2) fail("SubtractedSolid needs two children");
                lower(outer);
                lower(outer);
                emit(make_op(OP_ANDNOT, 0));
                depth--;
                return;
            }
            case MC_NODE_TRANSFORM: {  // transform.go:240-247
                if (nd.n_children != 1) fail("TransformSolid needs one child");
                XBoxD xb{};
                for (int i = 0; i < 3; i++) {
                    xb.lo[i] = nd.min[i];
                    xb.hi[i] = nd.max[i];
                }
                if (pos + (size_t)std::max(nd.n_steps, 0) > n) fail("truncated transform steps");
                const std::vector<XStepD> inv = transform_steps(nodes + pos, std::max(nd.n_steps, 0), true);
                pos += std::max(nd.n_steps, 0);
                xb.first_step = (int)P->xstep.size();
                xb.n_steps = (int)inv.size();
                P->xstep.insert(P->xstep.end(), inv.begin(), inv.end());
                int id = (int)P->xbox.size();
                P->xbox.push_back(xb);
                P->has_transform = true;
                emit(make_op(OP_XPUSH, id));
                if (++xdepth > MAX_XDEPTH) throw LowerError(MC_ERR_LIMIT, "transforms nested too deeply");
                P->max_xdepth = std::max(P->max_xdepth, xdepth);
                lower(outer >= 0 ? outer : id);
                xdepth--;
                emit(make_op(OP_XPOP, id));
                return;
            }
            case MC_NODE_CHECKED: {  // solid.go:46-50
                if (nd.n_children != 1) fail("CheckedFuncSolid needs one child");
                XBoxD xb{};
                for (int i = 0; i < 3; i++) {
                    xb.lo[i] = nd.min[i];
                    xb.hi[i] = nd.max[i];
                }
                xb.first_step = 0;
                xb.n_steps = 0;
                int id = (int)P->xbox.size();
                P->xbox.push_back(xb);
                lower(outer);
                emit(make_op(OP_BOXAND, id));
                return;
            }
            default: throw LowerError(MC_ERR_NOT_LOWERABLE, "node kind has no device lowering");
        }
    }
};

}  // namespace

void lower_scene(const mc_node* nodes, size_t n_nodes, const mc_tri_set* sets, size_t n_sets,
                 HostProgram* P) {
    *P = HostProgram();
    if (!nodes || n_nodes == 0) throw LowerError(MC_ERR_ARG, "empty node array");
    Lowerer L{nodes, n_nodes, sets, n_sets, P, 0, 0, 0, {}};
    L.lower(-1);
    if (L.pos != n_nodes) throw LowerError(MC_ERR_BAD_PROGRAM, "trailing nodes after the root");
    for (int i = 0; i < 3; i++) {
        P->root_min[i] = nodes[0].min[i];
        P->root_max[i] = nodes[0].max[i];
    }
    P->ops_allfalse.resize(P->ops.size() + 1);
    P->n_ops_allfalse = fold_program(P->ops.data(), (int)P->ops.size(), nullptr, P->ops_allfalse.data());
    P->fold_cap = 0;
    for (uint32_t op : P->ops) {
        uint32_t c = op_code(op);
        P->fold_cap += (c == OP_JLEAVES || c == OP_ALEAVES) ? 1 + (int)range_count(op_arg(op)) : 1;
    }
}

// ---------------------------------------------------------------- spacer

int spacer_axis(double lo, double hi, double delta, std::vector<double>* out, int64_t limit) {
    out->clear();
    if (!(delta > 0) || std::isinf(delta)) return MC_ERR_GRID;
    // for x := min - delta; x <= max + delta; x += delta (model3d/mc.go:598-600)
    for (double x = lo - delta; x <= hi + delta; x += delta) {
        if ((int64_t)out->size() >= limit) return MC_ERR_GRID;
        if (!out->empty() && !(x > out->back())) return MC_ERR_GRID;  // x += delta stalled
        out->push_back(x);
    }
    return MC_OK;
}

// LookupEdgePoint (model3d/mc.go:647-660) for one axis, decided ahead of the
// search for every coordinate a vertex can have on that axis.  A vertex is the
// midpoint (a + b) * 0.5 of its edge's corners (mc.go:401-407), so on its edge
// axis the coordinate is (vals[k] + vals[k+1]) * 0.5 and on the other axes
// (vals[k] + vals[k]) * 0.5, which is vals[k] unless the sum overflows.  For
// each the reference's test -- |math.Mod(c - origin, delta)| strictly between
// delta/4 and 3*delta/4, then idx = int((c - origin) / delta) -- is evaluated
// here in float64 with the reference's operations: out[2k] for the grid value
// k, out[2k+1] for the midpoint of edge k; -1 outside the band, -2 when
// values[idx + 1] would be out of range, else idx.
void edge_lookup_table(const std::vector<double>& vals, double delta, int32_t* out) {
    const size_t n = vals.size();
    const double origin = n ? vals[0] : 0.0;
    auto code = [&](double c) -> int32_t {
        const double av = c - origin;
        const double m = std::fabs(std::fmod(av, delta));
        if (!(m > delta / 4 && m < 3 * delta / 4)) return -1;
        const double q = av / delta;
        if (!(q >= 0) || q >= (double)n) return -2;
        const int64_t idx = (int64_t)q;  // Go int(): truncation
        return idx + 1 < (int64_t)n ? (int32_t)idx : -2;
    };
    for (size_t k = 0; k < n; k++) {
        out[2 * k] = code((vals[k] + vals[k]) * 0.5);
        out[2 * k + 1] = k + 1 < n ? code((vals[k] + vals[k + 1]) * 0.5) : -1;
    }
}

// ---------------------------------------------------------------- case table

namespace {
// Base cases of model3d/mc.go:462-586 (inside corners; triangles as corner pairs).
struct Base {
    uint8_t inside;
    int ntri;
    uint8_t t[5][6];
};
const Base kBase[23] = {
    {0x00, 0, {}},
    {0x01, 1, {{0, 1, 0, 2, 0, 4}}},
    {0x03, 2, {{0, 4, 1, 5, 0, 2}, {1, 5, 1, 3, 0, 2}}},
    {0x21, 2, {{0, 1, 0, 2, 0, 4}, {5, 7, 1, 5, 4, 5}}},
    {0x81, 2, {{0, 1, 0, 2, 0, 4}, {6, 7, 3, 7, 5, 7}}},
    {0x0e, 3, {{0, 1, 1, 5, 0, 2}, {0, 2, 1, 5, 2, 6}, {2, 6, 1, 5, 3, 7}}},
    {0x83, 3, {{0, 4, 1, 5, 0, 2}, {1, 5, 1, 3, 0, 2}, {6, 7, 3, 7, 5, 7}}},
    {0x92, 3, {{4, 6, 4, 5, 0, 4}, {1, 5, 1, 3, 0, 1}, {6, 7, 3, 7, 5, 7}}},
    {0x0f, 2, {{0, 4, 1, 5, 3, 7}, {0, 4, 3, 7, 2, 6}}},
    {0x4d, 4, {{0, 1, 4, 6, 0, 4}, {0, 1, 6, 7, 4, 6}, {0, 1, 1, 3, 6, 7}, {1, 3, 3, 7, 6, 7}}},
    {0x66, 4, {{0, 2, 2, 3, 6, 7}, {0, 2, 6, 7, 4, 6}, {0, 1, 4, 5, 5, 7}, {5, 7, 1, 3, 0, 1}}},
    {0x8d, 4, {{0, 4, 0, 1, 2, 6}, {0, 1, 5, 7, 2, 6}, {2, 6, 5, 7, 6, 7}, {0, 1, 1, 3, 5, 7}}},
    {0x1e, 4, {{0, 1, 1, 5, 0, 2}, {0, 2, 1, 5, 2, 6}, {2, 6, 1, 5, 3, 7}, {4, 5, 0, 4, 4, 6}}},
    {0x96, 4, {{0, 1, 1, 5, 1, 3}, {0, 2, 2, 3, 2, 6}, {4, 5, 0, 4, 4, 6}, {5, 7, 6, 7, 3, 7}}},
    {0x4e, 4, {{0, 2, 0, 1, 4, 6}, {0, 1, 3, 7, 4, 6}, {0, 1, 1, 5, 3, 7}, {4, 6, 3, 7, 6, 7}}},
    {0x6d, 5, {{0, 1, 4, 6, 0, 4}, {0, 1, 6, 7, 4, 6}, {0, 1, 1, 3, 6, 7}, {1, 3, 3, 7, 6, 7}, {5, 7, 1, 5, 4, 5}}},
    {0x7c, 5, {{5, 7, 1, 5, 0, 4}, {0, 4, 6, 7, 5, 7}, {0, 2, 6, 7, 0, 4}, {0, 2, 3, 7, 6, 7}, {0, 2, 1, 3, 3, 7}}},
    {0xf1, 3, {{1, 5, 0, 1, 0, 2}, {0, 2, 2, 6, 1, 5}, {1, 5, 2, 6, 3, 7}}},
    {0x7e, 2, {{0, 2, 0, 1, 0, 4}, {3, 7, 6, 7, 5, 7}}},
    {0xde, 4, {{0, 2, 4, 5, 0, 4}, {0, 2, 5, 7, 4, 5}, {0, 2, 1, 5, 5, 7}, {0, 1, 1, 5, 0, 2}}},
    {0xfc, 2, {{1, 5, 0, 4, 0, 2}, {1, 3, 1, 5, 0, 2}}},
    {0xfe, 1, {{0, 2, 0, 1, 0, 4}}},
    {0xff, 0, {}},
};
}  // namespace

std::vector<XStepD> transform_steps(const mc_node* steps, size_t n, bool inverse) {
    std::vector<XStepD> out;
    for (size_t i = 0; i < n; i++) {
        const mc_node& st = steps[i];
        XStepD s{};
        s.kind = st.kind;
        switch (st.kind) {
            case MC_XF_TRANSLATE:  // Inverse: Offset.Scale(-1), transform.go:52-54
                for (int k = 0; k < 3; k++) s.v[k] = inverse ? st.p[k] * -1 : st.p[k];
                break;
            case MC_XF_SCALE: s.v[0] = inverse ? 1 / st.p[0] : st.p[0]; break;  // transform.go:83-85
            case MC_XF_VECSCALE:                                              // Recip, transform.go:114-116
                for (int k = 0; k < 3; k++) s.v[k] = inverse ? 1 / st.p[k] : st.p[k];
                break;
            case MC_XF_MATRIX:  // transform.go:153-155
                if (inverse) inverse3(st.p, s.v);
                else
                    for (int k = 0; k < 9; k++) s.v[k] = st.p[k];
                break;
            default: throw LowerError(MC_ERR_BAD_PROGRAM, "bad transform step");
        }
        out.push_back(s);
    }
    // JoinedTransform.Inverse applies the inverses in reverse order (transform.go:213-219).
    if (inverse) std::reverse(out.begin(), out.end());
    return out;
}

int build_case_table(uint8_t counts[256], uint8_t tris[256][5][6]) {
    // The 24 rotations (allMcRotations, mc.go:312-353): closure of the
    // identity under the two generators, sorted lexicographically.
    const uint8_t gz[8] = {2, 0, 3, 1, 6, 4, 7, 5};
    const uint8_t gx[8] = {2, 3, 6, 7, 0, 1, 4, 5};
    std::vector<std::array<uint8_t, 8>> rots = {{0, 1, 2, 3, 4, 5, 6, 7}};
    for (size_t i = 0; i < rots.size(); i++)
        for (const uint8_t* g : {gz, gx}) {
            std::array<uint8_t, 8> r;
            for (int k = 0; k < 8; k++) r[k] = g[rots[i][k]];
            if (std::find(rots.begin(), rots.end(), r) == rots.end()) rots.push_back(r);
        }
    std::sort(rots.begin(), rots.end());
    std::memset(counts, 0, 256);
    std::memset(tris, 0, 256 * 5 * 6);
    bool seen[256] = {false};
    int owner[256];
    int conflicts = 0;
    for (int b = 0; b < 23; b++) {
        for (const auto& r : rots) {
            int ni = 0;
            for (int c = 0; c < 8; c++)
                if (kBase[b].inside & (1 << c)) ni |= 1 << r[c];
            if (seen[ni]) {
                conflicts += owner[ni] != b;
                continue;
            }
            seen[ni] = true;
            owner[ni] = b;
            counts[ni] = (uint8_t)kBase[b].ntri;
            for (int t = 0; t < kBase[b].ntri; t++)
                for (int k = 0; k < 6; k++) tris[ni][t][k] = r[kBase[b].t[t][k]];
        }
    }
    int covered = 0;
    for (int i = 0; i < 256; i++) covered += seen[i];
    return (covered == 256 && conflicts == 0 && rots.size() == 24) ? 0 : -1;
}

}  // namespace mcgpu

namespace {

// FNV-1a (64-bit offset basis and prime) over little-endian 64-bit words;
// a tail shorter than a word is zero-padded.  The length goes in first, so
// adjacent arrays cannot trade bytes.
struct Digest {
    uint64_t h = 1469598103934665603ull;
    void word(uint64_t w) { h = (h ^ w) * 1099511628211ull; }
    void bytes(const void* p, size_t n) {
        word(n);
        const unsigned char* b = (const unsigned char*)p;
        size_t i = 0;
        for (; i + 8 <= n; i += 8) {
            uint64_t w;
            std::memcpy(&w, b + i, 8);
            word(w);
        }
        if (i < n) {
            uint64_t w = 0;
            std::memcpy(&w, b + i, n - i);
            word(w);
        }
    }
    template <class T, class A>
    void vec(const std::vector<T, A>& v) { bytes(v.data(), v.size() * sizeof(T)); }
};

uint64_t program_digest(const mcgpu::HostProgram& P) {
    Digest d;
    d.vec(P.ops);
    d.vec(P.ops_allfalse);
    d.word((uint64_t)(int64_t)P.n_ops_allfalse);
    d.word((uint64_t)(int64_t)P.fold_cap);
    d.vec(P.leaf_kind);
    d.vec(P.leaf_d);
    d.vec(P.leaf_f);
    d.vec(P.cull);
    d.vec(P.cull_f);
    d.vec(P.xbox);
    d.vec(P.xstep);
    d.vec(P.trees);
    d.vec(P.nodes);
    d.vec(P.nodes_f);
    d.vec(P.tri_parent);
    d.vec(P.cell_start);
    d.vec(P.ents);
    d.vec(P.tris);
    d.vec(P.tris_f);
    d.vec(P.metas);
    d.vec(P.metas_f);
    d.vec(P.balls);
    d.vec(P.balls_f);
    d.bytes(P.root_min, sizeof P.root_min);
    d.bytes(P.root_max, sizeof P.root_max);
    d.word((uint64_t)(int64_t)P.max_stack);
    d.word((uint64_t)(int64_t)P.max_xdepth);
    d.word((uint64_t)P.has_collider | (uint64_t)P.has_transform << 1);
    return d.h;
}

}  // namespace

extern "C" mc_status mc_program_check(const mc_node* nodes, size_t n_nodes, const mc_tri_set* sets,
                                      size_t n_sets, mc_program_info* info, char* err, size_t err_cap) {
    using namespace mcgpu;
    auto message = [&](const char* m) {
        if (err && err_cap) {
            std::strncpy(err, m, err_cap - 1);
            err[err_cap - 1] = 0;
        }
    };
    message("");
    HostProgram P;
    try {
        lower_scene(nodes, n_nodes, sets, n_sets, &P);
    } catch (const LowerError& e) {
        message(e.what());
        return e.status;
    } catch (const std::exception& e) {
        message(e.what());
        return MC_ERR_BAD_PROGRAM;
    }
    if (info) {
        *info = mc_program_info{};
        info->n_ops = (int64_t)P.ops.size();
        info->n_leaves = (int64_t)P.leaf_kind.size();
        info->n_metaballs = (int64_t)P.metas.size();
        info->n_balls = (int64_t)P.balls.size();
        info->n_boxes = (int64_t)P.xbox.size();
        info->n_colliders = (int64_t)P.trees.size();
        info->max_stack = P.max_stack;
        info->threshold = P.metas.empty() ? std::numeric_limits<double>::quiet_NaN() : P.metas[0].thr;
        for (int i = 0; i < 3; i++) {
            info->root_min[i] = P.root_min[i];
            info->root_max[i] = P.root_max[i];
        }
        info->digest = program_digest(P);
    }
    return MC_OK;
}
