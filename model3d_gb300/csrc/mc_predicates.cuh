// mc_predicates.cuh — device containment predicates.
//
// Two implementations per leaf kind:
//   *_64: the reference predicate in IEEE float64 with the reference's
//         operation order; every operation is an explicit round-to-nearest
//         intrinsic so nvcc cannot contract a*b+c into an FMA.
//   *_32: an FP32 evaluation with a forward error bound.  It returns 1/0 when
//         the bound proves what the float64 predicate returns, and 2 when it
//         cannot decide (the caller then runs *_64).  The bound covers both
//         the FP32 rounding and the float64 rounding relative to the exact
//         value of the reference formula, so a decided answer always equals
//         the float64 answer.
//
// Error-bound notation: u = 2^-24.  For an input x rounded to float,
// |fl(x) - x| <= u|x|; a float sum/product adds u|result|.  Constants below
// are inflated slightly (2.001u instead of 2u, ...) to absorb second-order
// terms, the rounding of the bound arithmetic itself, and the float64 error
// (2^-53 relative, 2^29 times smaller than u).
#pragma once

#include "mc_internal.h"

namespace mcgpu {

#define D_ADD __dadd_rn
#define D_SUB __dsub_rn
#define D_MUL __dmul_rn
#define D_DIV __ddiv_rn
#define D_SQRT __dsqrt_rn

constexpr float U32 = 5.9604645e-08f;  // 2^-24

struct P3 {
    double x, y, z;
};
struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 to_f3(P3 p) { return F3{(float)p.x, (float)p.y, (float)p.z}; }
__device__ __forceinline__ double comp(const P3& p, int a) { return a == 0 ? p.x : (a == 1 ? p.y : p.z); }
__device__ __forceinline__ void set_comp(P3& p, int a, double v) {
    if (a == 0) p.x = v;
    else if (a == 1) p.y = v;
    else p.z = v;
}

// ------------------------------------------------------------------ FP64

// Sphere.Contains: coord.Dist(center) <= R (model3d/shapes.go:29-31,
// coords.go:272-277); sqrt(S) <= R is S <= TR (TR precomputed).
__device__ __forceinline__ bool sphere_64(const double* c, P3 p) {
    double dx = D_SUB(p.x, c[0]), dy = D_SUB(p.y, c[1]), dz = D_SUB(p.z, c[2]);
    double S = D_ADD(D_ADD(D_MUL(dx, dx), D_MUL(dy, dy)), D_MUL(dz, dz));
    return S <= c[3];
}

// Rect.Contains: c.Min(min) == min && c.Max(max) == max (shapes.go:171-173),
// i.e. min <= c <= max per axis with NaN false.
__device__ __forceinline__ bool rect_64(const double* c, P3 p) {
    return p.x >= c[0] && p.y >= c[1] && p.z >= c[2] && p.x <= c[3] && p.y <= c[4] && p.z <= c[5];
}

// Cylinder.Contains (shapes.go:588-598) with diff = P1 - P2,
// dir = diff.Normalize() and norm = diff.Norm() precomputed.
__device__ __forceinline__ bool cylinder_64(const double* c, P3 p) {
    double qx = D_SUB(p.x, c[0]), qy = D_SUB(p.y, c[1]), qz = D_SUB(p.z, c[2]);
    double frac = D_ADD(D_ADD(D_MUL(qx, c[3]), D_MUL(qy, c[4])), D_MUL(qz, c[5]));
    if (frac < 0 || frac > c[6]) return false;
    double d1 = D_SUB(D_ADD(c[0], D_MUL(c[3], frac)), p.x);
    double d2 = D_SUB(D_ADD(c[1], D_MUL(c[4], frac)), p.y);
    double d3 = D_SUB(D_ADD(c[2], D_MUL(c[5], frac)), p.z);
    double S = D_ADD(D_ADD(D_MUL(d1, d1), D_MUL(d2, d2)), D_MUL(d3, d3));
    return S <= c[7];
}

// Capsule.Contains = NewSegment(P1, P2).Dist(c) <= R (shapes.go:365-368,
// primitives.go:547-594); canonical order s0, s1, v = (s1-s0)/|s1-s0|.
__device__ __forceinline__ bool capsule_64(const double* c, P3 p) {
    double vx = D_SUB(p.x, c[0]), vy = D_SUB(p.y, c[1]), vz = D_SUB(p.z, c[2]);
    double mag = D_ADD(D_ADD(D_MUL(c[6], vx), D_MUL(c[7], vy)), D_MUL(c[8], vz));
    double qx, qy, qz;
    if (mag > c[9]) {
        qx = c[3], qy = c[4], qz = c[5];
    } else if (mag < 0) {
        qx = c[0], qy = c[1], qz = c[2];
    } else {
        qx = D_ADD(D_MUL(c[6], mag), c[0]);
        qy = D_ADD(D_MUL(c[7], mag), c[1]);
        qz = D_ADD(D_MUL(c[8], mag), c[2]);
    }
    double d1 = D_SUB(p.x, qx), d2 = D_SUB(p.y, qy), d3 = D_SUB(p.z, qz);
    double S = D_ADD(D_ADD(D_MUL(d1, d1), D_MUL(d2, d2)), D_MUL(d3, d3));
    return S <= c[10];
}

// Torus.Contains = genericSDF(c) >= 0 (shapes.go:1363-1365, :1451-1487) with
// the OrthoBasis of Axis precomputed; Inner - dist >= 0 is S <= T_inner.
__device__ __forceinline__ bool torus_64(const double* c, P3 p) {
    double cx = D_SUB(p.x, c[0]), cy = D_SUB(p.y, c[1]), cz = D_SUB(p.z, c[2]);
    double x = D_ADD(D_ADD(D_MUL(c[3], cx), D_MUL(c[4], cy)), D_MUL(c[5], cz));
    double y = D_ADD(D_ADD(D_MUL(c[6], cx), D_MUL(c[7], cy)), D_MUL(c[8], cz));
    double on = D_SQRT(D_ADD(D_MUL(x, x), D_MUL(y, y)));
    if (on == 0) {
        x = 1;
        y = 0;
        on = 1;
    }
    double sc = D_DIV(c[9], on);
    x = D_MUL(x, sc);
    y = D_MUL(y, sc);
    double d1 = D_SUB(D_ADD(D_MUL(c[3], x), D_MUL(c[6], y)), cx);
    double d2 = D_SUB(D_ADD(D_MUL(c[4], x), D_MUL(c[7], y)), cy);
    double d3 = D_SUB(D_ADD(D_MUL(c[5], x), D_MUL(c[8], y)), cz);
    double S = D_ADD(D_ADD(D_MUL(d1, d1), D_MUL(d2, d2)), D_MUL(d3, d3));
    return S <= c[10];
}

// The fixed ray direction of ColliderContains (model3d/collisions.go:124).
#define RAY_DX 0.5224892708603626
#define RAY_DY 0.10494477243214506
#define RAY_DZ 0.43558938446126527

// rayCollisionWithBounds + rayCollidesWithBounds (bvh.go:322-351,
// collisions.go:305-308).  Every rate is non-zero, so the rate == 0 branch
// never runs; the divisions are true IEEE divisions as in the reference.
__device__ __forceinline__ bool ray_box_64(const double* lo, const double* hi, P3 o) {
    double minF = -CUDART_INF, maxF = CUDART_INF;
    const double oo[3] = {o.x, o.y, o.z};
    const double rate[3] = {RAY_DX, RAY_DY, RAY_DZ};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        double t1 = D_DIV(D_SUB(lo[a], oo[a]), rate[a]);
        double t2 = D_DIV(D_SUB(hi[a], oo[a]), rate[a]);
        if (t1 > t2) {
            double t = t1;
            t1 = t2;
            t2 = t;
        }
        if (t2 < 0) return false;
        if (t1 > minF) minF = t1;
        if (t2 < maxF) maxF = t2;
    }
    return maxF >= minF && maxF >= 0;
}

// Triangle.RayCollisions via rayCollision (primitives.go:194-249).
__device__ __forceinline__ int ray_tri_64(const TriD& t, P3 p) {
    if (!t.valid) return 0;
    double ox = D_SUB(p.x, t.t0[0]), oy = D_SUB(p.y, t.t0[1]), oz = D_SUB(p.z, t.t0[2]);
    double b1 = D_MUL(t.inv_det, D_ADD(D_ADD(D_MUL(ox, t.c1[0]), D_MUL(oy, t.c1[1])), D_MUL(oz, t.c1[2])));
    if (b1 < 0 || b1 > 1) return 0;
    double c2x = D_SUB(D_MUL(oy, t.v1[2]), D_MUL(oz, t.v1[1]));
    double c2y = D_SUB(D_MUL(oz, t.v1[0]), D_MUL(ox, t.v1[2]));
    double c2z = D_SUB(D_MUL(ox, t.v1[1]), D_MUL(oy, t.v1[0]));
    double b2 = D_MUL(t.inv_det, D_ADD(D_ADD(D_MUL(RAY_DX, c2x), D_MUL(RAY_DY, c2y)), D_MUL(RAY_DZ, c2z)));
    if (b2 < 0 || D_ADD(b1, b2) > 1) return 0;
    double sc = D_MUL(t.inv_det, D_ADD(D_ADD(D_MUL(t.v2[0], c2x), D_MUL(t.v2[1], c2y)), D_MUL(t.v2[2], c2z)));
    return sc < 0 ? 0 : 1;
}

// ------------------------------------------------------------------ FP32

// Decide S64 <= TR from S32 with |S32 - S_exact| + |S64 - S_exact| <= E.
__device__ __forceinline__ int decide_le(float S, float E, float tr_lo, float tr_hi) {
    if (__fadd_ru(S, E) <= tr_lo) return 1;
    if (__fsub_rd(S, E) > tr_hi) return 0;
    return 2;
}

// Sphere: d_i = p_i - c_i, |d32_i - d_i| <= e_i = 2.001u(|p_i| + |c_i|);
// |S32 - S| <= sum e_i(2|d32_i| + e_i) + 3.01u S32.
__device__ __forceinline__ int sphere_32(const float* f, F3 p) {
    float dx = p.x - f[0], dy = p.y - f[1], dz = p.z - f[2];
    float S = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz));
    float ex = 2.001f * U32 * (fabsf(p.x) + fabsf(f[0]));
    float ey = 2.001f * U32 * (fabsf(p.y) + fabsf(f[1]));
    float ez = 2.001f * U32 * (fabsf(p.z) + fabsf(f[2]));
    float E = ex * (2.f * fabsf(dx) + ex) + ey * (2.f * fabsf(dy) + ey) + ez * (2.f * fabsf(dz) + ez);
    E = 1.001f * (E + 3.01f * U32 * S) + 1e-30f;
    return decide_le(S, E, f[4], f[5]);
}

// Rect: float rounding is monotone, so fl(p) > fl(m) proves p > m and
// fl(p) < fl(m) proves p < m; equality is undecided.
__device__ __forceinline__ int rect_32(const float* f, F3 p) {
    const float pp[3] = {p.x, p.y, p.z};
    int undecided = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (pp[a] < f[a] || pp[a] > f[3 + a]) return 0;
        undecided |= (pp[a] == f[a]) | (pp[a] == f[3 + a]);
        undecided |= (pp[a] != pp[a]) | (f[a] != f[a]) | (f[3 + a] != f[3 + a]);
    }
    return undecided ? 2 : 1;
}

// Cylinder: q = p - P2, frac = q.dir, d = dir*frac - q (= projection - p).
__device__ __forceinline__ int cylinder_32(const float* f, F3 p) {
    float qx = p.x - f[0], qy = p.y - f[1], qz = p.z - f[2];
    float eqx = 2.001f * U32 * (fabsf(p.x) + fabsf(f[0]));
    float eqy = 2.001f * U32 * (fabsf(p.y) + fabsf(f[1]));
    float eqz = 2.001f * U32 * (fabsf(p.z) + fabsf(f[2]));
    float frac = __fmaf_rn(qx, f[3], __fmaf_rn(qy, f[4], qz * f[5]));
    float ax = fabsf(f[3]), ay = fabsf(f[4]), az = fabsf(f[5]);
    float Ef = 1.001f * (ax * (eqx + 4.03f * U32 * fabsf(qx)) + ay * (eqy + 4.03f * U32 * fabsf(qy)) +
                         az * (eqz + 4.03f * U32 * fabsf(qz))) + 1e-30f;
    float flo = __fsub_rd(frac, Ef), fhi = __fadd_ru(frac, Ef);
    if (fhi < 0.f) return 0;          // frac < 0
    if (flo > f[7]) return 0;         // frac > norm
    if (!(flo >= 0.f && fhi <= f[6])) return 2;
    float d1 = __fmaf_rn(f[3], frac, -qx);
    float d2 = __fmaf_rn(f[4], frac, -qy);
    float d3 = __fmaf_rn(f[5], frac, -qz);
    float S = __fmaf_rn(d1, d1, __fmaf_rn(d2, d2, d3 * d3));
    float g = 1.0001f * Ef + 1.0001f * U32 * (fabsf(frac) + Ef);
    float e1 = ax * g + eqx + 1.0001f * U32 * fabsf(d1);
    float e2 = ay * g + eqy + 1.0001f * U32 * fabsf(d2);
    float e3 = az * g + eqz + 1.0001f * U32 * fabsf(d3);
    float E = e1 * (2.f * fabsf(d1) + e1) + e2 * (2.f * fabsf(d2) + e2) + e3 * (2.f * fabsf(d3) + e3);
    E = 1.001f * (E + 3.02f * U32 * S) + 1e-30f;
    return decide_le(S, E, f[8], f[9]);
}

// Capsule: v2 = p - s0, mag = v.v2; closest point chosen by mag vs [0, norm].
__device__ __forceinline__ int capsule_32(const float* f, F3 p) {
    float vx = p.x - f[0], vy = p.y - f[1], vz = p.z - f[2];
    float ex = 2.001f * U32 * (fabsf(p.x) + fabsf(f[0]));
    float ey = 2.001f * U32 * (fabsf(p.y) + fabsf(f[1]));
    float ez = 2.001f * U32 * (fabsf(p.z) + fabsf(f[2]));
    float mag = __fmaf_rn(f[6], vx, __fmaf_rn(f[7], vy, f[8] * vz));
    float ax = fabsf(f[6]), ay = fabsf(f[7]), az = fabsf(f[8]);
    float Em = 1.001f * (ax * (ex + 4.03f * U32 * fabsf(vx)) + ay * (ey + 4.03f * U32 * fabsf(vy)) +
                         az * (ez + 4.03f * U32 * fabsf(vz))) + 1e-30f;
    float mlo = __fsub_rd(mag, Em), mhi = __fadd_ru(mag, Em);
    float d1, d2, d3, e1, e2, e3;
    if (mlo > f[10]) {  // mag > norm: closest = s1
        d1 = p.x - f[3], d2 = p.y - f[4], d3 = p.z - f[5];
        e1 = 2.001f * U32 * (fabsf(p.x) + fabsf(f[3]));
        e2 = 2.001f * U32 * (fabsf(p.y) + fabsf(f[4]));
        e3 = 2.001f * U32 * (fabsf(p.z) + fabsf(f[5]));
    } else if (mhi < 0.f && mhi <= f[9]) {  // mag < 0 (and not > norm): closest = s0
        d1 = vx, d2 = vy, d3 = vz;
        e1 = ex, e2 = ey, e3 = ez;
    } else if (mlo >= 0.f && mhi <= f[9]) {  // interior: closest = v*mag + s0
        d1 = __fmaf_rn(-f[6], mag, vx);
        d2 = __fmaf_rn(-f[7], mag, vy);
        d3 = __fmaf_rn(-f[8], mag, vz);
        float g = 1.0001f * Em + 1.0001f * U32 * (fabsf(mag) + Em);
        e1 = ax * g + ex + 1.0001f * U32 * fabsf(d1);
        e2 = ay * g + ey + 1.0001f * U32 * fabsf(d2);
        e3 = az * g + ez + 1.0001f * U32 * fabsf(d3);
    } else {
        return 2;
    }
    float S = __fmaf_rn(d1, d1, __fmaf_rn(d2, d2, d3 * d3));
    float E = e1 * (2.f * fabsf(d1) + e1) + e2 * (2.f * fabsf(d2) + e2) + e3 * (2.f * fabsf(d3) + e3);
    E = 1.001f * (E + 3.02f * U32 * S) + 1e-30f;
    return decide_le(S, E, f[11], f[12]);
}

}  // namespace mcgpu
