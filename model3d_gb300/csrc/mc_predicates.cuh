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
    // Branch-free: frac < 0 or > norm for sure -> 0; not surely inside
    // [0, norm] -> undecided; else the distance decides.
    const bool out = fhi < 0.f || flo > f[7];
    const bool within = flo >= 0.f && fhi <= f[6];
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
    const int v = decide_le(S, E, f[8], f[9]);
    return out ? 0 : (within ? v : 2);
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
    // Closest point, selected without branches: s1 (mag > norm for sure),
    // s0 (mag < 0 for sure) or the projection (0 <= mag <= norm for sure);
    // undecided when no case is certain.
    const bool c1 = mlo > f[10];
    const bool c0 = !c1 && mhi < 0.f && mhi <= f[9];
    const bool ci = !c1 && !c0 && mlo >= 0.f && mhi <= f[9];
    const float g = 1.0001f * Em + 1.0001f * U32 * (fabsf(mag) + Em);
    const float i1 = __fmaf_rn(-f[6], mag, vx), i2 = __fmaf_rn(-f[7], mag, vy), i3 = __fmaf_rn(-f[8], mag, vz);
    const float d1 = c1 ? p.x - f[3] : (c0 ? vx : i1);
    const float d2 = c1 ? p.y - f[4] : (c0 ? vy : i2);
    const float d3 = c1 ? p.z - f[5] : (c0 ? vz : i3);
    const float e1 = c1 ? 2.001f * U32 * (fabsf(p.x) + fabsf(f[3])) : (c0 ? ex : ax * g + ex + 1.0001f * U32 * fabsf(i1));
    const float e2 = c1 ? 2.001f * U32 * (fabsf(p.y) + fabsf(f[4])) : (c0 ? ey : ay * g + ey + 1.0001f * U32 * fabsf(i2));
    const float e3 = c1 ? 2.001f * U32 * (fabsf(p.z) + fabsf(f[5])) : (c0 ? ez : az * g + ez + 1.0001f * U32 * fabsf(i3));
    float S = __fmaf_rn(d1, d1, __fmaf_rn(d2, d2, d3 * d3));
    float E = e1 * (2.f * fabsf(d1) + e1) + e2 * (2.f * fabsf(d2) + e2) + e3 * (2.f * fabsf(d3) + e3);
    E = 1.001f * (E + 3.02f * U32 * S) + 1e-30f;
    const int v = decide_le(S, E, f[11], f[12]);
    return (c1 || c0 || ci) ? v : 2;
}

// Torus (genericSDF ring point, shapes.go:1451-1487, as torus_64): with
// c = p - center, x = b1.c, y = b2.c, on = |(x, y)|, s = outer / on, the ring
// point is center + (b1 x + b2 y) s and S = |ring - p|^2 is compared with the
// threshold.  The bound carries the errors of x and y (as the cylinder's
// frac), of r2 = x^2 + y^2, of on = sqrt(r2) (|on - on*| <= Er2 / (on + on*)
// + u on) and of s (relative Eon / on_lo plus the roundings of the division
// and of outer).  Points near the axis, where that relative error exceeds
// 1%, are undecided; so are all points the reference would treat as on the
// axis (on == 0), which lie far inside that band.
__device__ __forceinline__ int torus_32(const float* f, F3 p) {
    const float cx = p.x - f[0], cy = p.y - f[1], cz = p.z - f[2];
    const float ex = 2.001f * U32 * (fabsf(p.x) + fabsf(f[0]));
    const float ey = 2.001f * U32 * (fabsf(p.y) + fabsf(f[1]));
    const float ez = 2.001f * U32 * (fabsf(p.z) + fabsf(f[2]));
    const float x = __fmaf_rn(f[3], cx, __fmaf_rn(f[4], cy, f[5] * cz));
    const float y = __fmaf_rn(f[6], cx, __fmaf_rn(f[7], cy, f[8] * cz));
    const float Ex = 1.001f * (fabsf(f[3]) * (ex + 4.03f * U32 * fabsf(cx)) + fabsf(f[4]) * (ey + 4.03f * U32 * fabsf(cy)) +
                               fabsf(f[5]) * (ez + 4.03f * U32 * fabsf(cz))) + 1e-30f;
    const float Ey = 1.001f * (fabsf(f[6]) * (ex + 4.03f * U32 * fabsf(cx)) + fabsf(f[7]) * (ey + 4.03f * U32 * fabsf(cy)) +
                               fabsf(f[8]) * (ez + 4.03f * U32 * fabsf(cz))) + 1e-30f;
    const float r2 = __fmaf_rn(x, x, y * y);
    const float Er2 = 1.001f * (Ex * (2.f * fabsf(x) + Ex) + Ey * (2.f * fabsf(y) + Ey) + 3.01f * U32 * r2) + 1e-30f;
    const float r2lo = __fsub_rd(r2, Er2);
    if (!(r2lo > 0.f)) return 2;
    const float on = __fsqrt_rn(r2), onlo = __fsqrt_rd(r2lo);
    const float Eon = 1.001f * (__fdiv_ru(Er2, on + onlo) + U32 * on) + 1e-30f;
    const float rsc = 1.001f * __fdiv_ru(Eon, onlo) + 2.01f * U32;  // relative error of s
    if (!(rsc <= 0.01f)) return 2;
    const float sc = __fdiv_rn(f[9], on);
    const float xs = x * sc, ys = y * sc;
    const float Exs = 1.01f * ((fabsf(x) + Ex) * sc * rsc + Ex * sc + U32 * fabsf(xs)) + 1e-30f;
    const float Eys = 1.01f * ((fabsf(y) + Ey) * sc * rsc + Ey * sc + U32 * fabsf(ys)) + 1e-30f;
    const float d1 = __fmaf_rn(f[3], xs, __fmaf_rn(f[6], ys, -cx));
    const float d2 = __fmaf_rn(f[4], xs, __fmaf_rn(f[7], ys, -cy));
    const float d3 = __fmaf_rn(f[5], xs, __fmaf_rn(f[8], ys, -cz));
    const float e1 = fabsf(f[3]) * Exs + fabsf(f[6]) * Eys + ex +
                     4.03f * U32 * (fabsf(f[3] * xs) + fabsf(f[6] * ys) + fabsf(cx));
    const float e2 = fabsf(f[4]) * Exs + fabsf(f[7]) * Eys + ey +
                     4.03f * U32 * (fabsf(f[4] * xs) + fabsf(f[7] * ys) + fabsf(cy));
    const float e3 = fabsf(f[5]) * Exs + fabsf(f[8]) * Eys + ez +
                     4.03f * U32 * (fabsf(f[5] * xs) + fabsf(f[8] * ys) + fabsf(cz));
    const float S = __fmaf_rn(d1, d1, __fmaf_rn(d2, d2, d3 * d3));
    float E = e1 * (2.f * fabsf(d1) + e1) + e2 * (2.f * fabsf(d2) + e2) + e3 * (2.f * fabsf(d3) + e3);
    E = 1.001f * (E + 3.02f * U32 * S) + 1e-30f;
    return decide_le(S, E, f[11], f[12]);
}

}  // namespace mcgpu

namespace mcgpu {

// ------------------------------------------------------------ FP32 collider

// 1 / rate of the fixed ray direction, rounded to float at compile time.
__device__ __forceinline__ float inv_rate(int a) {
    return a == 0 ? (float)(1.0 / RAY_DX) : (a == 1 ? (float)(1.0 / RAY_DY) : (float)(1.0 / RAY_DZ));
}
__device__ __forceinline__ float rate_f(int a) {
    return a == 0 ? (float)RAY_DX : (a == 1 ? (float)RAY_DY : (float)RAY_DZ);
}

// Per-ray constants of the FP32 slab test.  With t = fma(b, 1/r, -o/r) for a
// box coordinate b (|b| <= M_a, the tree's magnitude bound) the error against
// the float64 t = (b - o) / r is below 4.2u (M_a + |o_a|) / r_a: float
// rounding of b (outward, <= 2u|b|), of 1/r (u), of o and o/r (3u|o|/r) and
// of the fma (u|t|), plus the float64 rounding (2^-52 relative).
struct RayF {
    float oi[3];
    float E[3];
};
__device__ __forceinline__ RayF make_rayf(F3 pf, const float* mbox) {
    RayF r;
    const float o[3] = {pf.x, pf.y, pf.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        r.oi[a] = o[a] * inv_rate(a);
        r.E[a] = 4.21f * U32 * (mbox[a] + fabsf(o[a])) * inv_rate(a) + 1e-30f;
    }
    return r;
}

// rayCollisionWithBounds + rayCollidesWithBounds with every rate > 0 is
// exactly: hit <=> min_a t2_a >= max(0, max_a t1_a).  1 hit, 0 miss,
// 2 undecided (run ray_box_64).
__device__ __forceinline__ int ray_box_32(const BvhNodeF& n, const RayF& r) {
    float t2lo = CUDART_INF_F, t2hi = CUDART_INF_F, t1lo = 0.f, t1hi = 0.f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float t1 = __fmaf_rn(n.lo[a], inv_rate(a), -r.oi[a]);
        const float t2 = __fmaf_rn(n.hi[a], inv_rate(a), -r.oi[a]);
        t1lo = fmaxf(t1lo, __fsub_rd(t1, r.E[a]));
        t1hi = fmaxf(t1hi, __fadd_ru(t1, r.E[a]));
        t2lo = fminf(t2lo, __fsub_rd(t2, r.E[a]));
        t2hi = fminf(t2hi, __fadd_ru(t2, r.E[a]));
    }
    if (t2lo >= t1hi) return 1;
    if (t2hi < t1lo) return 0;
    return 2;
}

// Moller-Trumbore of Triangle.rayCollision (primitives.go:207-249) in FP32
// with running absolute error bounds on o = p - t0, s1 = o.c1, b1 = s1/det,
// c2 = o x v1, s2 = D.c2, b2, b1 + b2, s3 = v2.c2, scale = s3/det; every
// comparison the bounds cannot decide returns 2 (run ray_tri_64).
__device__ __forceinline__ int ray_tri_32(const TriF& t, F3 p) {
    if (!t.valid) return 0;
    const float ox = p.x - t.t0[0], oy = p.y - t.t0[1], oz = p.z - t.t0[2];
    const float eox = 2.001f * U32 * (fabsf(p.x) + fabsf(t.t0[0]));
    const float eoy = 2.001f * U32 * (fabsf(p.y) + fabsf(t.t0[1]));
    const float eoz = 2.001f * U32 * (fabsf(p.z) + fabsf(t.t0[2]));
    const float ai = fabsf(t.inv_det);
    const float s1 = __fmaf_rn(ox, t.c1[0], __fmaf_rn(oy, t.c1[1], oz * t.c1[2]));
    const float Es1 = 1.001f * (fabsf(t.c1[0]) * (eox + 4.03f * U32 * fabsf(ox)) +
                                fabsf(t.c1[1]) * (eoy + 4.03f * U32 * fabsf(oy)) +
                                fabsf(t.c1[2]) * (eoz + 4.03f * U32 * fabsf(oz))) + 1e-30f;
    const float b1 = t.inv_det * s1;
    const float Eb1 = 1.001f * (ai * (Es1 + U32 * (fabsf(s1) + Es1)) + U32 * fabsf(b1)) + 1e-30f;
    if (__fadd_ru(b1, Eb1) < 0.f || __fsub_rd(b1, Eb1) > 1.f) return 0;
    if (!(__fsub_rd(b1, Eb1) >= 0.f && __fadd_ru(b1, Eb1) <= 1.f)) return 2;
    const float c2x = __fmaf_rn(oy, t.v1[2], -(oz * t.v1[1]));
    const float c2y = __fmaf_rn(oz, t.v1[0], -(ox * t.v1[2]));
    const float c2z = __fmaf_rn(ox, t.v1[1], -(oy * t.v1[0]));
    const float Ec2x = 1.001f * (fabsf(t.v1[2]) * (eoy + 3.01f * U32 * fabsf(oy)) +
                                 fabsf(t.v1[1]) * (eoz + 3.01f * U32 * fabsf(oz))) + 1e-30f;
    const float Ec2y = 1.001f * (fabsf(t.v1[0]) * (eoz + 3.01f * U32 * fabsf(oz)) +
                                 fabsf(t.v1[2]) * (eox + 3.01f * U32 * fabsf(ox))) + 1e-30f;
    const float Ec2z = 1.001f * (fabsf(t.v1[1]) * (eox + 3.01f * U32 * fabsf(ox)) +
                                 fabsf(t.v1[0]) * (eoy + 3.01f * U32 * fabsf(oy))) + 1e-30f;
    const float s2 = __fmaf_rn(rate_f(0), c2x, __fmaf_rn(rate_f(1), c2y, rate_f(2) * c2z));
    const float Es2 = 1.001f * (rate_f(0) * (Ec2x + 4.03f * U32 * fabsf(c2x)) +
                                rate_f(1) * (Ec2y + 4.03f * U32 * fabsf(c2y)) +
                                rate_f(2) * (Ec2z + 4.03f * U32 * fabsf(c2z))) + 1e-30f;
    const float b2 = t.inv_det * s2;
    const float Eb2 = 1.001f * (ai * (Es2 + U32 * (fabsf(s2) + Es2)) + U32 * fabsf(b2)) + 1e-30f;
    if (__fadd_ru(b2, Eb2) < 0.f) return 0;
    const float bs = b1 + b2;
    const float Ebs = 1.001f * (Eb1 + Eb2 + U32 * fabsf(bs)) + 1e-30f;
    if (__fsub_rd(bs, Ebs) > 1.f) return 0;
    if (!(__fsub_rd(b2, Eb2) >= 0.f && __fadd_ru(bs, Ebs) <= 1.f)) return 2;
    const float s3 = __fmaf_rn(t.v2[0], c2x, __fmaf_rn(t.v2[1], c2y, t.v2[2] * c2z));
    const float Es3 = 1.001f * (fabsf(t.v2[0]) * (Ec2x + 4.03f * U32 * fabsf(c2x)) +
                                fabsf(t.v2[1]) * (Ec2y + 4.03f * U32 * fabsf(c2y)) +
                                fabsf(t.v2[2]) * (Ec2z + 4.03f * U32 * fabsf(c2z))) + 1e-30f;
    const float sc = t.inv_det * s3;
    const float Esc = 1.001f * (ai * (Es3 + U32 * (fabsf(s3) + Es3)) + U32 * fabsf(sc)) + 1e-30f;
    if (__fadd_ru(sc, Esc) < 0.f) return 0;
    if (__fsub_rd(sc, Esc) >= 0.f) return 1;
    return 2;
}

}  // namespace mcgpu
