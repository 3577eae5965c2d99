// mc_metaball.cuh — device evaluation of WeightedMetaballSolid leaves
// (model3d/metaball.go:165-242): the float64 sum in the reference's order,
// the FP32 interval filter, warp-cooperative escalation and the far-field
// split of classification tiles.  Included by mc_kernels.cu after the
// transform helpers it uses (apply_steps); layouts in mc_internal.h
// (MetaD / MetaF / BallD / BallF).
#pragma once

#include "mc_predicates.cuh"

namespace mcgpu {


// math.Ldexp and math.Pow(x, -k) for x > 0 (Go math/ldexp.go, math/pow.go),
// operation for operation: Frexp, repeated squaring of the mantissa with
// renormalisation to [0.5, 1), one reciprocal, Ldexp.
__device__ double go_ldexp_d(double frac, long long exp) {
    if (frac == 0 || isinf(frac) || isnan(frac)) return frac;
    if (fabs(frac) < 2.2250738585072014e-308) {
        frac = D_MUL(frac, 4503599627370496.0);
        exp -= 52;
    }
    unsigned long long x = (unsigned long long)__double_as_longlong(frac);
    exp += (long long)((x >> 52) & 0x7ff) - 1023;
    if (exp < -1075) return copysign(0.0, frac);
    if (exp > 1023) return frac < 0 ? -INFINITY : INFINITY;
    double m = 1;
    if (exp < -1022) {
        exp += 53;
        m = 1.1102230246251565e-16;  // 2^-53
    }
    x &= ~(0x7ffull << 52);
    x |= (unsigned long long)(exp + 1023) << 52;
    return D_MUL(m, __longlong_as_double((long long)x));
}

__device__ double go_pow_neg(double x, int k) {  // math.Pow(x, -k), k >= 1
    if (x == 1) return 1;
    if (isnan(x)) return x;
    if (isinf(x)) return 0;
    int xe_i;
    double x1 = frexp(x, &xe_i);
    long long xe = xe_i, ae = 0;
    double a1 = 1;
    for (int i = k; i != 0; i >>= 1) {
        if (xe < -(1 << 12) || (1 << 12) < xe) {
            ae += xe;
            break;
        }
        if (i & 1) {
            a1 = D_MUL(a1, x1);
            ae += xe;
        }
        x1 = D_MUL(x1, x1);
        xe <<= 1;
        if (x1 < .5) {
            x1 = D_ADD(x1, x1);
            xe--;
        }
    }
    return go_ldexp_d(D_DIV(1.0, a1), -ae);
}

__device__ __forceinline__ double dist3_64(double ax, double ay, double az, double bx, double by, double bz) {
    double d1 = D_SUB(ax, bx), d2 = D_SUB(ay, by), d3 = D_SUB(az, bz);  // Coord3D.Dist, coords.go:272-277
    return D_SQRT(D_ADD(D_ADD(D_MUL(d1, d1), D_MUL(d2, d2)), D_MUL(d3, d3)));
}

// math.Min / math.Max: -Inf (+Inf) first, then NaN, then -0 below +0.
__device__ __forceinline__ double go_min_d(double x, double y) {
    if (x == -INFINITY || y == -INFINITY) return -INFINITY;
    if (isnan(x) || isnan(y)) return x + y;
    if (x == 0 && y == 0) return signbit(x) ? x : y;
    return x < y ? x : y;
}
__device__ __forceinline__ double go_max_d(double x, double y) {
    if (x == INFINITY || y == INFINITY) return INFINITY;
    if (isnan(x) || isnan(y)) return x + y;
    if (x == 0 && y == 0) return signbit(x) ? y : x;
    return x > y ? x : y;
}

// filledCircleDist (shapes.go:783-812): basis rows b1, b2 (c + 0, c + 3),
// proj.z given (the axis row times q).
__device__ __forceinline__ void circle_dist_64(const double* b, double qx, double qy, double qz, double pz, double R,
                                               double* cur) {
    double px = D_ADD(D_ADD(D_MUL(b[0], qx), D_MUL(b[1], qy)), D_MUL(b[2], qz));
    double py = D_ADD(D_ADD(D_MUL(b[3], qx), D_MUL(b[4], qy)), D_MUL(b[5], qz));
    double n2 = D_SQRT(D_ADD(D_MUL(px, px), D_MUL(py, py)));
    double d;
    if (n2 < R) {
        d = fabs(pz);
    } else {
        n2 = D_SUB(n2, R);
        d = D_SQRT(D_ADD(D_MUL(n2, n2), D_MUL(pz, pz)));
    }
    if (d <= *cur) *cur = d;
}

// SDF of a ball's primitive in float64, reference order (shapes.go:100,
// :270-317, :481-514, :746-781, :1451-1487).
__device__ double ball_sdf_64(const BallD& b, P3 p) {
    const double* c = b.c;
    switch (b.kind) {
        case LK_SPHERE: return D_SUB(c[3], dist3_64(p.x, p.y, p.z, c[0], c[1], c[2]));
        case LK_RECT: {
            if (!(p.x >= c[0] && p.y >= c[1] && p.z >= c[2] && p.x <= c[3] && p.y <= c[4] && p.z <= c[5])) {
                // c.Min(MaxVal).Max(MinVal) with math.Min / math.Max
                double nx = go_max_d(go_min_d(p.x, c[3]), c[0]), ny = go_max_d(go_min_d(p.y, c[4]), c[1]),
                       nz = go_max_d(go_min_d(p.z, c[5]), c[2]);
                return -dist3_64(p.x, p.y, p.z, nx, ny, nz);
            }
            double d = INFINITY;
            double v[3] = {p.x, p.y, p.z};
            for (int i = 0; i < 3; i++) {
                double a = go_min_d(D_SUB(v[i], c[i]), D_SUB(c[3 + i], v[i]));
                if (a < d) d = a;
            }
            return d;
        }
        case LK_CAPSULE:
        case LK_CYLINDER: {
            const double qx = D_SUB(p.x, c[0]), qy = D_SUB(p.y, c[1]), qz = D_SUB(p.z, c[2]);
            const double dot = D_ADD(D_ADD(D_MUL(qx, c[6]), D_MUL(qy, c[7])), D_MUL(qz, c[8]));
            const double nrm = c[9], R = c[10];
            if (b.kind == LK_CAPSULE) {
                if (dot < 0 || dot > nrm) {
                    const double* e = dot < 0 ? c : c + 3;
                    return D_SUB(R, dist3_64(p.x, p.y, p.z, e[0], e[1], e[2]));
                }
                return D_SUB(R, dist3_64(p.x, p.y, p.z, D_ADD(D_MUL(c[6], dot), c[0]),
                                         D_ADD(D_MUL(c[7], dot), c[1]), D_ADD(D_MUL(c[8], dot), c[2])));
            }
            double cur = INFINITY;
            bool contained = false;
            if (dot >= 0 && dot < nrm) {
                double sd = D_SUB(R, dist3_64(p.x, p.y, p.z, D_ADD(D_MUL(c[6], dot), c[0]),
                                              D_ADD(D_MUL(c[7], dot), c[1]), D_ADD(D_MUL(c[8], dot), c[2])));
                if (sd > 0) {
                    contained = true;
                    cur = sd;
                } else {
                    cur = -sd;
                }
            }
            circle_dist_64(c + 11, qx, qy, qz, -dot, R, &cur);
            const double rx = D_SUB(p.x, c[3]), ry = D_SUB(p.y, c[4]), rz = D_SUB(p.z, c[5]);
            const double dot2 = D_ADD(D_ADD(D_MUL(c[6], rx), D_MUL(c[7], ry)), D_MUL(c[8], rz));
            circle_dist_64(c + 17, rx, ry, rz, dot2, R, &cur);
            return contained ? cur : -cur;
        }
        default: {  // torus
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
            return D_SUB(c[10], dist3_64(D_ADD(D_MUL(c[3], x), D_MUL(c[6], y)), D_ADD(D_MUL(c[4], x), D_MUL(c[7], y)),
                                         D_ADD(D_MUL(c[5], x), D_MUL(c[8], y)), cx, cy, cz));
        }
    }
}

// One float64 term w * f(MetaballField(c)) of the reference's sum
// (metaball.go:238-240).
__device__ __forceinline__ double ball_term_64(const XStepD* xstep, const MetaD& m, const BallD& b, P3 p) {
    const P3 q = b.n_steps ? apply_steps(xstep + b.first_step, b.n_steps, p) : p;
    const double r = -ball_sdf_64(b, q);  // MetaballField
    double t;
    if (m.falloff == MC_FALLOFF_POWER) {
        t = r <= 0 ? INFINITY : go_pow_neg(r, (int)m.param);
    } else if (r < 0) {
        t = INFINITY;
    } else if (r >= m.param) {
        t = 0;
    } else {
        double v = D_SUB(1.0, D_DIV(D_MUL(r, r), m.d2));
        t = D_MUL(v, v);
    }
    return D_MUL(b.w, t);
}

__device__ __forceinline__ bool meta_in_bounds(const MetaD& m, P3 p) {  // CheckedFuncSolid (solid.go:46-50)
    return p.x >= m.lo[0] && p.y >= m.lo[1] && p.z >= m.lo[2] && p.x <= m.hi[0] && p.y <= m.hi[1] && p.z <= m.hi[2];
}

// WeightedMetaballSolid.Contains in float64 (metaball.go:234-242).
__device__ __noinline__ bool metaball_64(const ProgView& P, const double* ld, P3 p) {
    const MetaD& m = P.metas[(int)ld[0]];
    if (m.never || !meta_in_bounds(m, p)) return false;
    double sum = 0;
    for (int i = 0; i < m.n_balls; i++) sum = D_ADD(sum, ball_term_64(P.xstep, m, P.balls[m.first_ball + i], p));
    return sum > m.thr;
}

// metaball_64 at the leader lane's point, with the active lanes of `mask`
// computing the terms and the leader adding them in ball order (the
// reference's sequential sum, so the result is the same bits).  The tables
// are the leader's (lanes of a batched launch may run different programs).
// Kernels that call this have at most 8 warps per block.
constexpr int kCoopBalls = 256;
__device__ __noinline__ bool metaball_64_coop(const MetaD& m, const BallD* balls, const XStepD* xstep, P3 p,
                                              unsigned mask, int leader) {
    __shared__ double terms[8][kCoopBalls];
    const int lane = threadIdx.x & 31;
    double* buf = terms[threadIdx.x >> 5];
    if (m.never || !meta_in_bounds(m, p)) return false;  // the same for every lane of mask
    const int rank = __popc(mask & ((1u << lane) - 1u)), nact = __popc(mask);
    double sum = 0;
    for (int base = 0; base < m.n_balls; base += kCoopBalls) {
        const int n = min(kCoopBalls, m.n_balls - base);
        for (int j = rank; j < n; j += nact) buf[j] = ball_term_64(xstep, m, balls[m.first_ball + base + j], p);
        __syncwarp(mask);
        if (lane == leader)
            for (int j = 0; j < n; j++) sum = D_ADD(sum, buf[j]);
        __syncwarp(mask);
    }
    return sum > m.thr;  // meaningful on the leader
}

// Resolve the lanes whose FP32 filter could not decide (r == 2).  When a few
// lanes of the warp escalate, the whole warp computes their float64 sums one
// point at a time; when many do, each lane computes its own.
__device__ __forceinline__ bool metaball_resolve(const ProgView& P, const double* ld, P3 p, int r) {
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    unsigned need = __ballot_sync(mask, r == 2);
    if (__popc(need) > 8) return r == 2 ? metaball_64(P, ld, p) : r == 1;
    bool res = r == 1;
    while (need) {
        const int leader = __ffs(need) - 1;
        need &= need - 1;
        const MetaD* ml = (const MetaD*)__shfl_sync(mask, (unsigned long long)(P.metas + (int)ld[0]), leader);
        const BallD* bl = (const BallD*)__shfl_sync(mask, (unsigned long long)P.balls, leader);
        const XStepD* xl = (const XStepD*)__shfl_sync(mask, (unsigned long long)P.xstep, leader);
        const P3 pl{__shfl_sync(mask, p.x, leader), __shfl_sync(mask, p.y, leader), __shfl_sync(mask, p.z, leader)};
        const bool v = metaball_64_coop(*ml, bl, xl, pl, mask, leader);
        if (lane == leader) res = v;
    }
    return res;
}



__device__ __forceinline__ float dist3_32(float x, float y, float z) { return __fsqrt_rn(x * x + y * y + z * z); }

__device__ __forceinline__ void circle_dist_32(const float* b, float qx, float qy, float qz, float pz, float R,
                                               float* cur) {
    float px = b[0] * qx + b[1] * qy + b[2] * qz;
    float py = b[3] * qx + b[4] * qy + b[5] * qz;
    float n2 = __fsqrt_rn(px * px + py * py);
    float d = n2 < R ? fabsf(pz) : __fsqrt_rn((n2 - R) * (n2 - R) + pz * pz);
    *cur = fminf(*cur, d);
}

// -SDF of a ball in float, in coordinates relative to the ball's anchor.
// Returns an absolute error bound of the value against the float64 value
// (+Inf near a torus axis).  The float offset q = fl(pf - a) is within
// e = u (|p| + |a| + |q|) per coordinate of p - A, so, the SDF being
// 1-Lipschitz, the offset costs at most sqrt(3) e; the rest is the kind's own
// rounding, kint (|q| + mag + |r|), with kint derived per kind as for the
// other filters (products and sums of bounded terms, each sqrt a half-ulp
// of its argument plus one rounding, branch flips continuous in the point).
__device__ float ball_field_32(const BallF& b, F3 pf, float* out) {
    const float* c = b.c;
    const float qx = pf.x - b.a[0], qy = pf.y - b.a[1], qz = pf.z - b.a[2];
    float sdf, guard = 0.f;
    switch (b.kind) {
        case LK_SPHERE: sdf = c[0] - dist3_32(qx, qy, qz); break;
        case LK_RECT: {
            if (!(qx >= c[0] && qy >= c[1] && qz >= c[2] && qx <= c[3] && qy <= c[4] && qz <= c[5])) {
                sdf = -dist3_32(qx - fmaxf(fminf(qx, c[3]), c[0]), qy - fmaxf(fminf(qy, c[4]), c[1]),
                                qz - fmaxf(fminf(qz, c[5]), c[2]));
            } else {
                sdf = fminf(fminf(fminf(qx - c[0], c[3] - qx), fminf(qy - c[1], c[4] - qy)),
                            fminf(qz - c[2], c[5] - qz));
            }
            break;
        }
        case LK_CAPSULE:
        case LK_CYLINDER: {
            const float dot = qx * c[3] + qy * c[4] + qz * c[5];
            const float nrm = c[6], R = c[7];
            const float t = fminf(fmaxf(dot, 0.f), nrm);
            const float sd = R - dist3_32(qx - c[3] * t, qy - c[4] * t, qz - c[5] * t);
            if (b.kind == LK_CAPSULE) {
                sdf = sd;
                break;
            }
            float cur = INFINITY;
            bool contained = false;
            if (dot >= 0.f && dot < nrm) {
                contained = sd > 0.f;
                cur = fabsf(sd);
            }
            circle_dist_32(c + 8, qx, qy, qz, -dot, R, &cur);
            const float rx = qx - c[0], ry = qy - c[1], rz = qz - c[2];
            circle_dist_32(c + 14, rx, ry, rz, c[3] * rx + c[4] * ry + c[5] * rz, R, &cur);
            sdf = contained ? cur : -cur;
            break;
        }
        default: {  // torus
            float x = c[0] * qx + c[1] * qy + c[2] * qz;
            float y = c[3] * qx + c[4] * qy + c[5] * qz;
            float on = __fsqrt_rn(x * x + y * y);
            // Near the axis the ring point's direction is ill-determined;
            // beyond outer/64 its error moves the distance by a bounded amount.
            if (!(on >= fabsf(c[6]) * 0.015625f)) guard = INFINITY;
            const float sc = c[6] / fmaxf(on, 1e-30f);
            x *= sc;
            y *= sc;
            sdf = c[7] - dist3_32(c[0] * x + c[3] * y - qx, c[1] * x + c[4] * y - qy, c[2] * x + c[5] * y - qz);
            break;
        }
    }
    const float r = -sdf;
    *out = r;
    const float P = fmaxf(fmaxf(fabsf(pf.x), fabsf(pf.y)), fabsf(pf.z));
    const float Q = fmaxf(fmaxf(fabsf(qx), fabsf(qy)), fabsf(qz));
    const float eq = __fmul_ru(1.0506e-07f, __fadd_ru(__fadd_ru(P, b.amag), Q));  // 1.74 * 1.01 u (...)
    return __fadd_ru(eq, __fmul_ru(b.kint, __fadd_ru(__fadd_ru(Q, b.mag), fabsf(r)))) + guard;
}

__device__ __forceinline__ float powk_ru(float x, int k) {
    float r = 1.f, b = x;
    for (; k; k >>= 1) {
        if (k & 1) r = __fmul_ru(r, b);
        b = __fmul_ru(b, b);
    }
    return r;
}
__device__ __forceinline__ float powk_rd(float x, int k) {
    float r = 1.f, b = x;
    for (; k; k >>= 1) {
        if (k & 1) r = __fmul_rd(r, b);
        b = __fmul_rd(b, b);
    }
    return r;
}

__device__ __forceinline__ float powk_rn(float x, int k) {
    float r = 1.f, b = x;
    for (; k; k >>= 1) {
        if (k & 1) r = __fmul_rn(r, b);
        b = __fmul_rn(b, b);
    }
    return r;
}

// Bracket [tlo, thi] of r^-k over r in [rlo, rhi] (rlo <= r <= rhi, E =
// rhi - r): +Inf where r <= 0 is possible.  The fast form computes r^-k once,
// to nearest, and widens it by the relative change of r^-k over the
// interval: with rho >= E / rlo and k rho <= 1/4, (1 + rho)^-k >= 1 - k rho
// (convexity) and (1 - rho)^-k <= 1 + 2 k rho.  __fdividef is within 2 ulp
// for divisors in [2^-126, 2^126].  Otherwise directed rounding throughout.
__device__ __forceinline__ void power_bracket(const MetaF& m, float r, float E, float rlo, float rhi, float* tlo,
                                              float* thi) {
    if (m.k <= 64 && rlo >= 1.1754944e-38f && rhi <= 8.5e37f) {
        const float pk = powk_rn(r, m.k);
        if (pk >= 1.1754944e-38f && pk <= 8.5e37f) {
            const float tf = __fdividef(1.f, pk);
            const float krho = __fmul_ru((float)m.k, __fmul_ru(__fdividef(E, rlo), 1.0000005f));
            if (krho <= 0.25f) {
                *thi = __fmul_ru(tf, __fadd_ru(1.f, __fadd_ru(__fmul_ru(2.f, krho), m.eps_pow)));
                *tlo = __fmul_rd(tf, __fsub_rd(1.f, __fadd_ru(krho, m.eps_pow)));
                return;
            }
        }
    }
    *tlo = rhi <= 0.f ? INFINITY : __frcp_rd(powk_ru(rhi, m.k));
    *thi = rlo <= 0.f ? INFINITY : __frcp_ru(powk_rd(rlo, m.k));
}

// Bracket [lo, hi] of the weighted term w f(r) for r in [rlo, rhi]; false
// when 0 * Inf is possible (NaN in the reference's sum).
__device__ __forceinline__ bool term_bracket(const MetaF& m, bool power, const BallF& b, float r, float E, float rlo,
                                             float rhi, float* lo, float* hi, float* ab) {
    float tlo, thi;  // bracket of f(r) for r in [rlo, rhi]
    if (power) {
        power_bracket(m, r, E, rlo, rhi, &tlo, &thi);
    } else {
        if (rhi < 0.f) {
            tlo = INFINITY;
        } else if (rhi >= m.d_lo) {
            tlo = 0.f;
        } else {
            const float v = fmaxf(__fsub_rd(1.f, __fmul_ru(__fmul_ru(rhi, rhi), m.inv_d2_hi)), 0.f);
            tlo = __fmul_rd(v, v);
        }
        if (rlo < 0.f) {
            thi = INFINITY;
        } else if (rlo >= m.d_hi) {
            thi = 0.f;
        } else {
            const float v = __fsub_ru(1.f, __fmul_rd(__fmul_rd(rlo, rlo), m.inv_d2_lo));
            thi = __fmul_ru(v, v);
        }
    }
    if (b.w_lo > 0.f) {
        *lo = __fmul_rd(b.w_lo, tlo);
        *hi = __fmul_ru(b.w_hi, thi);
    } else if (b.w_hi < 0.f) {
        *lo = __fmul_rd(b.w_lo, thi);
        *hi = __fmul_ru(b.w_hi, tlo);
    } else {  // weight 0 (or below the float range): 0 * Inf is NaN
        if (thi == INFINITY) return false;
        *lo = __fmul_rd(b.w_lo, thi);
        *hi = __fmul_ru(b.w_hi, thi);
    }
    const float wabs = fmaxf(fabsf(b.w_lo), fabsf(b.w_hi));
    *ab = __fmul_ru(wabs, power ? thi : fmaxf(thi, 1.f));
    return true;
}

// The sum's decision from its bracket: 1/0 when decided, 2 otherwise.
__device__ __forceinline__ int sum_decision(const MetaF& m, float slo, float shi, float sabs) {
    if (!(slo == slo) || !(shi == shi)) return 2;
    if (slo == INFINITY) return 1;   // a certain +Inf term and no possible -Inf term
    if (shi == -INFINITY) return 0;  // a certain -Inf term and no possible +Inf term
    const float margin = __fmul_ru(sabs, 9.094947e-13f);  // 2^-40: float64's own roundings
    if (__fsub_rd(slo, margin) > m.thr_hi) return 1;
    if (__fadd_ru(shi, margin) <= m.thr_lo) return 0;
    return 2;
}

// The InBounds part of the filter: 0 outside, 1 inside (decided exactly).
__device__ __forceinline__ bool meta_in_bounds_32(const MetaD& md, const MetaF& m, P3 p, F3 pf) {
    // pf = fl(p) with fl monotone, so pf < fl_down(lo) implies p < lo.
    if (pf.x < m.lo_dn[0] || pf.y < m.lo_dn[1] || pf.z < m.lo_dn[2] || pf.x > m.hi_up[0] || pf.y > m.hi_up[1] ||
        pf.z > m.hi_up[2])
        return false;
    if (pf.x > m.lo_up[0] && pf.y > m.lo_up[1] && pf.z > m.lo_up[2] && pf.x < m.hi_dn[0] && pf.y < m.hi_dn[1] &&
        pf.z < m.hi_dn[2])
        return true;
    return meta_in_bounds(md, p);
}

// Sum brackets over the balls in `list` (all balls when list is null),
// starting from [slo, shi] / sabs.  1/0 when decided, 2 otherwise.
__device__ __forceinline__ int metaball_32_sum(const ProgView& P, const MetaD& md, const MetaF& m, P3 p, F3 pf,
                                               const uint16_t* list, int nl, float slo, float shi, float sabs) {
    const bool power = md.falloff == MC_FALLOFF_POWER;
    const int n = list ? nl : md.n_balls;
    for (int k = 0; k < n; k++) {
        const int i = md.first_ball + (list ? list[k] : k);
        const BallF& b = P.balls_f[i];
        F3 q = pf;
        if (b.n_steps) {
            const BallD& bd = P.balls[i];
            q = to_f3(apply_steps(P.xstep + bd.first_step, bd.n_steps, p));
        }
        float r;
        const float E = ball_field_32(b, q, &r);
        const float rlo = __fsub_rd(r, E), rhi = __fadd_ru(r, E);
        if (!(rlo == rlo) || !(rhi == rhi)) return 2;
        float lo, hi, ab;
        if (!term_bracket(m, power, b, r, E, rlo, rhi, &lo, &hi, &ab)) return 2;
        slo = __fadd_rd(slo, lo);
        shi = __fadd_ru(shi, hi);
        sabs = __fadd_ru(sabs, ab);
    }
    return sum_decision(m, slo, shi, sabs);
}

// FP32 filter of metaball_64: 1/0 when decided, 2 otherwise.
__device__ __noinline__ int metaball_32(const ProgView& P, const double* ld, P3 p, F3 pf) {
    const int id = (int)ld[0];
    const MetaD& md = P.metas[id];
    const MetaF& m = P.metas_f[id];
    if (md.never || !meta_in_bounds_32(md, m, p, pf)) return 0;
    if (m.esc_all) return 2;
    return metaball_32_sum(P, md, m, p, pf, nullptr, 0, 0.f, 0.f, 0.f);
}

// Far-field split for a classification tile.  For every ball without a
// transform, the field over the tile's box lies within E + h of its float
// value at the box centre (the SDF is 1-Lipschitz; h = the half-diagonal,
// widened for float64's own rounding).  The balls whose weighted-term
// brackets are narrowest, up to a total width of 2^-8 thr, are summed once
// here as brackets (the cut-off is the largest of 16 powers of two that
// keeps the total within budget); the others are listed and evaluated per
// corner.  A corner whose sum the combined bracket cannot decide goes to
// the full filter.
constexpr int kNearMax = 128;
constexpr int kCuts = 16;
struct MbRegion {
    float slo, shi, sabs;
    int nnear;  // -1: no split (too many near balls, or no budget)
    uint16_t near[kNearMax];
};

__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_sum_ru(float v) {  // directed sums bound the sum in any order
    for (int o = 16; o; o >>= 1) v = __fadd_ru(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_sum_rd(float v) {
    for (int o = 16; o; o >>= 1) v = __fadd_rd(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Bracket of ball i's weighted term over the box (centre c, radius h);
// false when the ball cannot be bracketed (transformed, NaN, 0 * Inf).
__device__ __forceinline__ bool region_term(const ProgView& P, const MetaD& md, const MetaF& m, bool power, int i,
                                            F3 c, float h, float* tl, float* th, float* ta) {
    const BallF& b = P.balls_f[md.first_ball + i];
    if (b.n_steps) return false;
    float r;
    const float rad = __fadd_ru(ball_field_32(b, c, &r), h);
    const float rlo = __fsub_rd(r, rad), rhi = __fadd_ru(r, rad);
    if (!(rlo == rlo) || !(rhi == rhi)) return false;
    if (!term_bracket(m, power, b, r, rad, rlo, rhi, tl, th, ta)) return false;
    return __fsub_ru(*th, *tl) < INFINITY;
}

// All 32 lanes call this.
__device__ void metaball_region(const ProgView& P, const MetaD& md, const MetaF& m, const float lo[3],
                                const float hi[3], MbRegion& R) {
    const int lane = threadIdx.x & 31;
    const bool power = md.falloff == MC_FALLOFF_POWER;
    const F3 c{0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), 0.5f * (lo[2] + hi[2])};
    const float hx = fmaxf(__fsub_ru(c.x, lo[0]), __fsub_ru(hi[0], c.x));
    const float hy = fmaxf(__fsub_ru(c.y, lo[1]), __fsub_ru(hi[1], c.y));
    const float hz = fmaxf(__fsub_ru(c.z, lo[2]), __fsub_ru(hi[2], c.z));
    const float cmax = fmaxf(fmaxf(fabsf(c.x), fabsf(c.y)), fabsf(c.z));
    const float h = __fadd_ru(__fmul_ru(__fsqrt_ru(__fadd_ru(__fadd_ru(__fmul_ru(hx, hx), __fmul_ru(hy, hy)),
                                                          __fmul_ru(hz, hz))), 1.000001f),
                              __fmul_ru(cmax, 9.3132257e-10f));  // + 2^-30 |c|
    const float budget = __fmul_rd(m.thr_lo, 0.00390625f);      // 2^-8 thr
    const float base = __fdiv_rd(budget, (float)md.n_balls);
    if (!(base > 0.f) || !(budget < INFINITY)) {
        if (lane == 0) R.nnear = -1;
        __syncwarp();
        return;
    }
    // Pass 1: total width below each cut-off base * 2^j.
    float tot[kCuts];
#pragma unroll
    for (int j = 0; j < kCuts; j++) tot[j] = 0.f;
    for (int i = lane; i < md.n_balls; i += 32) {
        float tl, th, ta;
        if (!region_term(P, md, m, power, i, c, h, &tl, &th, &ta)) continue;
        const float w = __fsub_ru(th, tl);
        float cut = base;
#pragma unroll
        for (int j = 0; j < kCuts; j++) {
            if (w <= cut) tot[j] = __fadd_ru(tot[j], w);
            cut *= 2.f;
        }
    }
    float tau = 0.f, cut = base;
#pragma unroll
    for (int j = 0; j < kCuts; j++) {
        if (warp_sum_ru(tot[j]) <= budget) tau = cut;
        cut *= 2.f;
    }
    // Pass 2: sum the far brackets, list the near balls.
    float slo = 0.f, shi = 0.f, sab = 0.f;
    int nn = 0;
    bool ok = tau > 0.f;
    for (int base_i = 0; base_i < md.n_balls; base_i += 32) {
        const int i = base_i + lane;
        bool far = false;
        float tl = 0.f, th = 0.f, ta = 0.f;
        if (ok && i < md.n_balls && region_term(P, md, m, power, i, c, h, &tl, &th, &ta))
            far = __fsub_ru(th, tl) <= tau;
        if (far) {
            slo = __fadd_rd(slo, tl);
            shi = __fadd_ru(shi, th);
            sab = __fadd_ru(sab, ta);
        }
        const bool near = i < md.n_balls && !far;
        const unsigned nm = __ballot_sync(0xffffffffu, near);
        if (nn + __popc(nm) > kNearMax) ok = false;
        if (ok && near) R.near[nn + __popc(nm & ((1u << lane) - 1u))] = (uint16_t)i;
        nn += __popc(nm);
    }
    slo = warp_sum_rd(slo);
    shi = warp_sum_ru(shi);
    sab = warp_sum_ru(sab);
    if (lane == 0) {
        R.slo = slo;
        R.shi = shi;
        R.sabs = sab;
        R.nnear = ok ? nn : -1;
    }
    __syncwarp();
}

}  // namespace mcgpu
