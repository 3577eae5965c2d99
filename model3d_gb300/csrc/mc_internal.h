// mc_internal.h — device program layout shared by the host lowering
// (mc_lower.cpp) and the CUDA kernels (mc_kernels.cu).
//
// A lowered Solid is:
//   * a postfix boolean program over a 32-deep bit stack (ops[]),
//   * a table of leaves (primitive predicates and collider parity tests),
//     each with FP64 constants in the reference's operation order and FP32
//     constants for the filtered predicate,
//   * a table of box checks (TRANSFORM / CHECKED nodes) with the inverse
//     transform steps of TRANSFORM nodes,
//   * collider trees: the reference's JoinedCollider boxes, one record per
//     triangle with its parent box, and a ray grid of candidate triangles.
#pragma once

#include <stdint.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace mcgpu {

// ---- postfix ops: opcode in bits 28..31, argument in bits 0..27.
enum Op : uint32_t {
    OP_LEAF = 1,    // push leaf[arg](point)
    OP_OR = 2,      // b = pop; top |= b
    OP_AND = 3,     // b = pop; top &= b
    OP_ANDNOT = 4,  // b = pop; top &= !b        (SubtractedSolid)
    OP_NOT = 5,     // top = !top                (only produced by folding)
    OP_XPUSH = 6,   // save point; point = inverse transform arg (point)
    OP_XPOP = 7,    // restore point; top &= inbox(arg, point)
    OP_BOX = 8,     // push inbox(arg, point)    (only produced by folding)
    OP_BOXAND = 9,  // top &= inbox(arg, point)  (CheckedFuncSolid)
    OP_TRUE = 10,
    OP_FALSE = 11,
    OP_JLEAVES = 12,  // push OR of leaves [a, a + n)   (arg = a << 14 | n; n-ary JoinedSolid)
    OP_ALEAVES = 13,  // push AND of leaves [a, a + n)  (n-ary IntersectedSolid)
    OP_JLIST = 14,    // push OR of the arg leaves whose ids follow as raw words (only produced by folding)
};
__host__ __device__ inline uint32_t range_first(uint32_t arg) { return arg >> 14; }
__host__ __device__ inline uint32_t range_count(uint32_t arg) { return arg & 0x3fffu; }
__host__ __device__ inline uint32_t make_op(uint32_t code, uint32_t arg) { return (code << 28) | arg; }
__host__ __device__ inline uint32_t op_code(uint32_t op) { return op >> 28; }
__host__ __device__ inline uint32_t op_arg(uint32_t op) { return op & 0x0fffffffu; }

// ---- leaf kinds (same values as the MC_NODE_* leaves of the ABI).
enum LeafKind : int32_t {
    LK_SPHERE = 1,
    LK_RECT = 2,
    LK_CYLINDER = 3,
    LK_CAPSULE = 4,
    LK_TORUS = 5,
    LK_COLLIDER = 6,
    LK_METABALL = 7,
};

// FP64 constants per leaf (doubles), kind-specific layout:
//   SPHERE   : c.xyz, TR                    (TR: largest S with sqrt_rn(S) <= R)
//   RECT     : min.xyz, max.xyz
//   CYLINDER : P2.xyz, dir.xyz, norm, TR
//   CAPSULE  : s0.xyz, s1.xyz, v.xyz, norm, TR
//   TORUS    : center.xyz, b1.xyz, b2.xyz, outer, T_inner (FP32 also T_lo, T_hi)
//   COLLIDER : min.xyz, max.xyz, (double)tree index
//   METABALL : (double)index into metas / metas_f
constexpr int LEAF_D = 16;
// FP32 filter constants per leaf (floats), same order rounded to float, plus
// thresholds: [..., TR_lo, TR_hi] / [..., norm_lo, norm_hi, TR_lo, TR_hi].
constexpr int LEAF_F = 16;

constexpr int MAX_STACK = 31;     // bit-stack depth limit
constexpr int MAX_XDEPTH = 8;     // nested transforms
constexpr int MAX_OPS = 1 << 16;  // program length limit

// Inverse transform step: kind (MC_XF_*), 9 parameters.
struct XStepD {
    int32_t kind;
    int32_t pad;
    double v[9];
};

// A box check (TRANSFORM or CHECKED node): the node's bounds; TRANSFORM nodes
// carry [first_step, first_step + n_steps) inverse steps in apply order.
struct XBoxD {
    double lo[3];
    double hi[3];
    int32_t first_step;
    int32_t n_steps;
};

// Collider trees.  The reference counts the triangles T that its ray test
// hits AND that its traversal reaches: every JoinedCollider box above T
// passes the slab test (collisions.go:263-273, bvh.go:322-351).  A parent
// box is the min/max of its children's boxes, so it lies inside every
// ancestor's box, and fl((b - o) / r) is monotone in b for r > 0: the
// float64 slab interval of an ancestor contains the parent's.  T is
// therefore reached iff the slab test of its parent box passes, and only
// that box is stored per triangle (`tri_parent`, -1 when the tree is a
// single triangle).
struct BvhNodeD {
    double lo[3];
    double hi[3];
};
struct BvhNodeF {  // FP32 copy of the node box, rounded outward
    float lo[3];
    float hi[3];
};
// Per-triangle Moller-Trumbore constants with the ray direction fixed
// (model3d/primitives.go:207-249, collisions.go:124): t0, v1, v2,
// cross1 = D x v2, invDet = 1 / (cross1 . v1), valid = !parallel && det != 0.
struct TriD {
    double t0[3];
    double v1[3];
    double v2[3];
    double c1[3];
    double inv_det;
    int32_t valid;
    int32_t pad;
};
struct TriF {
    float t0[3];
    float v1[3];
    float v2[3];
    float c1[3];
    float inv_det;
    int32_t valid;
};

// Ray grid.  Every containment ray has the direction D of collisions.go:124,
// so a ray is a point of the plane x = 0 once projected along D:
// (a, b) = (p.y - KY p.x, p.z - KZ p.x), and t(p) = p.x / D.x grows by s
// along o + s D.  Each valid triangle is listed in the cells its projected
// bounding box covers, widened by a pad that exceeds every rounding error of
// the reference's float64 test and of the float projection of the ray
// origin, so a ray that the reference's test can hit lists that triangle in
// its cell.  Within a cell the entries are sorted by the triangle's largest
// t (plus the pad): a ray only tests the suffix with maxt >= t(origin),
// since triangles entirely behind the origin have a negative scale.
// Ill-conditioned triangles (none in ordinary meshes) go to an `all` list
// tested by every ray of the tree.
constexpr double RAYGRID_KY = 0.10494477243214506 / 0.5224892708603626;
constexpr double RAYGRID_KZ = 0.43558938446126527 / 0.5224892708603626;
constexpr double RAYGRID_INV_DX = 1.0 / 0.5224892708603626;
struct RayEnt {
    float maxt;   // largest t over the triangle, rounded up, plus the pad
    int32_t tri;  // absolute triangle index
};
struct TreeD {
    int32_t kind;  // 0: no triangles (nullCollider); 1: triangles
    int32_t n_cells;
    float mbox[3]; // per axis, an upper bound of |coordinate| over every box of the tree
    float amin, bmin, inv_cs;  // grid origin (float) and 1 / cell size
    int32_t ga, gb;            // cells along a and b
    int32_t cell_base;         // this tree's first cell_start entry
    int32_t all_first, all_count;  // RayEnt range tested by every ray
};

// Kernel mode: bit 0 is the precision (MC_PREC_*); MODE_MB adds the metaball
// leaf path.  Programs without metaball leaves run kernels built without it,
// so the evaluation loops of the other kinds compile as if it did not exist.
constexpr int MODE_MB = 2;
__host__ __device__ constexpr bool mode_f32(int mode) { return (mode & 1) == 1; }
__host__ __device__ constexpr bool mode_mb(int mode) { return (mode & MODE_MB) != 0; }

// Metaball leaves: WeightedMetaballSolid (model3d/metaball.go:165-242) is
// InBounds(lo, hi) && sum_i w_i f(-SDF_i(inv_i(c))) > thr, summed in ball
// order in float64.  The FP32 filter brackets every -SDF_i by an absolute
// error bound kerr * (S + |r|) (S = largest |coordinate| of the point plus the
// largest |constant| of the ball), brackets f over that interval with directed
// rounding, sums lower and upper bounds, and decides when the bracket (widened
// by 2^-40 of the summed magnitudes for the float64 roundings) clears thr.
constexpr int MAX_BALLS = 4096;
struct MetaD {
    double lo[3], hi[3];  // bounds of the CheckedFuncSolid
    double thr;           // f(radiusThreshold)
    double param;         // power k (MC_FALLOFF_POWER) or d (MC_FALLOFF_WYVILL)
    double d2;            // d * d, as the Wyvill closure precomputes it
    int32_t falloff;      // MC_FALLOFF_*
    int32_t first_ball, n_balls;
    int32_t never;        // thr is +Inf or NaN: sum > thr never holds
};
struct MetaF {
    float lo_dn[3], lo_up[3], hi_dn[3], hi_up[3];  // bounds rounded down / up
    float thr_lo, thr_hi;
    float d_lo, d_hi;
    float inv_d2_lo, inv_d2_hi;  // bounds of 1 / (d * d) (Wyvill)
    float eps_pow;    // relative error bound of the float r^-k (k <= 64), with margin
    int32_t k;        // power (MC_FALLOFF_POWER)
    int32_t esc_all;  // parameters outside the filter's range: always float64
};
// One ball; float64 constants by primitive (LK_*), for the exact path:
//   SPHERE   : center.xyz, R
//   RECT     : min.xyz, max.xyz
//   CAPSULE  : P1.xyz, P2.xyz, axis.xyz, norm, R       (axis = (P2-P1) * (1/norm))
//   CYLINDER : the capsule's 11, then OrthoBasis(-axis) (P1 cap) and
//              OrthoBasis(axis) (P2 cap): b1.xyz, b2.xyz each
//   TORUS    : center.xyz, b1.xyz, b2.xyz, outer, inner (b1, b2 = OrthoBasis(Axis))
// The FP32 filter works relative to an anchor A (the sphere's and torus's
// centre, the rect's centre, the capsule's and cylinder's P1), so that its
// rounding errors scale with the distance to the ball, not with the
// coordinates.  Float constants, relative to A:
//   SPHERE   : R
//   RECT     : (min - A).xyz, (max - A).xyz
//   CAPSULE  : (P2 - A).xyz, axis.xyz, norm, R
//   CYLINDER : the capsule's 8, then the four basis vectors
//   TORUS    : b1.xyz, b2.xyz, outer, inner
constexpr int BALL_C = 24;
struct BallD {
    int32_t kind;
    int32_t first_step, n_steps;  // inverse transform steps in xstep, apply order
    int32_t pad;
    double w;
    double c[BALL_C];
};
struct BallF {
    float w_lo, w_hi;  // weight rounded down / up
    float mag;         // largest |relative constant| (lengths, radii, offsets from A)
    float kint;        // internal rounding factor of the kind (times u)
    int32_t kind;      // as BallD, so the common path reads one record
    int32_t n_steps;
    float a[3];        // the anchor rounded to float
    float amag;        // max |a|
    float c[BALL_C];
};

// Device view of one lowered solid (passed by value to kernels).
struct ProgView {
    const uint32_t* ops;
    const uint32_t* ops_allfalse;  // program folded with every leaf culled
    const int32_t* leaf_kind;
    const double* leaf_d;   // n_leaves * LEAF_D
    const float* leaf_f;    // n_leaves * LEAF_F
    const double* cull;     // n_leaves * 6: lo.xyz, hi.xyz (world space, widened); NaN = never cull
    const float* cull_f;    // the same boxes rounded outward to float
    const XBoxD* xbox;
    const XStepD* xstep;
    const TreeD* trees;
    const BvhNodeD* nodes;
    const BvhNodeF* nodes_f;
    const int32_t* tri_parent;  // parent box of each triangle, -1 for a single-triangle tree
    const int32_t* cell_start;  // per tree: n_cells + 1 offsets into ents
    const RayEnt* ents;
    const TriD* tris;
    const TriF* tris_f;
    const MetaD* metas;
    const MetaF* metas_f;
    const BallD* balls;
    const BallF* balls_f;
    int32_t n_ops;
    int32_t n_ops_allfalse;  // -1: const false, -2: const true, else length
    int32_t n_leaves;
    int32_t n_xbox;
    int32_t has_metaball;  // launch the kernels built with the metaball path (MODE_MB)
    int32_t rows_ok;  // no TRANSFORM node: tiles may be evaluated row-vectorised
    int32_t fold_cap; // longest folded program (words)
};

// ---- Bisection arithmetic on float64 bit patterns.
// When both ends of a search edge have the same sign and exponent field E
// (every double between them does too) the reference's midpoint
// (f + t) / 2 is a pure mantissa operation: with K = (2^52 + M_f) +
// (2^52 + M_t) in [2^53, 2^54 - 2], f + t rounds to RNE(K / 2) at exponent
// E + 1 and the halving is exact, so the midpoint is RNE(K / 2) at exponent
// E (no carry out: K / 2 < 2^53).  E must keep f + t finite (E <= 0x7fd).
// The float rounding of such a value is RNE of its 53-bit significand to 24
// bits at float exponent E - 896, exact for E in [897, 1150] (normal floats;
// a carry out of the significand bumps the exponent, up to infinity).
constexpr unsigned long long kFrac52 = (1ull << 52) - 1;

__host__ __device__ inline bool bisect_bits_ok(unsigned long long a, unsigned long long b) {
    const unsigned long long e = (a >> 52) & 0x7ff;
    return (a >> 52) == (b >> 52) && e >= 897 && e <= 1150;
}

__host__ __device__ inline unsigned long long mid_bits(unsigned long long a, unsigned long long b) {
    const unsigned long long K = (a & kFrac52) + (b & kFrac52) + (1ull << 53);
    const unsigned long long h = K >> 1;
    const unsigned long long m = h + (K & h & 1ull);  // ties to even
    return (a & ~kFrac52) | (m & kFrac52);
}

__host__ __device__ inline uint32_t float_bits_of(unsigned long long d) {
    const unsigned long long M = (d & kFrac52) | (1ull << 52);
    unsigned long long m24 = M >> 29;
    const unsigned long long rem = M & ((1ull << 29) - 1);
    m24 += (rem > (1ull << 28) || (rem == (1ull << 28) && (m24 & 1ull))) ? 1ull : 0ull;
    const uint32_t fe = (uint32_t)((d >> 52) & 0x7ff) - 896u;
    return ((uint32_t)(d >> 63) << 31) | ((fe << 23) + (uint32_t)m24 - (1u << 23));
}

// Constant folding of a postfix program given which leaves are active
// (inactive leaves are known false over the region being evaluated).
// Writes the pruned program to q and returns its length, or FOLD_FALSE /
// FOLD_TRUE when the whole program is constant.  Fragments of a postfix
// program are contiguous, so discarding a folded subtree is a truncation.
// The stack needs MAX_STACK + MAX_XDEPTH + 2 entries.
constexpr int FOLD_FALSE = -1;
constexpr int FOLD_TRUE = -2;
constexpr int FOLD_STACK = MAX_STACK + MAX_XDEPTH + 2;

__host__ __device__ inline int ctz32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __ffs((int)x) - 1;
#else
    return __builtin_ctz(x);
#endif
}

__host__ __device__ inline int popcount32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

// Bits of word w that fall in [a, e).
__host__ __device__ inline uint32_t range_mask(uint32_t w, uint32_t a, uint32_t e) {
    uint32_t m = ~0u;
    if ((w << 5) < a) m &= ~0u << (a & 31);
    if (((w + 1) << 5) > e) m &= (e & 31) ? ((1u << (e & 31)) - 1u) : ~0u;
    return m;
}

// act: one bit per leaf (32 per word); nullptr means every leaf is inactive.
__host__ __device__ inline bool leaf_active(const uint32_t* act, uint32_t l) {
    return act && ((act[l >> 5] >> (l & 31)) & 1u);
}

__host__ __device__ inline int fold_program(const uint32_t* ops, int n, const uint32_t* act, uint32_t* q) {
    // Entries: >= 0 fragment start; -1 const false; -2 const true; <= -3 marker (-3 - start).
    int stk[FOLD_STACK];
    int sp = 0, qn = 0;
    for (int i = 0; i < n; i++) {
        uint32_t op = ops[i];
        uint32_t code = op_code(op), arg = op_arg(op);
        switch (code) {
            case OP_LEAF:
                if (leaf_active(act, arg)) {
                    stk[sp++] = qn;
                    q[qn++] = op;
                } else {
                    stk[sp++] = FOLD_FALSE;
                }
                break;
            case OP_JLEAVES:
            case OP_ALEAVES: {
                // Count the active leaves of the range word by word.
                const uint32_t a = range_first(arg), cnt = range_count(arg), e = a + cnt;
                uint32_t k = 0;
                if (act)
                    for (uint32_t w = a >> 5; w <= ((e - 1) >> 5); w++) k += popcount32(act[w] & range_mask(w, a, e));
                if (k == 0 || (code == OP_ALEAVES && k < cnt)) {
                    stk[sp++] = FOLD_FALSE;  // an inactive leaf is false everywhere here
                } else if (k == cnt) {
                    stk[sp++] = qn;
                    q[qn++] = op;
                } else {
                    stk[sp++] = qn;
                    if (k > 1) q[qn++] = make_op(OP_JLIST, k);
                    for (uint32_t w = a >> 5; w <= ((e - 1) >> 5); w++) {
                        uint32_t bits = act[w] & range_mask(w, a, e);
                        while (bits) {
                            uint32_t l = (w << 5) + (uint32_t)ctz32(bits);
                            bits &= bits - 1;
                            q[qn++] = k > 1 ? l : make_op(OP_LEAF, l);
                        }
                    }
                }
                break;
            }
            case OP_TRUE: stk[sp++] = FOLD_TRUE; break;
            case OP_FALSE: stk[sp++] = FOLD_FALSE; break;
            case OP_OR:
            case OP_AND: {
                int b = stk[--sp], a = stk[--sp];
                int dom = code == OP_OR ? FOLD_TRUE : FOLD_FALSE;   // absorbing constant
                int neu = code == OP_OR ? FOLD_FALSE : FOLD_TRUE;   // neutral constant
                if (a == dom || b == dom) {
                    if (a >= 0) qn = a;
                    else if (b >= 0) qn = b;
                    stk[sp++] = dom;
                } else if (a == neu) {
                    stk[sp++] = b;
                } else if (b == neu) {
                    stk[sp++] = a;
                } else {
                    q[qn++] = op;
                    stk[sp++] = a;
                }
                break;
            }
            case OP_ANDNOT: {  // a && !b
                int b = stk[--sp], a = stk[--sp];
                if (b == FOLD_TRUE || a == FOLD_FALSE) {
                    if (a >= 0) qn = a;
                    else if (b >= 0) qn = b;
                    stk[sp++] = FOLD_FALSE;
                } else if (b == FOLD_FALSE) {
                    stk[sp++] = a;
                } else if (a == FOLD_TRUE) {
                    q[qn++] = make_op(OP_NOT, 0);
                    stk[sp++] = b;
                } else {
                    q[qn++] = op;
                    stk[sp++] = a;
                }
                break;
            }
            case OP_NOT: {
                int a = stk[--sp];
                if (a == FOLD_TRUE) stk[sp++] = FOLD_FALSE;
                else if (a == FOLD_FALSE) stk[sp++] = FOLD_TRUE;
                else {
                    q[qn++] = op;
                    stk[sp++] = a;
                }
                break;
            }
            case OP_XPUSH:
                stk[sp++] = -3 - qn;
                q[qn++] = op;
                break;
            case OP_XPOP: {
                int e = stk[--sp];
                int ms = -3 - stk[--sp];
                if (e == FOLD_FALSE) {
                    qn = ms;
                    stk[sp++] = FOLD_FALSE;
                } else if (e == FOLD_TRUE) {
                    qn = ms;
                    q[qn++] = make_op(OP_BOX, arg);
                    stk[sp++] = ms;
                } else {
                    q[qn++] = op;
                    stk[sp++] = ms;
                }
                break;
            }
            case OP_BOX:
                stk[sp++] = qn;
                q[qn++] = op;
                break;
            case OP_BOXAND: {
                int a = stk[--sp];
                if (a == FOLD_FALSE) {
                    stk[sp++] = FOLD_FALSE;
                } else if (a == FOLD_TRUE) {
                    stk[sp++] = qn;
                    q[qn++] = make_op(OP_BOX, arg);
                } else {
                    q[qn++] = op;
                    stk[sp++] = a;
                }
                break;
            }
            default: break;
        }
    }
    int r = sp > 0 ? stk[0] : FOLD_FALSE;
    return r >= 0 ? qn : r;
}

}  // namespace mcgpu
