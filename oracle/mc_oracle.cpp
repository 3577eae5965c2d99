// mc_oracle.cpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// A CPU restatement of unixpickle/model3d's MarchingCubesSearch path, used by
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
// checker.  Nothing in the model3d_gb300 package links, imports or calls it.
//
// Every function follows the reference's float64 operation order (Go does not
// fuse a*b+c on amd64 with the default GOAMD64=v1; this file is compiled with
// -ffp-contract=off so GCC does not fuse either).  Citations are
// file:line inside the reference project.
//
// Parity status: the reference is Go and no Go toolchain exists on either
// machine, so this restatement cannot be diffed against reference output.
// It is pinned by the reference's own property tests restated in
// tests/test_oracle.py (lookup-table determinism and coverage, mesh
// manifoldness, sphere volume, out-of-bounds containment, collider vs brute
// force) and by hand-derived known answers (spacer counts).  No golden meshes
// exist in the reference (model3d/mc_test.go has none).
//
// Deviation (documented): GroupTriangles sorts with Go's unstable sort.Slice
// (model3d/bvh.go:219-255) over a slice in Go map order, so the reference's
// own collider tree is not deterministic on ties.  Here ties are broken by
// input order (std::stable_sort), and the product does the same.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../include/mcgpu.h"

namespace {

// ------------------------------------------------------------------ Go math

// math.Min (Go): NaN if either is NaN; -0 beats +0.
inline double go_min(double x, double y) {
    if (std::isinf(x) && x < 0) return x;
    if (std::isinf(y) && y < 0) return y;
    if (std::isnan(x) || std::isnan(y)) return std::numeric_limits<double>::quiet_NaN();
    if (x == 0 && x == y) return std::signbit(x) ? x : y;
    return x < y ? x : y;
}
// math.Max (Go).
inline double go_max(double x, double y) {
    if (std::isinf(x) && x > 0) return x;
    if (std::isinf(y) && y > 0) return y;
    if (std::isnan(x) || std::isnan(y)) return std::numeric_limits<double>::quiet_NaN();
    if (x == 0 && x == y) return std::signbit(x) ? y : x;
    return x > y ? x : y;
}

// Coord3D (model3d/coords.go:84-467).
struct V3 {
    double x = 0, y = 0, z = 0;
};
inline V3 xyz(double x, double y, double z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
inline double at(const V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
inline void set(V3& v, int i, double a) { if (i == 0) v.x = a; else if (i == 1) v.y = a; else v.z = a; }
inline V3 add(V3 a, V3 b) { return xyz(a.x + b.x, a.y + b.y, a.z + b.z); }          // coords.go:251-257
inline V3 scale(V3 a, double s) { return xyz(a.x * s, a.y * s, a.z * s); }           // coords.go:233-239
inline V3 sub(V3 a, V3 b) { return add(a, scale(b, -1)); }                            // coords.go:260-262
inline V3 add_scalar(V3 a, double s) { return xyz(a.x + s, a.y + s, a.z + s); }      // coords.go:243-248
inline V3 mul(V3 a, V3 b) { return xyz(a.x * b.x, a.y * b.y, a.z * b.z); }           // coords.go:225-227
inline V3 recip(V3 a) { return xyz(1 / a.x, 1 / a.y, 1 / a.z); }                      // coords.go:235-237
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }          // coords.go:211-213
inline V3 cross(V3 a, V3 b) {                                                          // coords.go:216-222
    return xyz(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline double norm(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }   // coords.go:201-203
inline V3 normalize(V3 a) { return scale(a, 1 / norm(a)); }                          // coords.go:379-381
inline V3 mid(V3 a, V3 b) { return scale(add(a, b), 0.5); }                          // coords.go:196-198
inline double dist(V3 a, V3 b) {                                                       // coords.go:272-277
    double d1 = a.x - b.x, d2 = a.y - b.y, d3 = a.z - b.z;
    return std::sqrt(d1 * d1 + d2 * d2 + d3 * d3);
}
inline V3 vmin(V3 a, V3 b) { return xyz(go_min(a.x, b.x), go_min(a.y, b.y), go_min(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return xyz(go_max(a.x, b.x), go_max(a.y, b.y), go_max(a.z, b.z)); }
// Go == on Coord3D: element-wise ==, so -0 == +0 and NaN != NaN.
inline bool veq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline double vsum(V3 a) { return a.x + a.y + a.z; }

// InBounds (model3d/bounder.go:23-27).
inline bool in_bounds(V3 mn, V3 mx, V3 c) { return veq(vmin(c, mn), mn) && veq(vmax(c, mx), mx); }

// OrthoBasis (model3d/coords.go:388-422).
void ortho_basis(V3 c, V3* out1, V3* out2) {
    double absX = std::fabs(c.x), absY = std::fabs(c.y), absZ = std::fabs(c.z);
    V3 b1;
    if (absX > absY && absX > absZ) {
        b1.x = c.y / absX;
        b1.y = -c.x / absX;
    } else {
        b1.y = c.z;
        b1.z = -c.y;
        if (absY > absZ) {
            b1.y /= absY;
            b1.z /= absY;
        } else {
            b1.y /= absZ;
            b1.z /= absZ;
        }
    }
    V3 b2 = xyz(b1.y * c.z - b1.z * c.y, b1.z * c.x - b1.x * c.z, b1.x * c.y - b1.y * c.x);
    *out1 = normalize(b1);
    *out2 = normalize(b2);
}

// ProjectOut (model3d/coords.go:425-428).
inline V3 project_out(V3 c, V3 c1) {
    V3 normed = normalize(c1);
    return sub(c, scale(normed, dot(normed, c)));
}

// circleAxisBound (model3d/shapes.go:562-571).
double circle_axis_bound(int axis, V3 normal, double sign) {
    V3 arr;
    set(arr, axis, sign);
    V3 proj = project_out(arr, normal);
    proj = scale(proj, 1 / (norm(proj) + 1e-8));
    return sign * (std::fabs(at(proj, axis)) + 1e-8);
}

// Matrix3 (model3d/matrix.go:12-146).
struct M3 {
    double m[9];
};
inline double det3(const M3& a) {  // matrix.go:56-58
    const double* m = a.m;
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
           m[2] * (m[3] * m[7] - m[4] * m[6]);
}
M3 inverse3(const M3& a) {  // matrix.go:68-92
    double det = det3(a);
    const double* m = a.m;
    M3 r = {{m[4] * m[8] - m[5] * m[7], m[2] * m[7] - m[1] * m[8], m[1] * m[5] - m[2] * m[4],
             m[5] * m[6] - m[3] * m[8], m[0] * m[8] - m[2] * m[6], m[2] * m[3] - m[0] * m[5],
             m[3] * m[7] - m[4] * m[6], m[1] * m[6] - m[0] * m[7], m[0] * m[4] - m[1] * m[3]}};
    double s = 1 / det;
    for (double& x : r.m) x = x * s;
    return r;
}
inline V3 mul_column(const M3& a, V3 c) {  // matrix.go:131-137
    const double* m = a.m;
    return xyz(m[0] * c.x + m[1] * c.y + m[2] * c.z, m[3] * c.x + m[4] * c.y + m[5] * c.z,
               m[6] * c.x + m[7] * c.y + m[8] * c.z);
}

// ------------------------------------------------------------ statistics

struct Counters {
    std::atomic<int64_t> contains{0}, leaf{0}, bvh_nodes{0}, bvh_tris{0};
};
thread_local int64_t tl_leaf = 0, tl_nodes = 0, tl_tris = 0;

// ------------------------------------------------------------------ solids

struct Solid {
    virtual ~Solid() {}
    virtual V3 Min() const = 0;
    virtual V3 Max() const = 0;
    virtual bool Contains(V3 c) const = 0;
    // SDF (negative outside), for the primitives that are metaballs.
    virtual double SDF(V3) const { throw std::runtime_error("not a metaball primitive"); }
};

// Sphere (model3d/shapes.go:13-31).
struct Sphere : Solid {
    V3 center;
    double radius;
    V3 Min() const override { return add_scalar(center, -radius); }
    V3 Max() const override { return add_scalar(center, radius); }
    bool Contains(V3 c) const override {
        tl_leaf++;
        return dist(c, center) <= radius;
    }
    double SDF(V3 c) const override { return radius - dist(c, center); }  // shapes.go:100-102
};

// Rect (model3d/shapes.go:145-173).
struct RectS : Solid {
    V3 mn, mx;
    V3 Min() const override { return mn; }
    V3 Max() const override { return mx; }
    bool Contains(V3 c) const override {
        tl_leaf++;
        return veq(vmin(c, mn), mn) && veq(vmax(c, mx), mx);
    }
    double SDF(V3 c) const override {  // genericSDF, shapes.go:270-317
        if (!(veq(vmin(c, mn), mn) && veq(vmax(c, mx), mx))) return -dist(c, vmax(vmin(c, mx), mn));
        double d = std::numeric_limits<double>::infinity();
        for (int i = 0; i < 3; i++) {
            double axisD = go_min(at(c, i) - at(mn, i), at(mx, i) - at(c, i));
            if (axisD < d) d = axisD;
        }
        return d;
    }
};

// Cylinder (model3d/shapes.go:542-598).
struct Cylinder : Solid {
    V3 p1, p2;
    double radius;
    V3 Min() const override {
        V3 minCenter = vmin(p1, p2);
        V3 axis = sub(p2, p1);
        V3 off = scale(xyz(circle_axis_bound(0, axis, -1), circle_axis_bound(1, axis, -1),
                           circle_axis_bound(2, axis, -1)),
                       radius);
        return add(minCenter, off);
    }
    V3 Max() const override {
        V3 maxCenter = vmax(p1, p2);
        V3 axis = sub(p2, p1);
        V3 off = scale(xyz(circle_axis_bound(0, axis, 1), circle_axis_bound(1, axis, 1),
                           circle_axis_bound(2, axis, 1)),
                       radius);
        return add(maxCenter, off);
    }
    bool Contains(V3 p) const override {
        tl_leaf++;
        V3 diff = sub(p1, p2);
        V3 direction = normalize(diff);
        double frac = dot(sub(p, p2), direction);
        if (frac < 0 || frac > norm(diff)) return false;
        V3 projection = add(p2, scale(direction, frac));
        return dist(projection, p) <= radius;
    }
    double SDF(V3 c) const override;
};

// Segment (model3d/primitives.go:543-594).
struct Segment {
    V3 a, b;
};
Segment new_segment(V3 p1, V3 p2) {
    if (p1.x < p2.x || (p1.x == p2.x && p1.y < p2.y) ||
        (p1.x == p2.x && p1.y == p2.y && p1.z < p2.z))
        return {p1, p2};
    return {p2, p1};
}
V3 segment_closest(const Segment& s, V3 c) {
    V3 v1 = sub(s.b, s.a);
    double nrm = norm(v1);
    V3 v = scale(v1, 1 / nrm);
    V3 v2 = sub(c, s.a);
    double mag = dot(v, v2);
    if (mag > nrm) return s.b;
    if (mag < 0) return s.a;
    return add(scale(v, mag), s.a);
}

// Capsule (model3d/shapes.go:348-368).
struct Capsule : Solid {
    V3 p1, p2;
    double radius;
    V3 Min() const override { return add_scalar(vmin(p1, p2), -radius); }
    V3 Max() const override { return add_scalar(vmax(p1, p2), radius); }
    bool Contains(V3 c) const override {
        tl_leaf++;
        Segment seg = new_segment(p1, p2);
        return dist(c, segment_closest(seg, c)) <= radius;
    }
    double SDF(V3 c) const override {  // genericSDF, shapes.go:481-514
        V3 v = sub(p2, p1);
        double nrm = norm(v);
        V3 axis = scale(v, 1 / nrm);
        double d = dot(sub(c, p1), axis);
        if (d < 0 || d > nrm) return radius - dist(c, d < 0 ? p1 : p2);  // proxy Sphere.SDF
        return radius - dist(c, segment_closest(Segment{p1, p2}, c));   // Segment{P1, P2}.Dist
    }
};

// filledCircleDist (model3d/shapes.go:783-812) without the normal/point outputs.
void filled_circle_dist(V3 c, V3 center, V3 axis, double radius, double* cur) {
    V3 b1, b2;
    ortho_basis(axis, &b1, &b2);
    M3 mat;  // NewMatrix3Columns(b1, b2, axis).Transpose(): rows b1, b2, axis
    double rows[9] = {b1.x, b1.y, b1.z, b2.x, b2.y, b2.z, axis.x, axis.y, axis.z};
    for (int i = 0; i < 9; i++) mat.m[i] = rows[i];
    V3 proj = mul_column(mat, sub(c, center));
    double norm2 = std::sqrt(proj.x * proj.x + proj.y * proj.y);  // proj.XY().Norm()
    if (norm2 < radius) {
        double d = std::fabs(proj.z);
        if (d <= *cur) *cur = d;
    } else {
        norm2 -= radius;
        double d = std::sqrt(norm2 * norm2 + proj.z * proj.z);
        if (d <= *cur) *cur = d;
    }
}

// Cylinder.genericSDF (model3d/shapes.go:746-781).
double Cylinder::SDF(V3 c) const {
    V3 axis = sub(p2, p1);
    double nrm = norm(axis);
    axis = scale(axis, 1 / nrm);
    double d_ = std::numeric_limits<double>::infinity();
    bool contained = false;
    double d = dot(axis, sub(c, p1));
    if (d >= 0 && d < nrm) {
        double sd = radius - dist(c, segment_closest(Segment{p1, p2}, c));
        if (sd > 0) {
            contained = true;
            d_ = sd;
        } else {
            d_ = -sd;
        }
    }
    filled_circle_dist(c, p1, scale(axis, -1), radius, &d_);
    filled_circle_dist(c, p2, axis, radius, &d_);
    return contained ? d_ : -d_;
}

// Torus (model3d/shapes.go:1323-1365, genericSDF :1451-1487).
struct Torus : Solid {
    V3 center, axis;
    double outer, inner;
    V3 Min() const override {
        V3 extra = xyz(inner, inner, inner);
        V3 off = scale(xyz(circle_axis_bound(0, axis, -1), circle_axis_bound(1, axis, -1),
                           circle_axis_bound(2, axis, -1)),
                       outer);
        return sub(add(off, center), extra);
    }
    V3 Max() const override {
        V3 extra = xyz(inner, inner, inner);
        V3 off = scale(xyz(circle_axis_bound(0, axis, 1), circle_axis_bound(1, axis, 1),
                           circle_axis_bound(2, axis, 1)),
                       outer);
        return add(add(off, center), extra);
    }
    double SDF(V3 c) const override {
        V3 b1, b2;
        ortho_basis(axis, &b1, &b2);
        V3 centered = sub(c, center);
        double x = dot(b1, centered);
        double y = dot(b2, centered);
        double outerNorm = std::sqrt(x * x + y * y);
        if (outerNorm == 0) {
            x = 1;
            y = 0;
            outerNorm = 1;
        }
        double sc = outer / outerNorm;
        x *= sc;
        y *= sc;
        V3 ringPoint = add(scale(b1, x), scale(b2, y));
        return inner - dist(ringPoint, centered);
    }
    bool Contains(V3 c) const override {
        tl_leaf++;
        return SDF(c) >= 0;
    }
};

// JoinedSolid (model3d/solid.go:71-98).
struct Joined : Solid {
    std::vector<std::unique_ptr<Solid>> ch;
    V3 Min() const override {
        V3 m = ch[0]->Min();
        for (size_t i = 1; i < ch.size(); i++) m = vmin(m, ch[i]->Min());
        return m;
    }
    V3 Max() const override {
        V3 m = ch[0]->Max();
        for (size_t i = 1; i < ch.size(); i++) m = vmax(m, ch[i]->Max());
        return m;
    }
    bool Contains(V3 c) const override {
        for (auto& s : ch)
            if (s->Contains(c)) return true;
        return false;
    }
};

// SubtractedSolid (model3d/solid.go:120-142).
struct Subtracted : Solid {
    std::unique_ptr<Solid> pos, neg;
    V3 Min() const override { return pos->Min(); }
    V3 Max() const override { return pos->Max(); }
    bool Contains(V3 c) const override { return pos->Contains(c) && !neg->Contains(c); }
};

// IntersectedSolid (model3d/solid.go:144-172).
struct Intersected : Solid {
    std::vector<std::unique_ptr<Solid>> ch;
    V3 Min() const override {
        V3 b = ch[0]->Min();
        for (size_t i = 1; i < ch.size(); i++) b = vmax(b, ch[i]->Min());
        return b;
    }
    V3 Max() const override {
        V3 b = ch[0]->Max();
        for (size_t i = 1; i < ch.size(); i++) b = vmin(b, ch[i]->Max());
        return vmax(b, Min());
    }
    bool Contains(V3 c) const override {
        for (auto& s : ch)
            if (!s->Contains(c)) return false;
        return true;
    }
};

// One step of a (possibly joined) transform (model3d/transform.go:40-230).
struct XStep {
    int kind;  // MC_XF_*
    V3 v;
    double s = 0;
    M3 m;
    V3 apply(V3 c) const {
        switch (kind) {
            case MC_XF_TRANSLATE: return add(c, v);         // transform.go:44-46
            case MC_XF_SCALE: return scale(c, s);           // transform.go:71-73
            case MC_XF_VECSCALE: return mul(c, v);          // transform.go:104-106
            default: return mul_column(m, c);               // transform.go:131-133
        }
    }
    void apply_bounds(V3* mn, V3* mx) const {
        switch (kind) {
            case MC_XF_TRANSLATE:  // transform.go:48-50
                *mn = add(*mn, v);
                *mx = add(*mx, v);
                return;
            case MC_XF_SCALE:  // transform.go:75-81
                if (s < 0) {
                    V3 a = scale(*mx, s), b = scale(*mn, s);
                    *mn = a;
                    *mx = b;
                } else {
                    *mn = scale(*mn, s);
                    *mx = scale(*mx, s);
                }
                return;
            case MC_XF_VECSCALE: {  // transform.go:108-112
                V3 a = mul(*mn, v), b = mul(*mx, v);
                *mn = vmin(a, b);
                *mx = vmax(b, a);
                return;
            }
            default: {  // transform.go:135-151
                V3 nmin, nmax;
                double xs[2] = {mn->x, mx->x}, ys[2] = {mn->y, mx->y}, zs[2] = {mn->z, mx->z};
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++)
                        for (int k = 0; k < 2; k++) {
                            V3 c = mul_column(m, xyz(xs[i], ys[j], zs[k]));
                            if (i == 0 && j == 0 && k == 0) {
                                nmin = c;
                                nmax = c;
                            } else {
                                nmin = vmin(nmin, c);
                                nmax = vmax(nmax, c);
                            }
                        }
                *mn = nmin;
                *mx = nmax;
                return;
            }
        }
    }
    XStep inverse() const {
        XStep r = *this;
        switch (kind) {
            case MC_XF_TRANSLATE: r.v = scale(v, -1); break;  // transform.go:52-54
            case MC_XF_SCALE: r.s = 1 / s; break;             // transform.go:83-85
            case MC_XF_VECSCALE: r.v = recip(v); break;       // transform.go:114-116
            default: r.m = inverse3(m); break;                // transform.go:153-155
        }
        return r;
    }
};

// TransformSolid (model3d/transform.go:240-247) = CheckedFuncSolid + inv.Apply.
struct Transformed : Solid {
    std::vector<XStep> fwd, inv;
    std::unique_ptr<Solid> child;
    V3 mn, mx;
    void init() {
        mn = child->Min();
        mx = child->Max();
        for (auto& s : fwd) s.apply_bounds(&mn, &mx);  // JoinedTransform.ApplyBounds
        inv.clear();
        for (int i = (int)fwd.size() - 1; i >= 0; i--) inv.push_back(fwd[i].inverse());
    }
    V3 Min() const override { return mn; }
    V3 Max() const override { return mx; }
    bool Contains(V3 c) const override {
        if (!(veq(vmin(c, mn), mn) && veq(vmax(c, mx), mx))) return false;  // solid.go:46-50
        V3 p = c;
        for (auto& s : inv) p = s.apply(p);
        return child->Contains(p);
    }
};

// CheckedFuncSolid over a child (model3d/solid.go:46-50, :294-318).
struct Checked : Solid {
    std::unique_ptr<Solid> child;
    V3 mn, mx;
    V3 Min() const override { return mn; }
    V3 Max() const override { return mx; }
    bool Contains(V3 c) const override {
        return veq(vmin(c, mn), mn) && veq(vmax(c, mx), mx) && child->Contains(c);
    }
};

// --------------------------------------------------------------- metaballs

// math.Ldexp (Go math/ldexp.go): normal results exact; a subnormal result is
// scaled into range and multiplied by 2^-53 (one rounding).
double go_ldexp(double frac, long exp) {
    if (frac == 0 || std::isinf(frac) || std::isnan(frac)) return frac;
    if (std::fabs(frac) < 2.2250738585072014e-308) {  // normalize
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

// math.Pow(x, y) for integer y, 0 < |y| < 2^20, x > 0 finite (Go math/pow.go):
// Frexp, repeated squaring over the bits of |y| with renormalisation to
// [0.5, 1), one reciprocal for y < 0, Ldexp.
double go_pow_int(double x, long y) {
    if (y == 0 || x == 1) return 1;
    if (y == 1) return x;
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

// The lowerable MetaballFalloffFuncs (model3d/metaball.go:17-103).
struct Falloff {
    int kind = MC_FALLOFF_POWER;
    double param = 4, d2 = 0;
    double operator()(double r) const {
        if (kind == MC_FALLOFF_POWER) {  // InversePowerMetaballFalloffFunc
            if (r <= 0) return HUGE_VAL;
            return go_pow_int(r, -(long)param);
        }
        if (r < 0) return HUGE_VAL;  // WyvillMetaballFalloffFunc
        if (r >= param) return 0;
        double ratio2 = (r * r) / d2;
        double value = 1 - ratio2;
        return value * value;
    }
};

// One metaball: a primitive (MetaballField = -SDF) inside TransformMetaball /
// VecScaleMetaball wrappers, flattened to forward steps innermost first
// (model3d/transform.go:319-414).
struct Ball {
    double w = 0;
    std::vector<XStep> fwd, inv;
    std::unique_ptr<Solid> prim;
    V3 Min() const {
        V3 a = prim->Min(), b = prim->Max();
        for (auto& s : fwd) s.apply_bounds(&a, &b);  // ApplyBounds of each wrapper
        return a;
    }
    V3 Max() const {
        V3 a = prim->Min(), b = prim->Max();
        for (auto& s : fwd) s.apply_bounds(&a, &b);
        return b;
    }
    double field(V3 c) const {
        for (auto& s : inv) c = s.apply(c);  // the wrappers' inverse applies, outermost first
        return -prim->SDF(c);
    }
    // MetaballDistBound: the outermost wrapper's inverse ApplyDistance first
    // (transform.go:56, :87, :186, :339-341, :399-401).
    double dist_bound(double d) const {
        for (int i = (int)fwd.size() - 1; i >= 0; i--) {
            const XStep& s = fwd[i];
            if (s.kind == MC_XF_SCALE) {
                d = d * (1 / s.s);
            } else if (s.kind == MC_XF_VECSCALE) {
                V3 a = xyz(std::fabs(s.v.x), std::fabs(s.v.y), std::fabs(s.v.z));
                double mx = a.x > a.y ? (a.x > a.z ? a.x : a.z) : (a.y > a.z ? a.y : a.z);  // MaxCoord
                d = d * (1 / mx);
            }
        }
        return d;
    }
};

// WeightedMetaballSolid (model3d/metaball.go:165-242): the bounds by the
// outset search, then CheckedFuncSolid of the weighted falloff sum.
struct MetaballS : Solid {
    Falloff f;
    double threshold = 0;
    std::vector<Ball> balls;
    V3 mn, mx;
    void init(double radius_threshold) {
        threshold = f(radius_threshold);
        bool any = false;
        for (auto& b : balls) {
            if (!(b.w > 0)) continue;
            if (!any) {
                mn = b.Min();
                mx = b.Max();
                any = true;
            } else {
                mn = vmin(mn, b.Min());
                mx = vmax(mx, b.Max());
            }
        }
        if (!any) throw std::runtime_error("metaball without positive weights");
        auto value_for_outset = [&](double x) {
            double sum = 0;
            for (auto& b : balls)
                if (b.w > 0) sum += b.w * f(b.dist_bound(x));
            return sum;
        };
        double max_outset = dist(mx, mn);
        double min_outset = max_outset * 1e-8;
        for (int i = 0; i < 32; i++) {
            if (value_for_outset(max_outset) > threshold)
                max_outset *= 2.0;
            else
                break;
        }
        if (value_for_outset(max_outset) > threshold) throw std::runtime_error("could not find maximum outset");
        for (int i = 0; i < 32; i++) {
            double mid = (min_outset + max_outset) / 2;
            if (value_for_outset(mid) > threshold)
                min_outset = mid;
            else
                max_outset = mid;
        }
        mn = add_scalar(mn, -max_outset);
        mx = add_scalar(mx, max_outset);
    }
    V3 Min() const override { return mn; }
    V3 Max() const override { return mx; }
    bool Contains(V3 c) const override {
        tl_leaf++;
        if (!in_bounds(mn, mx, c)) return false;
        double sum = 0;
        for (auto& b : balls) sum += b.w * f(b.field(c));
        return sum > threshold;
    }
};

// --------------------------------------------------------------- colliders

struct Tri {
    V3 p[3];
};
inline V3 tri_min(const Tri& t) { return vmin(vmin(t.p[0], t.p[1]), t.p[2]); }  // primitives.go:36-38
inline V3 tri_max(const Tri& t) { return vmax(vmax(t.p[0], t.p[1]), t.p[2]); }  // primitives.go:41-43

const V3 kRayDir = {0.5224892708603626, 0.10494477243214506, 0.43558938446126527};  // collisions.go:124

// Triangle.RayCollisions via rayCollision (model3d/primitives.go:194-249).
int tri_ray_count(const Tri& t, V3 origin) {
    tl_tris++;
    V3 n = normalize(cross(sub(t.p[1], t.p[0]), sub(t.p[2], t.p[0])));  // Normal(), :27-33
    double d = dot(n, normalize(kRayDir));
    if (d < 1e-8 && d > -1e-8) return 0;
    V3 v1 = sub(t.p[1], t.p[0]);
    V3 v2 = sub(t.p[2], t.p[0]);
    V3 cross1 = cross(kRayDir, v2);
    double det = dot(cross1, v1);
    if (det == 0) return 0;
    double invDet = 1 / det;
    V3 o = sub(origin, t.p[0]);
    double bary1 = invDet * dot(o, cross1);
    if (bary1 < 0 || bary1 > 1) return 0;
    V3 cross2 = cross(o, v1);
    double bary2 = invDet * dot(kRayDir, cross2);
    if (bary2 < 0 || bary1 + bary2 > 1) return 0;
    double sc = invDet * dot(v2, cross2);
    return sc < 0 ? 0 : 1;
}

// rayCollisionWithBounds (model3d/bvh.go:322-351) + rayCollidesWithBounds
// (model3d/collisions.go:305-308).
bool ray_hits_box(V3 origin, V3 mn, V3 mx) {
    tl_nodes++;
    double minFrac = -std::numeric_limits<double>::infinity();
    double maxFrac = std::numeric_limits<double>::infinity();
    for (int axis = 0; axis < 3; axis++) {
        double o = at(origin, axis), rate = at(kRayDir, axis);
        if (rate == 0) {
            if (o < at(mn, axis) || o > at(mx, axis)) return false;
            continue;
        }
        double t1 = (at(mn, axis) - o) / rate;
        double t2 = (at(mx, axis) - o) / rate;
        if (t1 > t2) std::swap(t1, t2);
        if (t2 < 0) return false;  // (0, -1): maxFrac < minFrac
        if (t1 > minFrac) minFrac = t1;
        if (t2 < maxFrac) maxFrac = t2;
    }
    return maxFrac >= minFrac && maxFrac >= 0;
}

// A collider tree node: a triangle leaf or a JoinedCollider.
struct CNode {
    bool leaf = false;
    int tri = -1;
    V3 mn, mx;
    std::vector<int> ch;  // indices into nodes
};

struct Collider {
    std::vector<Tri> tris;
    std::vector<CNode> nodes;
    int root = -1;  // -1: nullCollider
    V3 Min() const { return root < 0 ? V3() : nodes[root].mn; }  // collisions.go:360-366
    V3 Max() const { return root < 0 ? V3() : nodes[root].mx; }
    int count(int id, V3 o) const {
        const CNode& n = nodes[id];
        if (n.leaf) return tri_ray_count(tris[n.tri], o);
        if (!ray_hits_box(o, n.mn, n.mx)) return 0;  // JoinedCollider.RayCollisions, :263-273
        int c = 0;
        for (int k : n.ch) c += count(k, o);
        return c;
    }
    int ray_count(V3 o) const { return root < 0 ? 0 : count(root, o); }
};

// flaggedBounder (model3d/bvh.go:294-300).
struct FB {
    int idx;
    V3 mn, mx, md;
    bool flag;
};

double bounds_area(V3 mn, V3 mx) {  // bvh.go:289-292
    V3 d = sub(mx, mn);
    return 2 * (d.x * (d.y + d.z) + d.y * d.z);
}

double multiple_bounds_area(FB* const* bs, size_t n) {  // bvh.go:257-287
    V3 mn = bs[0]->mn, mx = bs[0]->mx;
    for (size_t i = 1; i < n; i++) {
        const FB* b = bs[i];
        if (b->mn.x < mn.x) mn.x = b->mn.x;
        if (b->mn.y < mn.y) mn.y = b->mn.y;
        if (b->mn.z < mn.z) mn.z = b->mn.z;
        if (b->mx.x > mx.x) mx.x = b->mx.x;
        if (b->mx.y > mx.y) mx.y = b->mx.y;
        if (b->mx.z > mx.z) mx.z = b->mx.z;
    }
    return bounds_area(mn, mx);
}

using Sorted = std::vector<FB*>[3];

void group_bounders(std::vector<FB*> s[3], int* out) {  // bvh.go:135-156
    size_t n = s[0].size();
    if (n == 2) {
        out[0] = s[0][0]->idx;
        out[1] = s[0][1]->idx;
        return;
    } else if (n == 1) {
        out[0] = s[0][0]->idx;
        return;
    } else if (n == 0) {
        return;
    }
    size_t midIdx = n / 2;
    // bestSplitAxis (bvh.go:199-217)
    int axis = 0;
    double minArea = multiple_bounds_area(s[0].data(), midIdx) +
                     multiple_bounds_area(s[0].data() + midIdx, n - midIdx);
    for (int i = 1; i < 3; i++) {
        double a = multiple_bounds_area(s[i].data(), midIdx) +
                   multiple_bounds_area(s[i].data() + midIdx, n - midIdx);
        if (a < minArea) {
            minArea = a;
            axis = i;
        }
    }
    // splitBounders (bvh.go:158-197)
    for (size_t i = 0; i < n; i++) s[axis][i]->flag = i < midIdx;
    std::vector<FB*> lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        if (a == axis) {
            lo[a].assign(s[a].begin(), s[a].begin() + midIdx);
            hi[a].assign(s[a].begin() + midIdx, s[a].end());
            continue;
        }
        lo[a].reserve(midIdx);
        hi[a].reserve(n - midIdx);
        for (FB* b : s[a]) (b->flag ? lo[a] : hi[a]).push_back(b);
    }
    for (int a = 0; a < 3; a++) std::vector<FB*>().swap(s[a]);
    group_bounders(lo, out);
    group_bounders(hi, out + midIdx);
}

// GroupTriangles (model3d/bvh.go:118-133) -> permutation of triangle indices.
std::vector<int> group_triangles(const std::vector<Tri>& tris) {
    std::vector<FB> flagged(tris.size());
    for (size_t i = 0; i < tris.size(); i++) {
        V3 mn = tri_min(tris[i]), mx = tri_max(tris[i]);
        flagged[i] = {(int)i, mn, mx, mid(mn, mx), false};
    }
    std::vector<FB*> s[3];
    for (int a = 0; a < 3; a++) {
        s[a].resize(flagged.size());
        for (size_t i = 0; i < flagged.size(); i++) s[a][i] = &flagged[i];
        std::stable_sort(s[a].begin(), s[a].end(),
                         [a](const FB* p, const FB* q) { return at(p->md, a) < at(q->md, a); });
    }
    std::vector<int> out(tris.size());
    if (!tris.empty()) group_bounders(s, out.data());
    return out;
}

// GroupedTrianglesToCollider (collisions.go:169-181) with NewJoinedCollider
// flattening (collisions.go:217-253).  Returns node index or -1 (null).
int build_grouped(Collider& c, const int* order, size_t n) {
    if (n == 0) return -1;
    if (n == 1) {
        CNode leaf;
        leaf.leaf = true;
        leaf.tri = order[0];
        leaf.mn = tri_min(c.tris[order[0]]);
        leaf.mx = tri_max(c.tris[order[0]]);
        c.nodes.push_back(leaf);
        return (int)c.nodes.size() - 1;
    }
    size_t midIdx = n / 2;
    int c1 = build_grouped(c, order, midIdx);
    int c2 = build_grouped(c, order + midIdx, n - midIdx);
    CNode j;
    j.mn = c.nodes[c1].mn;
    j.mx = c.nodes[c1].mx;
    j.mn = vmin(j.mn, c.nodes[c2].mn);
    j.mx = vmax(j.mx, c.nodes[c2].mx);
    for (int k : {c1, c2}) {
        const CNode& ck = c.nodes[k];
        if (!ck.leaf && veq(ck.mn, j.mn) && veq(ck.mx, j.mx)) {
            j.ch.insert(j.ch.end(), ck.ch.begin(), ck.ch.end());
        } else {
            j.ch.push_back(k);
        }
    }
    c.nodes.push_back(j);
    return (int)c.nodes.size() - 1;
}

// ColliderSolid with inset = radius = 0 (model3d/solid.go:247-305).
struct ColliderSolidS : Solid {
    std::shared_ptr<Collider> col;
    V3 mn, mx;
    V3 Min() const override { return mn; }
    V3 Max() const override { return mx; }
    bool Contains(V3 c) const override {
        tl_leaf++;
        if (!in_bounds(mn, mx, c)) return false;
        return col->ray_count(c) % 2 == 1;  // ColliderContains, collisions.go:119-134
    }
};

// ---------------------------------------------------------- scene parsing

struct Parser {
    const mc_node* nodes;
    size_t n;
    const mc_tri_set* sets;
    size_t n_sets;
    size_t pos = 0;
    std::vector<std::shared_ptr<Collider>> colliders;

    V3 pv(const mc_node& nd, int off) { return xyz(nd.p[off], nd.p[off + 1], nd.p[off + 2]); }

    std::vector<XStep> parse_steps(int n_steps) {
        std::vector<XStep> out;
        for (int i = 0; i < n_steps; i++) {
            if (pos >= n) throw std::runtime_error("truncated transform");
            const mc_node& st = nodes[pos++];
            XStep x;
            x.kind = st.kind;
            if (st.kind == MC_XF_TRANSLATE || st.kind == MC_XF_VECSCALE) {
                x.v = pv(st, 0);
            } else if (st.kind == MC_XF_SCALE) {
                x.s = st.p[0];
            } else if (st.kind == MC_XF_MATRIX) {
                for (int k = 0; k < 9; k++) x.m.m[k] = st.p[k];
            } else {
                throw std::runtime_error("bad transform step");
            }
            out.push_back(x);
        }
        return out;
    }

    std::unique_ptr<Solid> parse() {
        if (pos >= n) throw std::runtime_error("truncated node array");
        const mc_node& nd = nodes[pos++];
        switch (nd.kind) {
            case MC_NODE_SPHERE: {
                auto s = std::make_unique<Sphere>();
                s->center = pv(nd, 0);
                s->radius = nd.p[3];
                return s;
            }
            case MC_NODE_RECT: {
                auto s = std::make_unique<RectS>();
                s->mn = pv(nd, 0);
                s->mx = pv(nd, 3);
                return s;
            }
            case MC_NODE_CYLINDER: {
                auto s = std::make_unique<Cylinder>();
                s->p1 = pv(nd, 0);
                s->p2 = pv(nd, 3);
                s->radius = nd.p[6];
                return s;
            }
            case MC_NODE_CAPSULE: {
                auto s = std::make_unique<Capsule>();
                s->p1 = pv(nd, 0);
                s->p2 = pv(nd, 3);
                s->radius = nd.p[6];
                return s;
            }
            case MC_NODE_TORUS: {
                auto s = std::make_unique<Torus>();
                s->center = pv(nd, 0);
                s->axis = pv(nd, 3);
                s->outer = nd.p[6];
                s->inner = nd.p[7];
                return s;
            }
            case MC_NODE_COLLIDER: {
                if (nd.mesh < 0 || (size_t)nd.mesh >= n_sets) throw std::runtime_error("bad mesh index");
                if ((size_t)nd.mesh >= colliders.size()) colliders.resize(nd.mesh + 1);
                if (!colliders[nd.mesh]) {
                    auto c = std::make_shared<Collider>();
                    const mc_tri_set& ts = sets[nd.mesh];
                    c->tris.resize(ts.n);
                    for (int64_t i = 0; i < ts.n; i++)
                        for (int k = 0; k < 3; k++)
                            c->tris[i].p[k] = xyz(ts.tris[i * 9 + k * 3], ts.tris[i * 9 + k * 3 + 1],
                                                  ts.tris[i * 9 + k * 3 + 2]);
                    std::vector<int> order;
                    if (ts.grouped) {
                        order.resize(ts.n);
                        for (int64_t i = 0; i < ts.n; i++) order[i] = (int)i;
                    } else {
                        order = group_triangles(c->tris);
                    }
                    c->root = build_grouped(*c, order.data(), order.size());
                    colliders[nd.mesh] = c;
                }
                auto s = std::make_unique<ColliderSolidS>();
                s->col = colliders[nd.mesh];
                s->mn = s->col->Min();
                s->mx = s->col->Max();
                return s;
            }
            case MC_NODE_JOIN:
            case MC_NODE_INTERSECT: {
                if (nd.n_children < 1) throw std::runtime_error("empty join/intersect");
                std::vector<std::unique_ptr<Solid>> ch;
                for (int i = 0; i < nd.n_children; i++) ch.push_back(parse());
                if (nd.kind == MC_NODE_JOIN) {
                    auto s = std::make_unique<Joined>();
                    s->ch = std::move(ch);
                    return s;
                }
                auto s = std::make_unique<Intersected>();
                s->ch = std::move(ch);
                return s;
            }
            case MC_NODE_SUBTRACT: {
                if (nd.n_children != 2) throw std::runtime_error("subtract needs 2 children");
                auto s = std::make_unique<Subtracted>();
                s->pos = parse();
                s->neg = parse();
                return s;
            }
            case MC_NODE_TRANSFORM: {
                if (nd.n_children != 1) throw std::runtime_error("transform needs 1 child");
                auto s = std::make_unique<Transformed>();
                s->fwd = parse_steps(nd.n_steps);
                s->child = parse();
                s->init();
                return s;
            }
            case MC_NODE_METABALL: {
                if (nd.n_children < 0) throw std::runtime_error("negative ball count");
                auto s = std::make_unique<MetaballS>();
                s->f.kind = (int)nd.p[1];
                s->f.param = nd.p[2];
                if (s->f.kind == MC_FALLOFF_WYVILL) {
                    if (!(nd.p[2] > 0)) throw std::runtime_error("Wyvill d must be positive");
                    s->f.d2 = nd.p[2] * nd.p[2];
                } else if (s->f.kind != MC_FALLOFF_POWER || !(nd.p[2] >= 1 && nd.p[2] < (1 << 20)) ||
                           nd.p[2] != std::floor(nd.p[2])) {
                    throw std::runtime_error("falloff not lowerable");
                }
                bool any_pos = false;
                for (int i = 0; i < nd.n_children; i++) {
                    if (pos >= n || nodes[pos].kind != MC_NODE_BALL) throw std::runtime_error("metaball child is not a ball");
                    const mc_node& bn = nodes[pos++];
                    Ball b;
                    b.w = bn.p[0];
                    any_pos = any_pos || b.w > 0;
                    b.fwd = parse_steps(bn.n_steps);
                    for (int k = (int)b.fwd.size() - 1; k >= 0; k--) b.inv.push_back(b.fwd[k].inverse());
                    if (pos >= n || nodes[pos].kind < MC_NODE_SPHERE || nodes[pos].kind > MC_NODE_TORUS)
                        throw std::runtime_error("ball primitive must be a sphere, rect, cylinder, capsule or torus");
                    b.prim = parse();
                    s->balls.push_back(std::move(b));
                }
                if (!any_pos) {  // NewRect(Origin, Origin), metaball.go:186-188
                    auto r = std::make_unique<RectS>();
                    return r;
                }
                s->init(nd.p[0]);
                return s;
            }
            case MC_NODE_CHECKED: {
                if (nd.n_children != 1) throw std::runtime_error("checked needs 1 child");
                auto s = std::make_unique<Checked>();
                s->mn = xyz(nd.min[0], nd.min[1], nd.min[2]);
                s->mx = xyz(nd.max[0], nd.max[1], nd.max[2]);
                s->child = parse();
                return s;
            }
            default: throw std::runtime_error("unknown node kind");
        }
    }
};

// --------------------------------------------------- marching cubes tables

typedef uint8_t Rot[8];

// allMcRotations (model3d/mc.go:312-353).
std::vector<std::vector<uint8_t>> all_rotations() {
    const uint8_t zr[8] = {2, 0, 3, 1, 6, 4, 7, 5};
    const uint8_t xr[8] = {2, 3, 6, 7, 0, 1, 4, 5};
    std::vector<std::vector<uint8_t>> queue = {{0, 1, 2, 3, 4, 5, 6, 7}};
    std::map<std::vector<uint8_t>, bool> res;
    res[queue[0]] = true;
    size_t head = 0;
    while (head < queue.size()) {
        std::vector<uint8_t> next = queue[head++];
        for (const uint8_t* op : {zr, xr}) {
            std::vector<uint8_t> r(8);
            for (int i = 0; i < 8; i++) r[i] = op[next[i]];  // Compose
            if (!res.count(r)) {
                res[r] = true;
                queue.push_back(r);
            }
        }
    }
    std::vector<std::vector<uint8_t>> out;
    for (auto& kv : res) out.push_back(kv.first);  // std::map order == lexicographic sort
    return out;
}

// The 23 base cases of baseTriangleTable (model3d/mc.go:462-586): inside
// corners, then triangles as three corner pairs each.
struct BaseCase {
    std::vector<int> inside;
    std::vector<std::vector<int>> tris;
};
const std::vector<BaseCase>& base_cases() {
    static const std::vector<BaseCase> t = {
        {{}, {}},
        {{0}, {{0, 1, 0, 2, 0, 4}}},
        {{0, 1}, {{0, 4, 1, 5, 0, 2}, {1, 5, 1, 3, 0, 2}}},
        {{0, 5}, {{0, 1, 0, 2, 0, 4}, {5, 7, 1, 5, 4, 5}}},
        {{0, 7}, {{0, 1, 0, 2, 0, 4}, {6, 7, 3, 7, 5, 7}}},
        {{1, 2, 3}, {{0, 1, 1, 5, 0, 2}, {0, 2, 1, 5, 2, 6}, {2, 6, 1, 5, 3, 7}}},
        {{0, 1, 7}, {{0, 4, 1, 5, 0, 2}, {1, 5, 1, 3, 0, 2}, {6, 7, 3, 7, 5, 7}}},
        {{1, 4, 7}, {{4, 6, 4, 5, 0, 4}, {1, 5, 1, 3, 0, 1}, {6, 7, 3, 7, 5, 7}}},
        {{0, 1, 2, 3}, {{0, 4, 1, 5, 3, 7}, {0, 4, 3, 7, 2, 6}}},
        {{0, 2, 3, 6}, {{0, 1, 4, 6, 0, 4}, {0, 1, 6, 7, 4, 6}, {0, 1, 1, 3, 6, 7}, {1, 3, 3, 7, 6, 7}}},
        {{1, 2, 5, 6}, {{0, 2, 2, 3, 6, 7}, {0, 2, 6, 7, 4, 6}, {0, 1, 4, 5, 5, 7}, {5, 7, 1, 3, 0, 1}}},
        {{0, 2, 3, 7}, {{0, 4, 0, 1, 2, 6}, {0, 1, 5, 7, 2, 6}, {2, 6, 5, 7, 6, 7}, {0, 1, 1, 3, 5, 7}}},
        {{1, 2, 3, 4}, {{0, 1, 1, 5, 0, 2}, {0, 2, 1, 5, 2, 6}, {2, 6, 1, 5, 3, 7}, {4, 5, 0, 4, 4, 6}}},
        {{1, 2, 4, 7}, {{0, 1, 1, 5, 1, 3}, {0, 2, 2, 3, 2, 6}, {4, 5, 0, 4, 4, 6}, {5, 7, 6, 7, 3, 7}}},
        {{1, 2, 3, 6}, {{0, 2, 0, 1, 4, 6}, {0, 1, 3, 7, 4, 6}, {0, 1, 1, 5, 3, 7}, {4, 6, 3, 7, 6, 7}}},
        {{0, 2, 3, 5, 6},
         {{0, 1, 4, 6, 0, 4}, {0, 1, 6, 7, 4, 6}, {0, 1, 1, 3, 6, 7}, {1, 3, 3, 7, 6, 7}, {5, 7, 1, 5, 4, 5}}},
        {{2, 3, 4, 5, 6},
         {{5, 7, 1, 5, 0, 4}, {0, 4, 6, 7, 5, 7}, {0, 2, 6, 7, 0, 4}, {0, 2, 3, 7, 6, 7}, {0, 2, 1, 3, 3, 7}}},
        {{0, 4, 5, 6, 7}, {{1, 5, 0, 1, 0, 2}, {0, 2, 2, 6, 1, 5}, {1, 5, 2, 6, 3, 7}}},
        {{1, 2, 3, 4, 5, 6}, {{0, 2, 0, 1, 0, 4}, {3, 7, 6, 7, 5, 7}}},
        {{1, 2, 3, 4, 6, 7}, {{0, 2, 4, 5, 0, 4}, {0, 2, 5, 7, 4, 5}, {0, 2, 1, 5, 5, 7}, {0, 1, 1, 5, 0, 2}}},
        {{2, 3, 4, 5, 6, 7}, {{1, 5, 0, 4, 0, 2}, {1, 3, 1, 5, 0, 2}}},
        {{1, 2, 3, 4, 5, 6, 7}, {{0, 2, 0, 1, 0, 4}}},
        {{0, 1, 2, 3, 4, 5, 6, 7}, {}},
    };
    return t;
}

struct Table {
    uint8_t count[256];
    uint8_t tris[256][5][6];
    int conflicts = 0;  // two base cases mapping to one case (would make Go's map order matter)
    int covered = 0;
};

// mcLookupTable (model3d/mc.go:434-456).
Table build_table() {
    Table t{};
    auto rots = all_rotations();
    bool have[256] = {false};
    int owner[256];
    for (int i = 0; i < 256; i++) owner[i] = -1;
    const auto& bases = base_cases();
    for (size_t b = 0; b < bases.size(); b++) {
        int baseInts = 0;
        for (int c : bases[b].inside) baseInts |= 1 << c;
        for (auto& rot : rots) {
            int ni = 0;
            for (int c = 0; c < 8; c++)
                if (baseInts & (1 << c)) ni |= 1 << rot[c];
            if (have[ni]) {
                if (owner[ni] != (int)b) t.conflicts++;
                continue;
            }
            have[ni] = true;
            owner[ni] = (int)b;
            t.count[ni] = (uint8_t)bases[b].tris.size();
            for (size_t k = 0; k < bases[b].tris.size(); k++)
                for (int j = 0; j < 6; j++) t.tris[ni][k][j] = rot[bases[b].tris[k][j]];
        }
    }
    for (int i = 0; i < 256; i++) t.covered += have[i];
    return t;
}

// ------------------------------------------------------------------ spacer

// One axis of newSquareSpacer (model3d/mc.go:594-608).
int spacer_axis(double lo, double hi, double delta, std::vector<double>* out, int64_t limit) {
    out->clear();
    if (!(delta > 0)) return MC_ERR_GRID;
    for (double x = lo - delta; x <= hi + delta; x += delta) {
        if ((int64_t)out->size() >= limit) return MC_ERR_GRID;
        if (!out->empty() && out->back() == x) return MC_ERR_GRID;
        out->push_back(x);
    }
    return MC_OK;
}

// ------------------------------------------------------------- thread pool

template <class F>
void parallel_for(int64_t n, int threads, F f) {
    if (threads <= 1 || n <= 1) {
        for (int64_t i = 0; i < n; i++) f(i, 0);
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; t++)
        ts.emplace_back([&, t] {
            for (;;) {
                int64_t i = next.fetch_add(1);
                if (i >= n) break;
                f(i, t);
            }
        });
    for (auto& th : ts) th.join();
}

struct Scene {
    std::unique_ptr<Solid> root;
    std::vector<std::shared_ptr<Collider>> colliders;
};

int parse_scene(const mc_node* nodes, size_t n, const mc_tri_set* sets, size_t n_sets, Scene* out,
                std::string* err) {
    try {
        Parser p{nodes, n, sets, n_sets};
        out->root = p.parse();
        if (p.pos != n) throw std::runtime_error("trailing nodes");
        out->colliders = p.colliders;
    } catch (const std::exception& e) {
        *err = e.what();
        return MC_ERR_BAD_PROGRAM;
    }
    return MC_OK;
}

struct Stats {
    int64_t nx = 0, ny = 0, nz = 0, contains = 0, leaf = 0, nodes = 0, tris = 0;
};

struct KeyHash {
    size_t operator()(const V3& v) const {
        uint64_t a, b, c;
        double x = v.x == 0 ? 0.0 : v.x, y = v.y == 0 ? 0.0 : v.y, z = v.z == 0 ? 0.0 : v.z;
        std::memcpy(&a, &x, 8);
        std::memcpy(&b, &y, 8);
        std::memcpy(&c, &z, 8);
        uint64_t h = a * 0x9e3779b185ebca87ULL ^ b * 0xc2b2ae3d27d4eb4fULL ^ c * 0x165667b19e3779f9ULL;
        h ^= h >> 33;
        h *= 0xff51afd7ed558ccdULL;
        h ^= h >> 33;
        return (size_t)h;
    }
};
struct KeyEq {
    bool operator()(const V3& a, const V3& b) const { return veq(a, b); }
};

// Counters of one oracle call: per-thread counts flushed into atomics.
struct Acc {
    std::atomic<int64_t> leaf{0}, ndc{0}, trc{0}, calls{0};
    void flush() {
        leaf += tl_leaf;
        ndc += tl_nodes;
        trc += tl_tris;
        tl_leaf = tl_nodes = tl_tris = 0;
    }
};


}  // namespace

// ======================================================================
// C ABI of the oracle (used only by tests/, smoke() and bench.py).

extern "C" {

typedef struct oracle_mesh {
    double* tris;      // n_triangles x 9, in generation order
    double* interior;  // n_triangles x 9 when requested: each corner's interior point (mc.go:191-198)
    int64_t n_triangles;
    int64_t n_vertices;  // unique vertices (exact-coordinate dedup, model3d/mesh.go:822-849)
    int64_t nx, ny, nz;
    int64_t contains_calls;
    int64_t leaf_evals;
    int64_t bvh_nodes;
    int64_t bvh_tris;
    char error[256];
} oracle_mesh;

void oracle_mesh_free(oracle_mesh* m) {
    if (!m) return;
    std::free(m->tris);
    std::free(m->interior);
    m->tris = nullptr;
    m->interior = nullptr;
}

// GroupTriangles (model3d/bvh.go:118-217) of a triangle soup (T x 9
// float64, in the given order): out[i] = the index of the triangle that
// SaveGroupedSTL (model3d/mesh.go:724-742) writes i-th.  Ties in the three
// midpoint sorts keep the input order (the deviation noted at the top).
void oracle_group_triangles(const double* tris, int64_t T, int32_t* out) {
    std::vector<Tri> t((size_t)T);
    for (int64_t i = 0; i < T; i++) {
        const double* p = tris + 9 * i;
        t[(size_t)i].p[0] = xyz(p[0], p[1], p[2]);
        t[(size_t)i].p[1] = xyz(p[3], p[4], p[5]);
        t[(size_t)i].p[2] = xyz(p[6], p[7], p[8]);
    }
    std::vector<int> o = group_triangles(t);
    for (int64_t i = 0; i < T; i++) out[i] = o[(size_t)i];
}

// EncodeSTL (model3d/export.go:20-66, fileformats/stl.go:27-58) of a
// triangle soup (T x 9 float64, in the given order): 80 zero bytes, uint32
// LE count, then per triangle float32(Normal()), float32 vertices, 2 zero
// bytes.  Normal = crossProduct().Normalize() (primitives.go:27-33).
void oracle_encode_stl(const double* tris, int64_t T, uint8_t* out) {
    std::memset(out, 0, 84);
    const uint32_t n = (uint32_t)T;
    std::memcpy(out + 80, &n, 4);
    for (int64_t t = 0; t < T; t++) {
        const double* p = tris + 9 * t;
        V3 a = xyz(p[0], p[1], p[2]), b = xyz(p[3], p[4], p[5]), c = xyz(p[6], p[7], p[8]);
        V3 e1 = sub(b, a), e2 = sub(c, a);
        V3 cr = xyz(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
        double norm = std::sqrt(cr.x * cr.x + cr.y * cr.y + cr.z * cr.z);
        V3 nrm = scale(cr, 1 / norm);
        float rec[12] = {(float)nrm.x, (float)nrm.y, (float)nrm.z};
        for (int k = 0; k < 9; k++) rec[3 + k] = (float)p[k];
        uint8_t* o = out + 84 + 50 * t;
        std::memcpy(o, rec, 48);
        o[48] = o[49] = 0;
    }
}

// Transform.Apply of JoinedTransform(steps) -- or of its Inverse()
// (transform.go:213-219: inverses in reverse order) -- at every point,
// in place (the mapping of Mesh.Transform, mesh.go:615-645).
int oracle_apply_transform(const mc_node* steps, size_t n, int inverse, double* pts, int64_t n_pts) {
    std::vector<XStep> xs;
    for (size_t i = 0; i < n; i++) {
        const mc_node& st = steps[i];
        XStep x;
        x.kind = st.kind;
        if (st.kind == MC_XF_TRANSLATE || st.kind == MC_XF_VECSCALE) {
            x.v = xyz(st.p[0], st.p[1], st.p[2]);
        } else if (st.kind == MC_XF_SCALE) {
            x.s = st.p[0];
        } else if (st.kind == MC_XF_MATRIX) {
            for (int k = 0; k < 9; k++) x.m.m[k] = st.p[k];
        } else {
            return MC_ERR_BAD_PROGRAM;
        }
        xs.push_back(x);
    }
    if (inverse) {
        std::vector<XStep> inv;
        for (int i = (int)xs.size() - 1; i >= 0; i--) inv.push_back(xs[i].inverse());
        xs.swap(inv);
    }
    for (int64_t i = 0; i < n_pts; i++) {
        V3 c = xyz(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        for (auto& x : xs) c = x.apply(c);
        pts[3 * i] = c.x;
        pts[3 * i + 1] = c.y;
        pts[3 * i + 2] = c.z;
    }
    return MC_OK;
}

int oracle_case_table(uint8_t counts[256], uint8_t tris[256][5][6], int* conflicts, int* covered) {
    Table t = build_table();
    std::memcpy(counts, t.count, 256);
    std::memcpy(tris, t.tris, sizeof(t.tris));
    if (conflicts) *conflicts = t.conflicts;
    if (covered) *covered = t.covered;
    return 0;
}

int oracle_rotations(uint8_t out[24][8]) {
    auto r = all_rotations();
    for (size_t i = 0; i < r.size() && i < 24; i++)
        for (int k = 0; k < 8; k++) out[i][k] = r[i][k];
    return (int)r.size();
}

int oracle_spacer_axis(double lo, double hi, double delta, double* out, int64_t cap, int64_t* n) {
    std::vector<double> v;
    int st = spacer_axis(lo, hi, delta, &v, (int64_t)1 << 40);
    *n = (int64_t)v.size();
    for (int64_t i = 0; i < (int64_t)v.size() && i < cap; i++) out[i] = v[i];
    return st;
}

int oracle_bounds(const mc_node* nodes, size_t n, const mc_tri_set* sets, size_t n_sets, double mn[3],
                  double mx[3]) {
    Scene sc;
    std::string err;
    int st = parse_scene(nodes, n, sets, n_sets, &sc, &err);
    if (st) return st;
    V3 a = sc.root->Min(), b = sc.root->Max();
    mn[0] = a.x; mn[1] = a.y; mn[2] = a.z;
    mx[0] = b.x; mx[1] = b.y; mx[2] = b.z;
    return 0;
}

// Solid.Contains for n points.  counts (optional): leaf evals, bvh nodes, bvh tris.
int oracle_contains(const mc_node* nodes, size_t n, const mc_tri_set* sets, size_t n_sets,
                    const double* pts, int64_t npts, int threads, uint8_t* out, int64_t counts[3]) {
    Scene sc;
    std::string err;
    int st = parse_scene(nodes, n, sets, n_sets, &sc, &err);
    if (st) return st;
    std::atomic<int64_t> leaf{0}, nd{0}, tr{0};
    int64_t chunk = 4096;
    parallel_for((npts + chunk - 1) / chunk, threads, [&](int64_t c, int) {
        tl_leaf = tl_nodes = tl_tris = 0;
        for (int64_t i = c * chunk; i < std::min(npts, (c + 1) * chunk); i++)
            out[i] = sc.root->Contains(xyz(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2])) ? 1 : 0;
        leaf += tl_leaf;
        nd += tl_nodes;
        tr += tl_tris;
    });
    if (counts) {
        counts[0] = leaf;
        counts[1] = nd;
        counts[2] = tr;
    }
    return 0;
}

// MarchingCubesSearch (model3d/mc.go:45-49).  z_begin/z_end restrict the
// cube loop to slabs z in [z_begin, z_end) (z_end < 0: all) — used to time a
// bounded sample of a large grid; the default covers the whole grid exactly
// as the reference does.
// VertexSlice dedup (mesh.go:770-778), mcSearch (mc.go:182-258) and the
// output arrays of a triangle soup of midpoint vertices; shared by
// MarchingCubesSearch and MarchingCubesSearchFilter.
static int finish_search(const Solid& s, const std::vector<double>& Xs, const std::vector<double>& Ys,
                  const std::vector<double>& Zs, std::vector<double>& soup, int iters, int threads, int want_interior,
                  Acc& acc, oracle_mesh* out) {
    const int64_t NX = Xs.size();
    int64_t T = soup.size() / 9;
    // Unique vertices (VertexSlice, mesh.go:770-778).
    std::unordered_map<V3, int64_t, KeyHash, KeyEq> vid;
    std::vector<V3> verts;
    std::vector<int64_t> tri_v(T * 3);
    vid.reserve(T * 2 + 16);
    for (int64_t i = 0; i < T * 3; i++) {
        V3 p = xyz(soup[3 * i], soup[3 * i + 1], soup[3 * i + 2]);
        auto it = vid.find(p);
        if (it == vid.end()) {
            it = vid.emplace(p, (int64_t)verts.size()).first;
            verts.push_back(p);
        }
        tri_v[i] = it->second;
    }
    out->n_vertices = verts.size();

    // mcSearch (mc.go:182-221); MarchingCubesInterior runs it for iters == 0 too.
    std::vector<V3> inner;
    if (iters != 0 || want_interior) {
        V3 origin = xyz(Xs[0], Ys[0], Zs[0]);
        if (NX < 2 && !verts.empty()) return MC_ERR_EDGE_INDEX;  // Xs[1] out of range
        double dl = NX >= 2 ? Xs[1] - Xs[0] : 0;
        const std::vector<double>* vals[3] = {&Xs, &Ys, &Zs};
        std::vector<V3> outv(verts.size());
        if (want_interior) inner.resize(verts.size());
        std::atomic<int> err2{0};
        int64_t chunk = 1024;
        parallel_for(((int64_t)verts.size() + chunk - 1) / chunk, threads, [&](int64_t c, int) {
            for (int64_t i = c * chunk; i < std::min<int64_t>(verts.size(), (c + 1) * chunk); i++) {
                V3 cc = verts[i];
                // LookupEdgePoint (mc.go:647-660)
                int axis = -1;
                double lo = 0, hi = 0;
                for (int a = 0; a < 3; a++) {
                    double modulus = std::fabs(std::fmod(at(cc, a) - at(origin, a), dl));
                    if (modulus > dl / 4 && modulus < 3 * dl / 4) {
                        int64_t idx = (int64_t)((at(cc, a) - at(origin, a)) / dl);
                        if (idx < 0 || idx + 1 >= (int64_t)vals[a]->size()) {
                            err2 = MC_ERR_EDGE_INDEX;
                            break;
                        }
                        axis = a;
                        lo = (*vals[a])[idx];
                        hi = (*vals[a])[idx + 1];
                        break;
                    }
                }
                if (axis < 0) {
                    if (!err2) err2 = MC_ERR_NOT_ON_EDGE;
                    continue;
                }
                // mcSearchPoint (mc.go:223-258)
                double falseP = lo, trueP = hi;
                V3 tp = cc;
                set(tp, axis, trueP);
                if (!s.Contains(tp)) std::swap(falseP, trueP);
                V3 arr = cc;
                for (int k = 0; k < iters; k++) {
                    double midP = (falseP + trueP) / 2;
                    set(arr, axis, midP);
                    if (s.Contains(arr))
                        trueP = midP;
                    else
                        falseP = midP;
                }
                set(arr, axis, (falseP + trueP) / 2);
                outv[i] = arr;
                if (want_interior) {  // mc.go:252-255
                    V3 ip = arr;
                    set(ip, axis, trueP);
                    inner[i] = ip;
                }
            }
            acc.calls += 0;
            acc.flush();
        });
        acc.calls += (int64_t)verts.size() * (1 + iters);
        if (err2) {
            std::snprintf(out->error, sizeof(out->error),
                          err2 == MC_ERR_NOT_ON_EDGE ? "vertex not on edge" : "index out of range");
            return err2;
        }
        for (int64_t i = 0; i < T * 3; i++) {
            V3 p = outv[tri_v[i]];
            soup[3 * i] = p.x;
            soup[3 * i + 1] = p.y;
            soup[3 * i + 2] = p.z;
        }
    }
    out->n_triangles = T;
    out->tris = (double*)std::malloc(std::max<size_t>(1, soup.size()) * sizeof(double));
    if (!soup.empty()) std::memcpy(out->tris, soup.data(), soup.size() * sizeof(double));
    if (want_interior) {
        out->interior = (double*)std::malloc(std::max<size_t>(1, soup.size()) * sizeof(double));
        for (int64_t i = 0; i < T * 3; i++) {
            const V3 p = inner[tri_v[i]];
            out->interior[3 * i] = p.x;
            out->interior[3 * i + 1] = p.y;
            out->interior[3 * i + 2] = p.z;
        }
    }
    out->contains_calls = acc.calls;
    out->leaf_evals = acc.leaf;
    out->bvh_nodes = acc.ndc;
    out->bvh_tris = acc.trc;
    return MC_OK;
}

int oracle_mc_search(const mc_node* nodes, size_t n, const mc_tri_set* sets, size_t n_sets,
                     double delta, int iters, int threads, int64_t z_begin, int64_t z_end, int want_interior,
                     oracle_mesh* out) {
    std::memset(out, 0, sizeof(*out));
    Scene sc;
    std::string err;
    int st = parse_scene(nodes, n, sets, n_sets, &sc, &err);
    if (st) {
        std::snprintf(out->error, sizeof(out->error), "%s", err.c_str());
        return st;
    }
    const Solid& s = *sc.root;
    // validateBounds (bounder.go:29-52) on the caller's Min()/Max() of the
    // root, as the reference calls s.Min()/s.Max() on the caller's object.
    V3 mn = xyz(nodes[0].min[0], nodes[0].min[1], nodes[0].min[2]);
    V3 mx = xyz(nodes[0].max[0], nodes[0].max[1], nodes[0].max[2]);
    if (std::isnan(vsum(mn)) || std::isnan(vsum(mx)) || std::isinf(vsum(mn)) || std::isinf(vsum(mx)) ||
        mx.x < mn.x || mx.y < mn.y || mx.z < mn.z) {
        std::snprintf(out->error, sizeof(out->error), "invalid bounds");
        return MC_ERR_INVALID_BOUNDS;
    }
    Table table = build_table();
    std::vector<double> Xs, Ys, Zs;
    const int64_t lim = 1 << 20;
    if (spacer_axis(mn.x, mx.x, delta, &Xs, lim) || spacer_axis(mn.y, mx.y, delta, &Ys, lim) ||
        spacer_axis(mn.z, mx.z, delta, &Zs, lim))
        return MC_ERR_GRID;
    const int64_t NX = Xs.size(), NY = Ys.size(), NZ = Zs.size();
    out->nx = NX;
    out->ny = NY;
    out->nz = NZ;
    if (z_end < 0 || z_end > NZ) z_end = NZ;
    if (z_begin < 0) z_begin = 0;
    int64_t zlo = std::max<int64_t>(0, z_begin), zhi = z_end;  // slabs to classify

    Acc acc;
    auto flush = [&] { acc.flush(); };
    std::atomic<int64_t>& calls = acc.calls;

    // Scan + FetchZ (mc.go:614-692): classify every corner of each slab.
    int64_t nslab = zhi - zlo;
    std::vector<uint8_t> grid((size_t)std::max<int64_t>(nslab, 0) * NX * NY);
    std::atomic<int> bad{0};
    parallel_for(nslab, threads, [&](int64_t zi, int) {
        int64_t z = zlo + zi;
        bool onEdge = z == 0 || z == NZ - 1;
        uint8_t* v = &grid[(size_t)zi * NX * NY];
        for (int64_t i = 0; i < NY; i++)
            for (int64_t j = 0; j < NX; j++) {
                bool b = s.Contains(xyz(Xs[j], Ys[i], Zs[z]));
                v[i * NX + j] = b;
                if (b && (onEdge || i == 0 || j == 0 || i == NY - 1 || j == NX - 1)) bad = 1;
            }
        calls += NX * NY;
        flush();
    });
    if (bad) {
        std::snprintf(out->error, sizeof(out->error), "solid is true outside of bounds");
        return MC_ERR_BOUNDS_INSIDE;
    }

    // Cube loop of MarchingCubes (mc.go:20-35).
    auto square = [&](int64_t zi, int64_t x, int64_t y) {  // GetSquare, mc.go:698-710
        int r = 0, mask = 1;
        const uint8_t* v = &grid[(size_t)zi * NX * NY];
        for (int64_t y1 = y; y1 < y + 2; y1++)
            for (int64_t x1 = x; x1 < x + 2; x1++) {
                if (v[y1 * NX + x1]) r |= mask;
                mask <<= 1;
            }
        return r;
    };
    std::vector<std::vector<double>> parts((size_t)std::max<int64_t>(nslab, 0));
    parallel_for(nslab > 0 ? nslab - 1 : 0, threads, [&](int64_t zi, int) {
        int64_t z = zlo + zi + 1;  // nextZ: bottom = z-1, top = z
        std::vector<double>& part = parts[zi];
        for (int64_t y = 0; y < NY - 1; y++)
            for (int64_t x = 0; x < NX - 1; x++) {
                int bits = square(zi, x, y) | (square(zi + 1, x, y) << 4);
                int cnt = table.count[bits];
                if (!cnt) continue;
                V3 a = xyz(Xs[x], Ys[y], Zs[z - 1]);
                V3 b = xyz(Xs[x + 1], Ys[y + 1], Zs[z]);
                V3 corners[8] = {a,
                                 xyz(b.x, a.y, a.z),
                                 xyz(a.x, b.y, a.z),
                                 xyz(b.x, b.y, a.z),
                                 xyz(a.x, a.y, b.z),
                                 xyz(b.x, a.y, b.z),
                                 xyz(a.x, b.y, b.z),
                                 b};  // mcCornerCoordinates, mc.go:289-301
                for (int t = 0; t < cnt; t++) {
                    const uint8_t* m = table.tris[bits][t];
                    for (int k = 0; k < 3; k++) {  // mcTriangle.Triangle, mc.go:401-407
                        V3 p = mid(corners[m[2 * k]], corners[m[2 * k + 1]]);
                        part.push_back(p.x);
                        part.push_back(p.y);
                        part.push_back(p.z);
                    }
                }
            }
    });
    std::vector<double> soup;
    for (auto& p : parts) soup.insert(soup.end(), p.begin(), p.end());
    return finish_search(s, Xs, Ys, Zs, soup, iters, threads, want_interior, acc, out);
}

// MarchingCubesSearchFilter (mc.go:83-155): the block kd-split with the
// caller's filter f (called with the block's bounds widened by delta * 1e-3,
// as min x, y, z, max x, y, z), each kept leaf block's corners evaluated by
// its own cache (mcBlockCache.Populate, mc.go:847-868, with the border panic
// for the block's corners on the grid's border), its cubes' triangles, then
// mcSearch of their vertices.  Single-threaded over blocks; f is called in
// the reference's depth-first visiting order.
typedef int (*oracle_rect_filter)(const double* rect, void* user);

int oracle_mc_search_filter(const mc_node* nodes, size_t n, const mc_tri_set* sets, size_t n_sets, double delta,
                            int iters, int threads, oracle_rect_filter f, void* user, oracle_mesh* out) {
    std::memset(out, 0, sizeof(*out));
    Scene sc;
    std::string err;
    int st = parse_scene(nodes, n, sets, n_sets, &sc, &err);
    if (st) {
        std::snprintf(out->error, sizeof(out->error), "%s", err.c_str());
        return st;
    }
    const Solid& s = *sc.root;
    V3 mn = xyz(nodes[0].min[0], nodes[0].min[1], nodes[0].min[2]);
    V3 mx = xyz(nodes[0].max[0], nodes[0].max[1], nodes[0].max[2]);
    if (std::isnan(vsum(mn)) || std::isnan(vsum(mx)) || std::isinf(vsum(mn)) || std::isinf(vsum(mx)) ||
        mx.x < mn.x || mx.y < mn.y || mx.z < mn.z) {
        std::snprintf(out->error, sizeof(out->error), "invalid bounds");
        return MC_ERR_INVALID_BOUNDS;
    }
    Table table = build_table();
    std::vector<double> Xs, Ys, Zs;
    const int64_t lim = 1 << 20;
    if (spacer_axis(mn.x, mx.x, delta, &Xs, lim) || spacer_axis(mn.y, mx.y, delta, &Ys, lim) ||
        spacer_axis(mn.z, mx.z, delta, &Zs, lim))
        return MC_ERR_GRID;
    const int64_t NX = Xs.size(), NY = Ys.size(), NZ = Zs.size();
    out->nx = NX;
    out->ny = NY;
    out->nz = NZ;
    Acc acc;
    std::vector<double> soup;
    if (NX < 2 || NY < 2 || NZ < 2) return finish_search(s, Xs, Ys, Zs, soup, iters, threads, 0, acc, out);

    struct Block {
        int64_t lo[3], hi[3];
    };
    const std::vector<double>* vals[3] = {&Xs, &Ys, &Zs};
    const double eps = delta * 1e-3;
    auto keep = [&](const Block& b) {  // blockFilter + mcBlock.Bounds (mc.go:96-102, :748-752)
        double r[6];
        for (int a = 0; a < 3; a++) {
            r[a] = (*vals[a])[b.lo[a]] + -eps;
            r[3 + a] = (*vals[a])[b.hi[a]] + eps;
        }
        return f(r, user) != 0;
    };
    auto volume = [](const Block& b) { return (b.hi[0] - b.lo[0]) * (b.hi[1] - b.lo[1]) * (b.hi[2] - b.lo[2]); };
    // mcBlock.Pieces (mc.go:791-801) with mcBlock.Split (mc.go:803-826).
    std::function<void(const Block&, int64_t, std::vector<Block>*)> pieces = [&](const Block& b, int64_t minv,
                                                                                 std::vector<Block>* outb) {
        if (!keep(b)) return;
        if (volume(b) / 2 < minv) {
            outb->push_back(b);
            return;
        }
        const int64_t lx = b.hi[0] - b.lo[0], ly = b.hi[1] - b.lo[1], lz = b.hi[2] - b.lo[2];
        int axis = 0;
        if (ly >= lx && ly >= lz) axis = 1;
        else if (lz >= lx && lz >= ly) axis = 2;
        Block b1 = b, b2 = b;
        b1.hi[axis] = (b.hi[axis] + b.lo[axis]) / 2;
        b2.lo[axis] = b1.hi[axis];
        pieces(b1, minv, outb);
        pieces(b2, minv, outb);
    };
    Block root{{0, 0, 0}, {NX - 1, NY - 1, NZ - 1}};
    std::vector<Block> queued, leaves;
    pieces(root, std::max<int64_t>(volume(root) / 4096, 64), &queued);
    for (const Block& b : queued) pieces(b, 64, &leaves);

    for (const Block& b : leaves) {
        // mcBlockCache.Populate (mc.go:847-868)
        const int64_t sx = b.hi[0] - b.lo[0] + 1, sy = b.hi[1] - b.lo[1] + 1, sz = b.hi[2] - b.lo[2] + 1;
        std::vector<uint8_t> v((size_t)sx * sy * sz);
        for (int64_t z = b.lo[2]; z <= b.hi[2]; z++)
            for (int64_t y = b.lo[1]; y <= b.hi[1]; y++)
                for (int64_t x = b.lo[0]; x <= b.hi[0]; x++) {
                    const bool in = s.Contains(xyz(Xs[x], Ys[y], Zs[z]));
                    const bool edge = z == 0 || z == NZ - 1 || y == 0 || y == NY - 1 || x == 0 || x == NX - 1;
                    if (in && edge) {
                        std::snprintf(out->error, sizeof(out->error), "solid is true outside of bounds");
                        return MC_ERR_BOUNDS_INSIDE;
                    }
                    v[(size_t)((z - b.lo[2]) * sy + (y - b.lo[1])) * sx + (x - b.lo[0])] = in;
                }
        acc.calls += sx * sy * sz;
        acc.flush();
        auto square = [&](int64_t x, int64_t y, int64_t z) {  // mcBlockCache.getSquare (mc.go:878-892)
            int r = 0, mask = 1;
            for (int64_t y1 = y; y1 < y + 2; y1++)
                for (int64_t x1 = x; x1 < x + 2; x1++) {
                    if (v[(size_t)((z - b.lo[2]) * sy + (y1 - b.lo[1])) * sx + (x1 - b.lo[0])]) r |= mask;
                    mask <<= 1;
                }
            return r;
        };
        for (int64_t z = b.lo[2]; z < b.hi[2]; z++)
            for (int64_t y = b.lo[1]; y < b.hi[1]; y++)
                for (int64_t x = b.lo[0]; x < b.hi[0]; x++) {
                    const int bits = square(x, y, z) | (square(x, y, z + 1) << 4);
                    const int cnt = table.count[bits];
                    if (!cnt) continue;
                    V3 a = xyz(Xs[x], Ys[y], Zs[z]);
                    V3 c = xyz(Xs[x + 1], Ys[y + 1], Zs[z + 1]);
                    V3 corners[8] = {a,
                                     xyz(c.x, a.y, a.z),
                                     xyz(a.x, c.y, a.z),
                                     xyz(c.x, c.y, a.z),
                                     xyz(a.x, a.y, c.z),
                                     xyz(c.x, a.y, c.z),
                                     xyz(a.x, c.y, c.z),
                                     c};  // mcCornerCoordinates, mc.go:289-301
                    for (int t = 0; t < cnt; t++) {
                        const uint8_t* m = table.tris[bits][t];
                        for (int k = 0; k < 3; k++) {
                            V3 p = mid(corners[m[2 * k]], corners[m[2 * k + 1]]);
                            soup.push_back(p.x);
                            soup.push_back(p.y);
                            soup.push_back(p.z);
                        }
                    }
                }
    }
    return finish_search(s, Xs, Ys, Zs, soup, iters, threads, 0, acc, out);
}

}  // extern "C"
