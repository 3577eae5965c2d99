"""Solid types mirroring model3d's lowerable solids, and their serialisation.

Each class keeps the reference's field names and computes Min()/Max() with
the reference's float64 formulas, so the spacer built from the root bounds is
the reference's.  ``serialize(solid)`` turns a tree into the prefix-order
``mc_node`` records of include/mcgpu.h plus the triangle sets of its
colliders; the GPU library lowers those records to its device program.

Anything that is not one of these types cannot be lowered and raises
``NotLowerable`` — there is no CPU fallback.
"""
from __future__ import annotations

import math
import struct
from typing import List, Sequence

import numpy as np

from .geometry import Coord3D, Matrix3, XYZ, go_max, go_min, NewMatrix3Rotation

# Node kinds (include/mcgpu.h).
SPHERE, RECT, CYLINDER, CAPSULE, TORUS, COLLIDER, METABALL, BALL = 1, 2, 3, 4, 5, 6, 7, 8
JOIN, SUBTRACT, INTERSECT, TRANSFORM, CHECKED = 16, 17, 18, 19, 20
XF_TRANSLATE, XF_SCALE, XF_VECSCALE, XF_MATRIX = 32, 33, 34, 35

NODE_DTYPE = np.dtype([
    ("kind", "<i4"), ("n_children", "<i4"), ("n_steps", "<i4"), ("mesh", "<i4"),
    ("min", "<f8", (3,)), ("max", "<f8", (3,)), ("p", "<f8", (12,)),
])
assert NODE_DTYPE.itemsize == 160
_NODE_PACK = struct.Struct("<4i18d")  # the same record, packed
_ZEROS = (0.0,) * 12


class NotLowerable(TypeError):
    """Raised for solids with no device lowering (the reference type exists,
    but this library does not evaluate it on the GPU)."""


def _circle_axis_bound(axis: int, normal: Coord3D, sign: float) -> float:
    """circleAxisBound (model3d/shapes.go:562-571)."""
    arr = [0.0, 0.0, 0.0]
    arr[axis] = sign
    proj = Coord3D(*arr).ProjectOut(normal)
    proj = proj.Scale(1 / (proj.Norm() + 1e-8))
    return sign * (abs(proj.Array()[axis]) + 1e-8)


def _circle_axis_offset(normal: Coord3D, sign: float, scale: float) -> Coord3D:
    """XYZ(circleAxisBound(0..2, normal, sign)).Scale(scale), with the same
    float64 operations as _circle_axis_bound (ProjectOut = c - n (n . c) with
    n = normal.Normalize(), coords.go:379-381, :425-428) on plain floats."""
    x, y, z = normal.X, normal.Y, normal.Z
    inv = 1 / math.sqrt(x * x + y * y + z * z)
    nx, ny, nz = x * inv, y * inv, z * inv
    out = []
    for axis in range(3):
        cx, cy, cz = (sign if axis == 0 else 0.0), (sign if axis == 1 else 0.0), (sign if axis == 2 else 0.0)
        d = nx * cx + ny * cy + nz * cz
        px, py, pz = cx + (nx * d) * -1, cy + (ny * d) * -1, cz + (nz * d) * -1
        f = 1 / (math.sqrt(px * px + py * py + pz * pz) + 1e-8)
        v = (px * f, py * f, pz * f)[axis]
        out.append((sign * (abs(v) + 1e-8)) * scale)
    return Coord3D(out[0], out[1], out[2])


class Solid:
    """A boolean function over space with bounds (model3d/solid.go:16-21)."""

    def Min(self) -> Coord3D:
        raise NotImplementedError

    def Max(self) -> Coord3D:
        raise NotImplementedError

    def _bounds(self):
        """(Min(), Max()) with the same float64 operations; the primitives
        and boolean nodes share work between the two (one tree walk)."""
        return self.Min(), self.Max()

    def _own_bounds(self, cls) -> bool:
        """Whether Min and Max are cls's own (not overridden by a subclass),
        so that cls's _bounds computes what they would."""
        t = type(self)
        return t.Min is cls.Min and t.Max is cls.Max


class Sphere(Solid):
    """model3d/shapes.go:13-31."""

    def __init__(self, Center: Coord3D, Radius: float):
        self.Center, self.Radius = Center, float(Radius)

    def Min(self):
        return self.Center.AddScalar(-self.Radius)

    def Max(self):
        return self.Center.AddScalar(self.Radius)

    def _bounds(self):
        if not self._own_bounds(Sphere):
            return self.Min(), self.Max()
        return self.Center.AddScalar(-self.Radius), self.Center.AddScalar(self.Radius)


class Rect(Solid):
    """model3d/shapes.go:145-173."""

    def __init__(self, MinVal: Coord3D, MaxVal: Coord3D):
        self.MinVal, self.MaxVal = MinVal, MaxVal

    def Min(self):
        return self.MinVal

    def Max(self):
        return self.MaxVal

    def Expand(self, delta: float) -> "Rect":
        """Rect.Expand (model3d/shapes.go:339-344)."""
        return Rect(self.MinVal.AddScalar(-delta), self.MaxVal.AddScalar(delta))


def NewRect(min: Coord3D, max: Coord3D) -> Rect:
    return Rect(min, max)


class Cylinder(Solid):
    """model3d/shapes.go:542-598."""

    def __init__(self, P1: Coord3D, P2: Coord3D, Radius: float):
        self.P1, self.P2, self.Radius = P1, P2, float(Radius)

    def Min(self):
        minCenter = self.P1.Min(self.P2)
        axis = self.P2.Sub(self.P1)
        return minCenter.Add(_circle_axis_offset(axis, -1.0, self.Radius))

    def Max(self):
        maxCenter = self.P1.Max(self.P2)
        axis = self.P2.Sub(self.P1)
        return maxCenter.Add(_circle_axis_offset(axis, 1.0, self.Radius))

    def _bounds(self):
        if not self._own_bounds(Cylinder):
            return self.Min(), self.Max()
        # circleAxisBound is odd in its sign argument, exactly: every
        # operation of _circle_axis_offset commutes with negation.
        off = _circle_axis_offset(self.P2.Sub(self.P1), 1.0, self.Radius)
        return self.P1.Min(self.P2).Add(XYZ(-off.X, -off.Y, -off.Z)), self.P1.Max(self.P2).Add(off)


class Capsule(Solid):
    """model3d/shapes.go:348-368."""

    def __init__(self, P1: Coord3D, P2: Coord3D, Radius: float):
        self.P1, self.P2, self.Radius = P1, P2, float(Radius)

    def Min(self):
        return self.P1.Min(self.P2).AddScalar(-self.Radius)

    def Max(self):
        return self.P1.Max(self.P2).AddScalar(self.Radius)

    def _bounds(self):
        if not self._own_bounds(Capsule):
            return self.Min(), self.Max()
        return self.P1.Min(self.P2).AddScalar(-self.Radius), self.P1.Max(self.P2).AddScalar(self.Radius)


class Torus(Solid):
    """model3d/shapes.go:1323-1365."""

    def __init__(self, Center: Coord3D, Axis: Coord3D, OuterRadius: float, InnerRadius: float):
        self.Center, self.Axis = Center, Axis
        self.OuterRadius, self.InnerRadius = float(OuterRadius), float(InnerRadius)

    def Min(self):
        r = self.InnerRadius
        extra = XYZ(r, r, r)
        off = _circle_axis_offset(self.Axis, -1.0, self.OuterRadius)
        return off.Add(self.Center).Sub(extra)

    def Max(self):
        r = self.InnerRadius
        extra = XYZ(r, r, r)
        off = _circle_axis_offset(self.Axis, 1.0, self.OuterRadius)
        return off.Add(self.Center).Add(extra)


class JoinedSolid(Solid):
    """model3d/solid.go:71-118."""

    def __init__(self, solids: Sequence[Solid]):
        self.solids = list(solids)
        if not self.solids:
            raise ValueError("JoinedSolid needs at least one solid")

    def Min(self):
        m = self.solids[0].Min()
        for s in self.solids[1:]:
            m = m.Min(s.Min())
        return m

    def Max(self):
        m = self.solids[0].Max()
        for s in self.solids[1:]:
            m = m.Max(s.Max())
        return m

    def _bounds(self):
        if not self._own_bounds(JoinedSolid):
            return self.Min(), self.Max()
        lo, hi = self.solids[0]._bounds()
        for s in self.solids[1:]:
            a, b = s._bounds()
            lo, hi = lo.Min(a), hi.Max(b)
        return lo, hi

    def Optimize(self) -> Solid:
        """JoinedSolid.Optimize (model3d/solid.go:100-118)."""
        grouped = GroupBounders(list(self.solids))
        return _grouped_solids_to_solid(grouped)


def _grouped_solids_to_solid(s: List[Solid]) -> Solid:
    if len(s) == 1:
        return CacheSolidBounds(s[0])
    h = len(s) // 2
    return CacheSolidBounds(JoinedSolid([_grouped_solids_to_solid(s[:h]),
                                         _grouped_solids_to_solid(s[h:])]))


class SubtractedSolid(Solid):
    """model3d/solid.go:120-142."""

    def __init__(self, Positive: Solid, Negative: Solid):
        self.Positive, self.Negative = Positive, Negative

    def Min(self):
        return self.Positive.Min()

    def Max(self):
        return self.Positive.Max()

    def _bounds(self):
        if not self._own_bounds(SubtractedSolid):
            return self.Min(), self.Max()
        return self.Positive._bounds()


def Subtract(x: Solid, y: Solid) -> SubtractedSolid:
    return SubtractedSolid(x, y)


class IntersectedSolid(Solid):
    """model3d/solid.go:144-172."""

    def __init__(self, solids: Sequence[Solid]):
        self.solids = list(solids)
        if not self.solids:
            raise ValueError("IntersectedSolid needs at least one solid")

    def Min(self):
        b = self.solids[0].Min()
        for s in self.solids[1:]:
            b = b.Max(s.Min())
        return b

    def Max(self):
        b = self.solids[0].Max()
        for s in self.solids[1:]:
            b = b.Min(s.Max())
        return b.Max(self.Min())

    def _bounds(self):
        if not self._own_bounds(IntersectedSolid):
            return self.Min(), self.Max()
        lo, hi = self.solids[0]._bounds()
        for s in self.solids[1:]:
            a, b = s._bounds()
            lo, hi = lo.Max(a), hi.Min(b)
        return lo, hi.Max(lo)


# ------------------------------------------------------------- transforms

class Transform:
    """model3d/transform.go:5-21."""

    def ApplyBounds(self, min: Coord3D, max: Coord3D):
        raise NotImplementedError

    def _steps(self):
        raise NotImplementedError


class Translate(Transform):
    def __init__(self, Offset: Coord3D):
        self.Offset = Offset

    def ApplyBounds(self, min, max):
        return min.Add(self.Offset), max.Add(self.Offset)

    def _steps(self):
        return [(XF_TRANSLATE, self.Offset.Array())]


class Scale(Transform):
    def __init__(self, Scale: float):
        self.Scale = float(Scale)

    def ApplyBounds(self, min, max):
        if self.Scale < 0:
            return max.Scale(self.Scale), min.Scale(self.Scale)
        return min.Scale(self.Scale), max.Scale(self.Scale)

    def _steps(self):
        return [(XF_SCALE, [self.Scale])]


class VecScale(Transform):
    def __init__(self, Scale: Coord3D):
        self.Scale = Scale

    def ApplyBounds(self, min, max):
        min, max = min.Mul(self.Scale), max.Mul(self.Scale)
        return min.Min(max), max.Max(min)

    def _steps(self):
        return [(XF_VECSCALE, self.Scale.Array())]


class Matrix3Transform(Transform):
    def __init__(self, Matrix: Matrix3):
        self.Matrix = Matrix

    def ApplyBounds(self, min, max):
        newMin = newMax = None
        for i, x in enumerate([min.X, max.X]):
            for j, y in enumerate([min.Y, max.Y]):
                for k, z in enumerate([min.Z, max.Z]):
                    c = self.Matrix.MulColumn(XYZ(x, y, z))
                    if i == 0 and j == 0 and k == 0:
                        newMin, newMax = c, c
                    else:
                        newMin = newMin.Min(c)
                        newMax = newMax.Max(c)
        return newMin, newMax

    def _steps(self):
        return [(XF_MATRIX, list(self.Matrix.m))]


class JoinedTransform(Transform):
    def __init__(self, transforms: Sequence[Transform]):
        self.transforms = list(transforms)

    def ApplyBounds(self, min, max):
        for t in self.transforms:
            min, max = t.ApplyBounds(min, max)
        return min, max

    def _steps(self):
        out = []
        for t in self.transforms:
            out.extend(t._steps())
        return out


class OrthoMatrix3Transform(Matrix3Transform):
    """orthoMatrix3Transform: a distance-preserving Matrix3Transform
    (model3d/transform.go:159-190)."""


def Rotation(axis: Coord3D, theta: float) -> Matrix3Transform:
    """model3d/transform.go:165-172."""
    return OrthoMatrix3Transform(NewMatrix3Rotation(axis, theta))


class _TransformedSolid(Solid):
    """TransformSolid's result (model3d/transform.go:240-247)."""

    def __init__(self, t: Transform, s: Solid):
        self.transform, self.solid = t, s
        self.min, self.max = t.ApplyBounds(s.Min(), s.Max())

    def Min(self):
        return self.min

    def Max(self):
        return self.max


def TransformSolid(t: Transform, s: Solid) -> Solid:
    return _TransformedSolid(t, s)


def TranslateSolid(s: Solid, offset: Coord3D) -> Solid:
    return TransformSolid(Translate(offset), s)


def ScaleSolid(s: Solid, v: float) -> Solid:
    return TransformSolid(Scale(v), s)


def VecScaleSolid(s: Solid, v: Coord3D) -> Solid:
    return TransformSolid(VecScale(v), s)


def RotateSolid(s: Solid, axis: Coord3D, angle: float) -> Solid:
    return TransformSolid(Rotation(axis, angle), s)


class _CheckedSolid(Solid):
    """CheckedFuncSolid(min, max, s.Contains) (model3d/solid.go:46-50)."""

    def __init__(self, s: Solid, min: Coord3D, max: Coord3D):
        self.solid, self.min, self.max = s, min, max

    def Min(self):
        return self.min

    def Max(self):
        return self.max


def ForceSolidBounds(s: Solid, min: Coord3D, max: Coord3D) -> Solid:
    return _CheckedSolid(s, min, max)


def CacheSolidBounds(s: Solid) -> Solid:
    return ForceSolidBounds(s, s.Min(), s.Max())


# -------------------------------------------------------------- colliders

class MeshCollider:
    """A triangle collider made by MeshToCollider / GroupedTrianglesToCollider
    (model3d/collisions.go:138-181).  ``tris`` is (n, 9) float64."""

    def __init__(self, tris: np.ndarray, grouped: bool):
        self.tris = np.ascontiguousarray(np.asarray(tris, dtype=np.float64).reshape(-1, 9))
        self.grouped = bool(grouped)

    def Min(self) -> Coord3D:
        return self._bound(np.min, go_min)

    def Max(self) -> Coord3D:
        return self._bound(np.max, go_max)

    def _bound(self, red, op):
        if len(self.tris) == 0:
            return Coord3D()  # nullCollider (model3d/collisions.go:358-366)
        v = self.tris.reshape(-1, 3)
        out = []
        for a in range(3):
            col = v[:, a]  # a strided view: no copy
            r = float(red(col))  # NaN when any coordinate is NaN (np.min/np.max propagate it)
            if r != r:  # but math.Min lets -Inf win over NaN, math.Max +Inf
                inf = -math.inf if op is go_min else math.inf
                if (col == inf).any():
                    r = inf
            elif r == 0.0:  # -0 wins in Min, +0 in Max, as math.Min/Max order them
                neg = np.signbit(col[col == 0]).any()
                pos = (~np.signbit(col[col == 0])).any()
                r = -0.0 if (op is go_min and neg) or (op is go_max and not pos) else 0.0
            out.append(r)
        return Coord3D(*out)


def MeshToCollider(tris) -> MeshCollider:
    """tris: (n, 9) array of triangles in the mesh's TriangleSlice order."""
    return MeshCollider(tris, grouped=False)


def GroupedTrianglesToCollider(tris) -> MeshCollider:
    return MeshCollider(tris, grouped=True)


class ColliderSolid(Solid):
    """NewColliderSolid (model3d/solid.go:247-253); ray-parity containment."""

    def __init__(self, collider: MeshCollider):
        if not isinstance(collider, MeshCollider):
            raise NotLowerable("only mesh colliders can be lowered")
        self.collider = collider
        self.min, self.max = collider.Min(), collider.Max()

    def Min(self):
        return self.min

    def Max(self):
        return self.max


def NewColliderSolid(c: MeshCollider) -> ColliderSolid:
    return ColliderSolid(c)


# ---------------------------------------------------- GroupBounders (solids)

def GroupBounders(objs: List[Solid]) -> List[Solid]:
    """GroupBounders (model3d/bvh.go:131-217) over solids, ties by input order."""
    fl = []
    for i, b in enumerate(objs):
        mn, mx = b.Min(), b.Max()
        fl.append([i, mn, mx, mn.Mid(mx), False])
    srt = [sorted(fl, key=lambda f, a=a: f[3].Array()[a]) for a in range(3)]
    out = [None] * len(objs)

    def area(bs):
        mn, mx = bs[0][1], bs[0][2]
        mn, mx = Coord3D(mn.X, mn.Y, mn.Z), Coord3D(mx.X, mx.Y, mx.Z)
        for b in bs[1:]:
            if b[1].X < mn.X: mn.X = b[1].X
            if b[1].Y < mn.Y: mn.Y = b[1].Y
            if b[1].Z < mn.Z: mn.Z = b[1].Z
            if b[2].X > mx.X: mx.X = b[2].X
            if b[2].Y > mx.Y: mx.Y = b[2].Y
            if b[2].Z > mx.Z: mx.Z = b[2].Z
        d = mx.Sub(mn)
        return 2 * (d.X * (d.Y + d.Z) + d.Y * d.Z)

    def rec(s, off):
        n = len(s[0])
        if n == 2:
            out[off], out[off + 1] = objs[s[0][0][0]], objs[s[0][1][0]]
            return
        if n == 1:
            out[off] = objs[s[0][0][0]]
            return
        if n == 0:
            return
        mid = n // 2
        axis, best = 0, area(s[0][:mid]) + area(s[0][mid:])
        for a in (1, 2):
            v = area(s[a][:mid]) + area(s[a][mid:])
            if v < best:
                best, axis = v, a
        for i, b in enumerate(s[axis]):
            b[4] = i < mid
        lo = [None] * 3
        hi = [None] * 3
        for a in range(3):
            if a == axis:
                lo[a], hi[a] = s[a][:mid], s[a][mid:]
            else:
                lo[a] = [b for b in s[a] if b[4]]
                hi[a] = [b for b in s[a] if not b[4]]
        rec(lo, off)
        rec(hi, off + mid)

    rec(srt, 0)
    return out


# ------------------------------------------------------------ serialisation

def transform_records(t: Transform) -> np.ndarray:
    """The MC_XF_* records (mc_node array) of a transform's steps in
    JoinedTransform order."""
    steps = t._steps()
    out = np.zeros(len(steps), dtype=NODE_DTYPE)
    for i, (kind, p) in enumerate(steps):
        out[i]["kind"] = kind
        out[i]["p"][:len(p)] = p
    return out


def serialize(solid: Solid):
    """Prefix-order mc_node records and the triangle sets they refer to.

    Min()/Max() are computed for the nodes whose bounds the library reads:
    the root, colliders, transforms and checked solids."""
    from .metaballs import FALLOFF_POWER, MAX_POWER, MetaballSolidT, ball_steps

    recs = []
    sets: List[MeshCollider] = []
    set_ids = {}
    zero3 = (0.0, 0.0, 0.0)

    def node(kind, s=None, n_children=0, n_steps=0, mesh=0, p=()):
        if s is not None and (not recs or kind in (COLLIDER, TRANSFORM, CHECKED, METABALL)):
            lo, hi = s._bounds()
            mn, mx = lo.Array(), hi.Array()
        else:
            mn = mx = zero3
        recs.append(_NODE_PACK.pack(kind, n_children, n_steps, mesh, *mn, *mx, *p, *_ZEROS[len(p):]))

    def emit(s):
        if isinstance(s, Sphere):
            node(SPHERE, s, p=s.Center.Array() + [s.Radius])
        elif isinstance(s, Rect):
            node(RECT, s, p=s.MinVal.Array() + s.MaxVal.Array())
        elif isinstance(s, Cylinder):
            node(CYLINDER, s, p=s.P1.Array() + s.P2.Array() + [s.Radius])
        elif isinstance(s, Capsule):
            node(CAPSULE, s, p=s.P1.Array() + s.P2.Array() + [s.Radius])
        elif isinstance(s, Torus):
            node(TORUS, s, p=s.Center.Array() + s.Axis.Array() + [s.OuterRadius, s.InnerRadius])
        elif isinstance(s, ColliderSolid):
            key = id(s.collider)
            if key not in set_ids:
                set_ids[key] = len(sets)
                sets.append(s.collider)
            node(COLLIDER, s, mesh=set_ids[key])
        elif isinstance(s, JoinedSolid):
            node(JOIN, s, n_children=len(s.solids))
            for c in s.solids:
                fast(c)
        elif isinstance(s, IntersectedSolid):
            node(INTERSECT, s, n_children=len(s.solids))
            for c in s.solids:
                fast(c)
        elif isinstance(s, SubtractedSolid):
            node(SUBTRACT, s, n_children=2)
            fast(s.Positive)
            fast(s.Negative)
        elif isinstance(s, _TransformedSolid):
            steps = s.transform._steps()
            node(TRANSFORM, s, n_children=1, n_steps=len(steps))
            for kind, p in steps:
                node(kind, None, p=p)
            fast(s.solid)
        elif isinstance(s, _CheckedSolid):
            node(CHECKED, s, n_children=1)
            fast(s.solid)
        elif isinstance(s, MetaballSolidT):
            f = s.falloff
            if f.kind == 0 or (f.kind == FALLOFF_POWER and
                               (f.param != int(f.param) or f.param >= MAX_POWER)):
                raise NotLowerable("this falloff has no device lowering")
            node(METABALL, s, n_children=len(s.balls), p=[s.radiusThreshold, f.kind, f.param])
            for mb, w in zip(s.balls, s.weights):
                steps, prim = ball_steps(mb)
                node(BALL, None, n_children=1, n_steps=len(steps), p=[w])
                for kind, p in steps:
                    node(kind, None, p=p)
                fast(prim)
        else:
            raise NotLowerable(f"{type(s).__name__} has no device lowering")

    pack = _NODE_PACK.pack
    z = 0.0

    # Exact-type fast paths for the common nodes (a subclass takes the
    # isinstance chain above): the same records, packed without the
    # intermediate lists.  Bounds are serialised for the root only.
    def fast_sphere(s):
        if not recs:
            return emit(s)
        c = s.Center
        recs.append(pack(SPHERE, 0, 0, 0, z, z, z, z, z, z, c.X, c.Y, c.Z, s.Radius, z, z, z, z, z, z, z, z))

    def fast_rect(s):
        if not recs:
            return emit(s)
        a, b = s.MinVal, s.MaxVal
        recs.append(pack(RECT, 0, 0, 0, z, z, z, z, z, z, a.X, a.Y, a.Z, b.X, b.Y, b.Z, z, z, z, z, z, z))

    def fast_segment(kind):
        def f(s):
            if not recs:
                return emit(s)
            a, b = s.P1, s.P2
            recs.append(pack(kind, 0, 0, 0, z, z, z, z, z, z, a.X, a.Y, a.Z, b.X, b.Y, b.Z, s.Radius,
                             z, z, z, z, z))
        return f

    def fast_join(kind):
        def f(s):
            if not recs:
                return emit_node_children(kind, s)
            recs.append(pack(kind, len(s.solids), 0, 0, z, z, z, z, z, z, *_ZEROS))
            for c in s.solids:
                fast(c)
        return f

    def fast_subtract(s):
        if not recs:
            return emit_node_children(SUBTRACT, s)
        recs.append(pack(SUBTRACT, 2, 0, 0, z, z, z, z, z, z, *_ZEROS))
        fast(s.Positive)
        fast(s.Negative)

    def emit_node_children(kind, s):
        if kind == SUBTRACT:
            node(SUBTRACT, s, n_children=2)
            fast(s.Positive)
            fast(s.Negative)
        else:
            node(kind, s, n_children=len(s.solids))
            for c in s.solids:
                fast(c)

    handlers = {Sphere: fast_sphere, Rect: fast_rect, Cylinder: fast_segment(CYLINDER),
                Capsule: fast_segment(CAPSULE), JoinedSolid: fast_join(JOIN),
                IntersectedSolid: fast_join(INTERSECT), SubtractedSolid: fast_subtract}

    def fast(s):
        h = handlers.get(type(s))
        if h is None:
            emit(s)
        else:
            h(s)

    fast(solid)
    return np.frombuffer(bytearray(b"".join(recs)), dtype=NODE_DTYPE), sets
