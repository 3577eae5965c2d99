"""MarchingCubesFilter, MarchingCubesSearchFilter and MarchingCubesC2F
(model3d/mc.go:73-180) on the GPU, with the reference's block pruning.

The reference splits the grid's cubes into blocks (mcBlock.Pieces, a
kd-split that halves the longest side, mc.go:780-826), asks the filter
f(block bounds widened by delta * 1e-3) for every block it visits, and meshes
only the cubes of the leaf blocks that every visit kept; the search then
bisects only the vertices of those cubes' triangles.  Here the block
recursion runs on the host with the caller's f exactly as the reference
runs it, giving a mask of kept cubes; the device meshes and searches the
whole grid (on a GPU the pruning saves nothing worth a second pass), and the
triangles of cubes outside the mask are dropped, with the vertices no kept
triangle uses.  A triangle's cube comes from its three vertices' edge keys
(mc_result_keys).  Each vertex's search depends only on its own edge, so the
kept vertices are the reference's.

One difference remains, and only for a filter that drops cubes the surface
crosses (which the reference's contract forbids, mc.go:79-82): the border
check ("solid is true outside of bounds", mc.go:687-689) still covers the
whole grid, where the reference checks the corners of kept blocks only.

`RectCollider` is the collider's RectCollision (collisions.go:344-356,
primitives.go:446-500) for MarchingCubesC2F's filter.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _native as N
from .geometry import XYZ
from .mc import (DeviceSolid, MCError, Mesh, MarchingCubesSearch, _check, _opts, default_context, spacer_axis)
from .solids import NewRect


# ------------------------------------------------------------ block pruning

def _split(mn, mx):
    """mcBlock.Split (mc.go:803-826): halve the longest side (ties: y, then z)."""
    lx, ly, lz = mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]
    axis = 0
    if ly >= lx and ly >= lz:
        axis = 1
    elif lz >= lx and lz >= ly:
        axis = 2
    mid = (mx[axis] + mn[axis]) // 2
    mx1, mn2 = list(mx), list(mn)
    mx1[axis] = mid
    mn2[axis] = mid
    return (mn, tuple(mx1)), (tuple(mn2), mx)


def _volume(mn, mx):
    return (mx[0] - mn[0]) * (mx[1] - mn[1]) * (mx[2] - mn[2])


def kept_cubes(f, xs, ys, zs, delta) -> np.ndarray:
    """Cube mask (nz-1, ny-1, nx-1) of MarchingCubesFilter's block pruning
    (mc.go:83-148): blocks visited by Pieces(max(volume / 4096, 64)) and then,
    per queued block, Pieces(64), each visit calling f on the block's bounds
    widened by delta * 1e-3 (mcBlock.Bounds, mc.go:748-752)."""
    nx, ny, nz = len(xs), len(ys), len(zs)
    mask = np.zeros((max(nz - 1, 0), max(ny - 1, 0), max(nx - 1, 0)), dtype=bool)
    if min(nx, ny, nz) < 2:
        return mask
    eps = delta * 1e-3
    vals = (xs, ys, zs)

    def keep(mn, mx):
        lo = XYZ(*(float(vals[a][mn[a]]) for a in range(3))).AddScalar(-eps)
        hi = XYZ(*(float(vals[a][mx[a]]) for a in range(3))).AddScalar(eps)
        return bool(f(NewRect(lo, hi)))

    def pieces(block, min_volume, out):
        stack = [block]
        while stack:
            mn, mx = stack.pop()
            if not keep(mn, mx):
                continue
            if _volume(mn, mx) // 2 < min_volume:
                out.append((mn, mx))
            else:
                b1, b2 = _split(mn, mx)
                stack.append(b2)
                stack.append(b1)

    root = ((0, 0, 0), (nx - 1, ny - 1, nz - 1))
    queued = []
    pieces(root, max(_volume(*root) // 4096, 64), queued)
    for b in queued:
        leaves = []
        pieces(b, 64, leaves)
        for mn, mx in leaves:
            mask[mn[2]:mx[2], mn[1]:mx[1], mn[0]:mx[0]] = True
    return mask


def triangle_cubes(keys: np.ndarray, tris: np.ndarray) -> np.ndarray:
    """(T, 3) cube indices (x, y, z) of triangles from their vertices' edge
    keys: an edge along axis a at (x, y, z) lies on the cubes with that
    coordinate on a and coordinate - 1 or coordinate on the other axes; a
    triangle's three edges share exactly one cube."""
    k = keys[tris]  # (T, 3)
    ax = (k >> np.uint64(60)).astype(np.int64)
    c = np.stack([(k & np.uint64(0xFFFFF)).astype(np.int64), ((k >> np.uint64(20)) & np.uint64(0xFFFFF)).astype(np.int64),
                  ((k >> np.uint64(40)) & np.uint64(0xFFFFF)).astype(np.int64)], axis=-1)  # (T, 3 vertices, 3 axes)
    lower = c - (ax[..., None] != np.arange(3)[None, None]).astype(np.int64)
    cube = lower.max(axis=1)
    if not (cube <= c.min(axis=1)).all():
        raise RuntimeError("a triangle's edges do not share a cube")
    if ((c.min(axis=1) - cube) > 0).any():
        raise RuntimeError("a triangle's edges share more than one cube")
    return cube


def _search_with_keys(solid, delta, iters, precision, cull, ctx):
    ctx = ctx or (solid.ctx if isinstance(solid, DeviceSolid) else default_context())
    ds = solid if isinstance(solid, DeviceSolid) else DeviceSolid(solid, ctx)
    L = N.lib()
    o = _opts(precision, cull)
    V, T = ctypes.c_int64(), ctypes.c_int64()
    st = N.MCStats()
    _check(L.mc_search_device(ctx.ptr, ds.ptr, float(delta), int(iters), ctypes.byref(o), ctypes.byref(V),
                              ctypes.byref(T), ctypes.byref(st)), ctx.ptr)
    verts = np.empty((V.value, 3))
    tris = np.empty((T.value, 3), dtype=np.int32)
    keys = np.empty(V.value, dtype=np.uint64)
    _check(L.mc_result_copy(ctx.ptr, verts.ctypes.data, tris.ctypes.data), ctx.ptr)
    _check(L.mc_result_keys(ctx.ptr, keys.ctypes.data), ctx.ptr)
    mn, mx = ds.bounds()
    return ds, verts, tris, keys, st.as_dict(), mn, mx


def MarchingCubesSearchFilter(solid, f, delta: float, iters: int, *, precision: str = "fp32", cull: bool = True,
                              ctx=None) -> Mesh:
    """model3d.MarchingCubesSearchFilter (mc.go:150-155): MarchingCubesFilter's
    triangles, then the search of their vertices."""
    ds, verts, tris, keys, stats, mn, mx = _search_with_keys(solid, delta, iters, precision, cull, ctx)
    xs, ys, zs = (spacer_axis(mn[a], mx[a], delta) for a in range(3))
    mask = kept_cubes(f, xs, ys, zs, delta)
    if len(tris) == 0:
        return Mesh(verts, tris, stats)
    cube = triangle_cubes(keys, tris)
    keep = mask[cube[:, 2], cube[:, 1], cube[:, 0]]
    t = tris[keep]
    used = np.zeros(len(verts), dtype=bool)
    used[t.ravel()] = True
    remap = np.cumsum(used) - 1
    out = Mesh(np.ascontiguousarray(verts[used]), np.ascontiguousarray(remap[t].astype(np.int32)), stats)
    out.stats = dict(stats, vertices=int(used.sum()), triangles=int(len(t)),
                     cubes_kept=int(mask.sum()), cubes=int(mask.size))
    return out


def MarchingCubesFilter(solid, f, delta: float, **kw) -> Mesh:
    """model3d.MarchingCubesFilter (mc.go:83-148)."""
    return MarchingCubesSearchFilter(solid, f, delta, 0, **kw)


def MarchingCubesC2F(solid, bigDelta: float, smallDelta: float, extraSpace: float, iters: int, **kw) -> Mesh:
    """model3d.MarchingCubesC2F (mc.go:157-180): the coarse mesh at bigDelta,
    its collider, and the fine search filtered by RectCollision of each block
    expanded by extraSpace + 2 bigDelta sqrt(3)."""
    if bigDelta < smallDelta:
        raise MCError(N.MC_ERR_ARG, "bigDelta should be >= smallDelta for efficiency")
    extra = extraSpace + 2 * bigDelta * math.sqrt(3)
    coarse = MarchingCubesSearch(solid, bigDelta, iters, **kw)
    col = RectCollider(coarse.TriangleSoup())
    return MarchingCubesSearchFilter(solid, lambda r: col.RectCollision(r.Expand(extra)), smallDelta, iters, **kw)


# ------------------------------------------------------------ RectCollision

def _lex_less(a, b):
    """p1 < p2 in NewSegment's canonical order (primitives.go:547-554)."""
    return (a[..., 0] < b[..., 0]) | ((a[..., 0] == b[..., 0]) & (a[..., 1] < b[..., 1])) | \
        ((a[..., 0] == b[..., 0]) & (a[..., 1] == b[..., 1]) & (a[..., 2] < b[..., 2]))


def _segment(p1, p2):
    lt = _lex_less(p1, p2)[..., None]
    return np.where(lt, p1, p2), np.where(lt, p2, p1)


def _dot(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def _normalize(a):
    n = np.sqrt(a[..., 0] * a[..., 0] + a[..., 1] * a[..., 1] + a[..., 2] * a[..., 2])
    with np.errstate(all="ignore"):
        return a * (1 / n)[..., None]


def _segments_hit_rect(s0, s1, lo, hi):
    """Segment.RectCollision (primitives.go:632-638) through
    rayCollisionWithBounds (bvh.go:322-351), vectorised over segments."""
    d = s1 - s0
    n = len(s0)
    minf = np.full(n, -np.inf)
    maxf = np.full(n, np.inf)
    dead = np.zeros(n, dtype=bool)
    with np.errstate(all="ignore"):
        for a in range(3):
            o, r = s0[:, a], d[:, a]
            zero = r == 0
            dead |= zero & ((o < lo[a]) | (o > hi[a]))
            t1 = (lo[a] - o) / r
            t2 = (hi[a] - o) / r
            sw = t1 > t2
            t1, t2 = np.where(sw, t2, t1), np.where(sw, t1, t2)
            live = ~zero & ~dead
            dead |= live & (t2 < 0)
            live &= ~dead
            minf = np.where(live & (t1 > minf), t1, minf)
            maxf = np.where(live & (t2 < maxf), t2, maxf)
    return ~dead & (maxf >= minf) & (maxf >= 0) & (minf <= 1)


def _triangles_hit_segment(t, o, e):
    """Triangle.SegmentCollision (primitives.go:439-444): FirstRayCollision
    (rayCollision, primitives.go:207-249) of the ray o + s e, scale in [0, 1],
    for every triangle t (K, 3, 3) and one segment."""
    t0, t1, t2 = t[:, 0], t[:, 1], t[:, 2]
    with np.errstate(all="ignore"):
        nrm = _normalize(_cross(t1 - t0, t2 - t0))
        dn = _dot(nrm, _normalize(e)[None])
        parallel = (dn < 1e-8) & (dn > -1e-8)
        v1, v2 = t1 - t0, t2 - t0
        c1 = _cross(np.broadcast_to(e, v2.shape), v2)
        det = _dot(c1, v1)
        inv = 1 / det
        oo = o[None] - t0
        b1 = inv * _dot(oo, c1)
        c2 = _cross(oo, v1)
        b2 = inv * _dot(np.broadcast_to(e, c2.shape), c2)
        sc = inv * _dot(v2, c2)
        return ~parallel & (det != 0) & ~((b1 < 0) | (b1 > 1)) & ~((b2 < 0) | (b1 + b2 > 1)) & (sc >= 0) & (sc <= 1)


class RectCollider:
    """RectCollision of MeshToCollider(mesh) (collisions.go:138-181,
    :344-356): the tree of GroupTriangles' order split in halves, each joined
    node testing its box before its children.  A triangle is reached iff the
    box of its parent node meets the rect (every ancestor's box contains that
    box), so each query tests the triangles whose parent box meets the rect
    with Triangle.RectCollision (primitives.go:446-500)."""

    def __init__(self, tris):
        t = np.asarray(tris, dtype=np.float64).reshape(-1, 3, 3)
        self.tris = t[_group_order(t)]
        n = len(self.tris)
        tmin, tmax = self.tris.min(axis=1), self.tris.max(axis=1)
        self.pbox = np.zeros((n, 6))
        self.root_only = n == 1

        def build(a, b):  # -> (min, max) of [a, b); sets children's parent boxes
            if b - a == 1:
                return tmin[a], tmax[a]
            mid = a + (b - a) // 2
            l0, l1 = build(a, mid)
            r0, r1 = build(mid, b)
            lo, hi = np.minimum(l0, r0), np.maximum(l1, r1)
            for c0, c1 in ((a, mid), (mid, b)):
                if c1 - c0 == 1:
                    self.pbox[c0] = np.concatenate([lo, hi])
            return lo, hi

        if n >= 2:
            import sys
            sys.setrecursionlimit(max(10000, sys.getrecursionlimit()))
            build(0, n)

    def RectCollision(self, rect) -> bool:
        n = len(self.tris)
        if n == 0:
            return False
        lo = np.array(rect.MinVal.Array())
        hi = np.array(rect.MaxVal.Array())
        if self.root_only:
            cand = self.tris
        else:
            a = np.maximum(lo[None], self.pbox[:, :3])
            b = np.minimum(hi[None], self.pbox[:, 3:])
            cand = self.tris[(a <= b).all(axis=1)]
        if len(cand) == 0:
            return False
        for i in range(3):
            s0, s1 = _segment(cand[:, i], cand[:, (i + 1) % 3])
            if _segments_hit_rect(s0, s1, lo, hi).any():
                return True
        x0, y0, z0 = lo
        x1, y1, z1 = hi
        segs = []
        for x in (x0, x1):
            segs += [((x, y0, z0), (x, y0, z1)), ((x, y0, z0), (x, y1, z0)),
                     ((x, y1, z0), (x, y1, z1)), ((x, y0, z1), (x, y1, z1))]
        segs += [((x0, y0, z0), (x1, y0, z0)), ((x0, y1, z0), (x1, y1, z0)),
                 ((x0, y0, z1), (x1, y0, z1)), ((x0, y1, z1), (x1, y1, z1))]
        for p, q in segs:
            p, q = np.array(p), np.array(q)
            if not _lex_less(p, q):
                p, q = q, p
            if _triangles_hit_segment(cand, p, q - p).any():
                return True
        return False


def _group_order(t: np.ndarray) -> np.ndarray:
    """GroupTriangles (bvh.go:118-217) of (n, 3, 3) triangles as an index
    order: recursive halving along the axis whose two halves' bounding boxes
    have the least total area, ties in the midpoint sorts by input order."""
    n = len(t)
    if n <= 2:
        return np.arange(n)
    tmin, tmax = t.min(axis=1), t.max(axis=1)
    mid = (tmin + tmax) * 0.5
    srt = [np.argsort(mid[:, a], kind="stable") for a in range(3)]
    out = np.empty(n, dtype=np.int64)

    def area(idx):
        lo, hi = tmin[idx].min(axis=0), tmax[idx].max(axis=0)
        s = hi - lo
        return 2 * (s[0] * (s[1] + s[2]) + s[1] * s[2])  # boundsArea, bvh.go:289-292

    stack = [(srt, 0)]
    while stack:
        sb, at = stack.pop()
        m = len(sb[0])
        if m <= 2:
            out[at:at + m] = sb[0]
            continue
        h = m // 2
        best, axis = None, 0
        for a in range(3):
            v = area(sb[a][:h]) + area(sb[a][h:])
            if best is None or v < best:
                best, axis = v, a
        flag = np.zeros(n, dtype=bool)
        flag[sb[axis][:h]] = True
        left = [s[flag[s]] for s in sb]
        right = [s[~flag[s]] for s in sb]
        stack.append((right, at + h))
        stack.append((left, at))
    return out
