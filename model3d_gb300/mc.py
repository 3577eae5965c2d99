"""MarchingCubesSearch on the GPU behind model3d's API.

    mesh = MarchingCubesSearch(solid, delta, iters)

mirrors model3d.MarchingCubesSearch (model3d/mc.go:45-49): the same grid
(newSquareSpacer on the solid's bounds), the same lookup-table triangle
order and the same bisection search, with the reference's panics raised as
``MCError`` carrying the same message.  The mesh is returned indexed
(vertices + triangles); ``Mesh.TriangleSoup()`` gives the reference's
per-triangle coordinates.
"""
from __future__ import annotations

import ctypes
import sys
import threading
from typing import Optional

import numpy as np

from . import _native as N
from .solids import Solid, serialize


class MCError(RuntimeError):
    """A failed call.  ``str(err)`` is the reference's panic text where the
    reference panics (e.g. "solid is true outside of bounds")."""

    def __init__(self, status: int, detail: str = ""):
        self.status = status
        msg = N.status_string(status)
        super().__init__(msg if not detail or detail == msg else f"{msg}: {detail}")


def _check(status: int, ctx_ptr=None):
    if status != N.MC_OK:
        detail = N.lib().mc_last_error(ctx_ptr).decode() if ctx_ptr else ""
        raise MCError(status, detail)


class Context:
    """One CUDA stream and its buffers on one device (mc_ctx)."""

    def __init__(self, device: int = 0):
        L = N.lib()
        p = ctypes.c_void_p()
        _check(L.mc_create(ctypes.byref(p), int(device)))
        self._p = p
        self.device = device

    @property
    def ptr(self):
        return self._p

    def close(self):
        if getattr(self, "_p", None) and self._p.value:
            N.lib().mc_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        # At interpreter shutdown the finalisation order of contexts, solids
        # and meshes is arbitrary; the process is ending, so release nothing.
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def default_context(device: int = 0) -> Context:
    ctxs = getattr(_tls, "ctxs", None)
    if ctxs is None:
        ctxs = _tls.ctxs = {}
    if device not in ctxs:
        ctxs[device] = Context(device)
    return ctxs[device]


def _tri_sets(sets):
    """The mc_tri_set array of serialize()'s triangle sets, and the arrays it
    points into (keep them alive for the call)."""
    arr = (N.MCTriSet * max(1, len(sets)))()
    keep = []
    for i, s in enumerate(sets):
        t = np.ascontiguousarray(s.tris, dtype=np.float64)
        keep.append(t)
        arr[i].tris = t.ctypes.data
        arr[i].n = len(t)
        arr[i].grouped = int(s.grouped)
    return arr, keep


def check_program(solid: Solid) -> dict:
    """Lower `solid` on the host as DeviceSolid would (mc_program_check), with
    no GPU, and describe the program; raises MCError when it cannot be lowered."""
    nodes, sets = serialize(solid)
    arr, keep = _tri_sets(sets)
    info = N.MCProgramInfo()
    err = ctypes.create_string_buffer(256)
    st = N.lib().mc_program_check(nodes.ctypes.data, len(nodes), ctypes.addressof(arr), len(sets),
                                  ctypes.byref(info), err, len(err))
    if st != N.MC_OK:
        raise MCError(st, err.value.decode())
    out = {n: getattr(info, n) for n, _ in N.MCProgramInfo._fields_[:7]}
    out["threshold"] = info.threshold
    out["root_min"], out["root_max"] = list(info.root_min), list(info.root_max)
    out["digest"] = "%016x" % info.digest
    return out


class DeviceSolid:
    """A Solid lowered to the device (mc_solid): CSG bytecode and collider
    trees resident in HBM.  Reuse it across calls to avoid re-lowering."""

    def __init__(self, solid: Solid, ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        nodes, sets = serialize(solid)
        self.nodes = nodes
        self._sets = sets
        arr, keep = _tri_sets(sets)
        p = ctypes.c_void_p()
        _check(N.lib().mc_solid_create(self.ctx.ptr, nodes.ctypes.data, len(nodes),
                                       ctypes.addressof(arr), len(sets), ctypes.byref(p)),
               self.ctx.ptr)
        self._p = p

    @property
    def ptr(self):
        return self._p

    def bounds(self):
        mn, mx = np.zeros(3), np.zeros(3)
        _check(N.lib().mc_solid_bounds(self._p, mn.ctypes.data, mx.ctypes.data))
        return mn, mx

    def close(self):
        if getattr(self, "_p", None) and self._p.value:
            N.lib().mc_solid_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        # At interpreter shutdown the finalisation order of contexts, solids
        # and meshes is arbitrary; the process is ending, so release nothing.
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class Mesh:
    """Indexed triangle mesh: vertices (V,3) float64, triangles (T,3) int32
    (vertex order of the reference's lookup table)."""

    def __init__(self, vertices: np.ndarray, triangles: np.ndarray, stats: Optional[dict] = None):
        self.vertices = vertices
        self.triangles = triangles
        self.stats = stats or {}

    def NumTriangles(self) -> int:
        return len(self.triangles)

    def TriangleSoup(self) -> np.ndarray:
        """(T, 9) float64: each triangle's three vertices."""
        if len(self.triangles) == 0:
            return np.zeros((0, 9))
        return self.vertices[self.triangles].reshape(-1, 9)

    def Volume(self) -> float:
        """Mesh.Volume (model3d/measurements.go:18-31) up to summation order."""
        t = self.TriangleSoup().reshape(-1, 3, 3)
        return float(abs(np.linalg.det(t).sum() / 6.0)) if len(t) else 0.0

    def _arrays(self):
        v = np.ascontiguousarray(self.vertices, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(self.triangles, dtype=np.int32).reshape(-1, 3)
        return v, t

    def _grouped_stl(self, ctx: Optional["Context"]) -> np.ndarray:
        ctx = ctx or default_context()
        v, t = self._arrays()
        L = N.lib()
        n = ctypes.c_size_t()
        _check(L.mc_mesh_stl_grouped(ctx.ptr, v.ctypes.data, len(v), t.ctypes.data, len(t), None, 0,
                                     ctypes.byref(n)), ctx.ptr)
        buf = np.empty(n.value, dtype=np.uint8)
        _check(L.mc_mesh_stl_grouped(ctx.ptr, v.ctypes.data, len(v), t.ctypes.data, len(t), buf.ctypes.data,
                                     n.value, ctypes.byref(n)), ctx.ptr)
        return buf

    def EncodeGroupedSTL(self, ctx: Optional["Context"] = None) -> bytes:
        """The bytes SaveGroupedSTL writes (model3d/mesh.go:724-742): the
        triangles in GroupTriangles order (ties in the midpoint sorts keep
        this mesh's triangle order), binary STL records (export.go:28-60).
        Grouped and encoded on the device."""
        return self._grouped_stl(ctx).tobytes()

    def SaveGroupedSTL(self, path: str, ctx: Optional["Context"] = None) -> None:
        """Mesh.SaveGroupedSTL (model3d/mesh.go:724-742).  The encoded
        records are written from the array they were copied into, without
        a copy into a bytes object."""
        data = self._grouped_stl(ctx)
        with open(path, "wb") as f:
            f.write(memoryview(data))


def GroupTriangles(mesh: Mesh, *, ctx: Optional["Context"] = None) -> np.ndarray:
    """GroupTriangles (model3d/bvh.go:118-217) of a mesh's triangles on the
    device: order[i] is the triangle SaveGroupedSTL writes i-th.  Each
    midpoint sort is stable over the mesh's triangle order (the reference's
    sort.Slice over a slice in map order breaks ties arbitrarily)."""
    ctx = ctx or default_context()
    v, t = mesh._arrays()
    order = np.empty(len(t), dtype=np.int32)
    _check(N.lib().mc_mesh_group(ctx.ptr, v.ctypes.data, len(v), t.ctypes.data, len(t), order.ctypes.data), ctx.ptr)
    return order


def _opts(precision="fp32", cull=True, tile_y=0, tile_z=0, z_range=None):
    o = N.MCOpts()
    o.precision = N.MC_PREC_FP64 if precision in ("fp64", N.MC_PREC_FP64) else N.MC_PREC_FP32_FILTERED
    o.cull = 1 if cull else 0
    o.tile_y = int(tile_y)
    o.tile_z = int(tile_z)
    if z_range is not None:
        o.z_begin, o.z_end = int(z_range[0]), int(z_range[1])
    return o


def _as_device_solid(solid, ctx):
    if isinstance(solid, DeviceSolid):
        return solid
    return DeviceSolid(solid, ctx)


class _HostMesh:
    """Owner of the library-allocated host arrays of one mc_mesh; the numpy
    arrays of a Mesh keep it alive and it frees them (mc_mesh_free) last."""

    def __init__(self, m):
        self.m = N.MCMesh()
        ctypes.pointer(self.m)[0] = m

    def arrays(self):
        m = self.m

        def view(ptr, n, ctype, dtype):
            if n == 0:
                return np.zeros((0, 3), dtype)
            buf = (ctype * (3 * n)).from_address(ctypes.cast(ptr, ctypes.c_void_p).value)
            buf._owner = self
            return np.frombuffer(buf, dtype=dtype).reshape(n, 3)

        return (view(m.vertices, m.n_vertices, ctypes.c_double, np.float64),
                view(m.triangles, m.n_triangles, ctypes.c_int32, np.int32))

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            N.lib().mc_mesh_free(ctypes.byref(self.m))
        except Exception:
            pass


def MarchingCubesSearch(solid, delta: float, iters: int, *, precision: str = "fp32",
                        cull: bool = True, ctx: Optional[Context] = None, tile_y: int = 0,
                        tile_z: int = 0, z_range=None) -> Mesh:
    """model3d.MarchingCubesSearch (model3d/mc.go:45-49) on the GPU.  With
    z_range = (z_begin, z_end) only the cube layers [z_begin, z_end) of the
    grid are meshed (a z-slab; see shard.py)."""
    ctx = ctx or (solid.ctx if isinstance(solid, DeviceSolid) else default_context())
    ds = _as_device_solid(solid, ctx)
    o = _opts(precision, cull, tile_y, tile_z, z_range)
    m = N.MCMesh()
    _check(N.lib().mc_search(ctx.ptr, ds.ptr, float(delta), int(iters), ctypes.byref(o),
                             ctypes.byref(m)), ctx.ptr)
    verts, tris = _HostMesh(m).arrays()
    return Mesh(verts, tris, m.stats.as_dict())


def MarchingCubesInterior(solid, delta: float, iters: int, *, precision: str = "fp32",
                          cull: bool = True, ctx: Optional[Context] = None):
    """model3d.MarchingCubesInterior (model3d/mc.go:55-60) on the GPU: the
    mesh and, for each vertex i, a point known to be inside the solid (the
    last inside point of its bisection) as row i of a (V, 3) array -- the
    reference's CoordMap keyed by vertex."""
    ctx = ctx or (solid.ctx if isinstance(solid, DeviceSolid) else default_context())
    ds = _as_device_solid(solid, ctx)
    o = _opts(precision, cull)
    o.interior = 1
    V, T = ctypes.c_int64(), ctypes.c_int64()
    st = N.MCStats()
    L = N.lib()
    _check(L.mc_search_device(ctx.ptr, ds.ptr, float(delta), int(iters), ctypes.byref(o),
                              ctypes.byref(V), ctypes.byref(T), ctypes.byref(st)), ctx.ptr)
    verts = np.empty((V.value, 3))
    tris = np.empty((T.value, 3), dtype=np.int32)
    inner = np.empty((V.value, 3))
    _check(L.mc_result_copy(ctx.ptr, verts.ctypes.data, tris.ctypes.data), ctx.ptr)
    _check(L.mc_result_interior_copy(ctx.ptr, inner.ctypes.data), ctx.ptr)
    return Mesh(verts, tris, st.as_dict()), inner


def MarchingCubesConj(solid, delta: float, iters: int, *xforms, precision: str = "fp32",
                      cull: bool = True, ctx: Optional[Context] = None) -> Mesh:
    """model3d.MarchingCubesConj (model3d/mc.go:66-71) on the GPU: the search
    on TransformSolid(JoinedTransform(xforms), solid), then the inverse
    transform applied to the mesh vertices on the device (Mesh.Transform)."""
    from .solids import JoinedTransform, TransformSolid, transform_records
    joined = JoinedTransform(list(xforms))
    ctx = ctx or default_context()
    ds = DeviceSolid(TransformSolid(joined, solid), ctx)
    o = _opts(precision, cull)
    V, T = ctypes.c_int64(), ctypes.c_int64()
    st = N.MCStats()
    L = N.lib()
    _check(L.mc_search_device(ctx.ptr, ds.ptr, float(delta), int(iters), ctypes.byref(o),
                              ctypes.byref(V), ctypes.byref(T), ctypes.byref(st)), ctx.ptr)
    steps = transform_records(joined)
    _check(L.mc_result_transform(ctx.ptr, steps.ctypes.data, len(steps), 1), ctx.ptr)
    verts = np.empty((V.value, 3))
    tris = np.empty((T.value, 3), dtype=np.int32)
    _check(L.mc_result_copy(ctx.ptr, verts.ctypes.data, tris.ctypes.data), ctx.ptr)
    return Mesh(verts, tris, st.as_dict())


def MarchingCubesSearchSTL(solid, delta: float, iters: int, *, precision: str = "fp32",
                           cull: bool = True, ctx: Optional[Context] = None) -> bytes:
    """model3d.MarchingCubesSearch(...).EncodeSTL() (model3d/export.go:20-66)
    with the binary STL encoded on the device: 84 + 50 T bytes (triangles in
    this library's order)."""
    ctx = ctx or (solid.ctx if isinstance(solid, DeviceSolid) else default_context())
    ds = _as_device_solid(solid, ctx)
    o = _opts(precision, cull)
    V, T = ctypes.c_int64(), ctypes.c_int64()
    st = N.MCStats()
    L = N.lib()
    _check(L.mc_search_device(ctx.ptr, ds.ptr, float(delta), int(iters), ctypes.byref(o),
                              ctypes.byref(V), ctypes.byref(T), ctypes.byref(st)), ctx.ptr)
    n = ctypes.c_size_t()
    _check(L.mc_result_stl(ctx.ptr, None, 0, ctypes.byref(n)), ctx.ptr)
    buf = np.empty(n.value, dtype=np.uint8)
    _check(L.mc_result_stl(ctx.ptr, buf.ctypes.data, n.value, ctypes.byref(n)), ctx.ptr)
    return buf.tobytes()


def MarchingCubesSearchGroupedSTL(solid, delta: float, iters: int, *, precision: str = "fp32",
                                  cull: bool = True, ctx: Optional[Context] = None) -> bytes:
    """model3d.MarchingCubesSearch(...) then SaveGroupedSTL's bytes
    (model3d/mesh.go:724-742), the mesh never leaving the device: search,
    GroupTriangles and the STL encoding all run there."""
    ctx = ctx or (solid.ctx if isinstance(solid, DeviceSolid) else default_context())
    ds = _as_device_solid(solid, ctx)
    o = _opts(precision, cull)
    V, T = ctypes.c_int64(), ctypes.c_int64()
    st = N.MCStats()
    L = N.lib()
    _check(L.mc_search_device(ctx.ptr, ds.ptr, float(delta), int(iters), ctypes.byref(o),
                              ctypes.byref(V), ctypes.byref(T), ctypes.byref(st)), ctx.ptr)
    n = ctypes.c_size_t()
    _check(L.mc_result_stl_grouped(ctx.ptr, None, 0, ctypes.byref(n)), ctx.ptr)
    buf = np.empty(n.value, dtype=np.uint8)
    _check(L.mc_result_stl_grouped(ctx.ptr, buf.ctypes.data, n.value, ctypes.byref(n)), ctx.ptr)
    return buf.tobytes()


def MarchingCubesSearchBatch(jobs, *, precision: str = "fp32", cull: bool = True,
                             ctx: Optional[Context] = None, tile_y: int = 0, tile_z: int = 0):
    """Many MarchingCubesSearch calls in one batched launch (mc_search_batch).

    jobs: sequence of (solid or DeviceSolid, delta, iters).  Returns a list
    with a Mesh per job, or the MCError of a job that failed.  Repeating the
    same batch replays a captured CUDA graph."""
    ctx = ctx or default_context()
    dss = [_as_device_solid(s, ctx) for s, _, _ in jobs]
    arr = (N.MCJob * max(1, len(jobs)))()
    for i, (ds, (_, d, it)) in enumerate(zip(dss, jobs)):
        arr[i].solid = ds.ptr.value
        arr[i].delta = float(d)
        arr[i].iters = int(it)
    outs = (N.MCMesh * max(1, len(jobs)))()
    status = (ctypes.c_int * max(1, len(jobs)))()
    o = _opts(precision, cull, tile_y, tile_z)
    st = N.lib().mc_search_batch(ctx.ptr, arr, len(jobs), ctypes.byref(o), outs, status)
    res = []
    for i in range(len(jobs)):
        if status[i] != N.MC_OK:
            res.append(MCError(status[i]))
            continue
        verts, tris = _HostMesh(outs[i]).arrays()
        res.append(Mesh(verts, tris, outs[i].stats.as_dict()))
    if st != N.MC_OK and all(not isinstance(r, MCError) for r in res):
        raise MCError(st, N.lib().mc_last_error(ctx.ptr).decode())
    return res


def autotune(solid, delta: float, iters: int = 8, *, precision: str = "fp32",
             ctx: Optional[Context] = None):
    """Time the classification tile shapes on this solid and grid; the
    fastest becomes the context's default.  Returns (tile_y, tile_z, ms)."""
    ctx = ctx or (solid.ctx if isinstance(solid, DeviceSolid) else default_context())
    ds = _as_device_solid(solid, ctx)
    o = _opts(precision)
    best = N.MCOpts()
    ms = ctypes.c_double()
    _check(N.lib().mc_autotune(ctx.ptr, ds.ptr, float(delta), int(iters), ctypes.byref(o),
                               ctypes.byref(best), ctypes.byref(ms)), ctx.ptr)
    return best.tile_y, best.tile_z, ms.value


def measure_peaks(ctx: Optional[Context] = None):
    """(fp32 TFLOP/s, fp64 TFLOP/s, L2 read GB/s) of this GPU (micro-kernels)."""
    ctx = ctx or default_context()
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _check(N.lib().mc_measure_peaks(ctx.ptr, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), ctx.ptr)
    return a.value, b.value, c.value


def MarchingCubes(solid, delta: float, **kw) -> Mesh:
    """model3d.MarchingCubes (model3d/mc.go:14-37): the search with iters=0."""
    return MarchingCubesSearch(solid, delta, 0, **kw)


def Contains(solid, points, *, precision: str = "fp32", ctx: Optional[Context] = None) -> np.ndarray:
    """Solid.Contains at each of the (n, 3) points, evaluated on the GPU."""
    ctx = ctx or (solid.ctx if isinstance(solid, DeviceSolid) else default_context())
    ds = _as_device_solid(solid, ctx)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(len(pts), dtype=np.uint8)
    o = _opts(precision)
    _check(N.lib().mc_contains(ctx.ptr, ds.ptr, pts.ctypes.data, len(pts), ctypes.byref(o),
                               out.ctypes.data), ctx.ptr)
    return out.astype(bool)


def case_table():
    """The library's 256-case lookup table (counts, tris[256][5][6])."""
    counts = np.zeros(256, dtype=np.uint8)
    tris = np.zeros((256, 5, 6), dtype=np.uint8)
    _check(N.lib().mc_case_table(counts.ctypes.data, tris.ctypes.data))
    return counts, tris


def spacer_axis(lo: float, hi: float, delta: float) -> np.ndarray:
    n = ctypes.c_int64()
    N.lib().mc_spacer_axis(lo, hi, delta, None, 0, ctypes.byref(n))
    out = np.zeros(n.value)
    _check(N.lib().mc_spacer_axis(lo, hi, delta, out.ctypes.data, n.value, ctypes.byref(n)))
    return out


def canonical(soup: np.ndarray) -> np.ndarray:
    """Triangles as 9 float64 bit patterns each, rows sorted: two meshes are
    bit-identical iff their canonical arrays are equal (vertex order inside a
    triangle is kept, only the triangle list is sorted)."""
    bits = np.ascontiguousarray(soup, dtype=np.float64).reshape(-1, 9).view(np.uint64)
    if len(bits) == 0:
        return bits
    order = np.lexsort(bits.T[::-1])
    return bits[order]
