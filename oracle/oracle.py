"""ctypes binding of the oracle (liboracle.so) — TEST INFRASTRUCTURE ONLY.

The oracle is the CPU restatement of the reference MarchingCubesSearch path
in oracle/mc_oracle.cpp.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg load it, to check results against; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


class OracleMesh(ctypes.Structure):
    _fields_ = [
        ("tris", ctypes.POINTER(ctypes.c_double)),
        ("interior", ctypes.POINTER(ctypes.c_double)),
        ("n_triangles", ctypes.c_int64),
        ("n_vertices", ctypes.c_int64),
        ("nx", ctypes.c_int64),
        ("ny", ctypes.c_int64),
        ("nz", ctypes.c_int64),
        ("contains_calls", ctypes.c_int64),
        ("leaf_evals", ctypes.c_int64),
        ("bvh_nodes", ctypes.c_int64),
        ("bvh_tris", ctypes.c_int64),
        ("error", ctypes.c_char * 256),
    ]


class TriSet(ctypes.Structure):
    _fields_ = [("tris", ctypes.c_void_p), ("n", ctypes.c_int64),
                ("grouped", ctypes.c_int32), ("reserved", ctypes.c_int32)]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "mc_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_mc_search.restype = ctypes.c_int
        L.oracle_mc_search.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                       ctypes.c_size_t, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                       ctypes.c_int, ctypes.POINTER(OracleMesh)]
        L.oracle_apply_transform.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.c_int64]
        L.oracle_encode_stl.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        L.oracle_group_triangles.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        L.oracle_mesh_free.argtypes = [ctypes.POINTER(OracleMesh)]
        L.oracle_contains.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                      ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int64,
                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_bounds.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                    ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_spacer_axis.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_void_p, ctypes.c_int64,
                                         ctypes.POINTER(ctypes.c_int64)]
        L.oracle_case_table.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.oracle_rotations.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _scene(nodes, sets):
    nodes = np.ascontiguousarray(nodes)
    arr = (TriSet * max(1, len(sets)))()
    keep = []
    for i, s in enumerate(sets):
        t = np.ascontiguousarray(s.tris, dtype=np.float64)
        keep.append(t)
        arr[i].tris = t.ctypes.data
        arr[i].n = len(t)
        arr[i].grouped = int(s.grouped)
    return nodes, arr, keep


class OracleError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"oracle status {status}: {msg}")
        self.status = status


def mc_search(nodes, sets, delta, iters, threads=None, z_range=(0, -1), interior=False):
    """Returns dict(tris=(T,9) float64 soup in generation order, stats...);
    with interior=True also interior=(T,9): each corner's interior point
    (MarchingCubesInterior, model3d/mc.go:55-60)."""
    nodes, arr, keep = _scene(nodes, sets)
    out = OracleMesh()
    threads = threads or os.cpu_count() or 1
    st = lib().oracle_mc_search(nodes.ctypes.data, len(nodes), ctypes.addressof(arr), len(sets),
                                float(delta), int(iters), int(threads), int(z_range[0]),
                                int(z_range[1]), int(bool(interior)), ctypes.byref(out))
    if st != 0:
        msg = out.error.decode()
        lib().oracle_mesh_free(ctypes.byref(out))
        raise OracleError(st, msg)
    T = out.n_triangles
    tris = np.ctypeslib.as_array(out.tris, shape=(max(T, 1) * 9,))[:T * 9].reshape(T, 9).copy()
    res = dict(tris=tris, n_vertices=out.n_vertices, nx=out.nx, ny=out.ny, nz=out.nz,
               contains_calls=out.contains_calls, leaf_evals=out.leaf_evals,
               bvh_nodes=out.bvh_nodes, bvh_tris=out.bvh_tris)
    if interior:
        res["interior"] = np.ctypeslib.as_array(out.interior, shape=(max(T, 1) * 9,))[:T * 9].reshape(T, 9).copy()
    lib().oracle_mesh_free(ctypes.byref(out))
    return res


RECT_FILTER = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p)


def mc_search_filter(nodes, sets, delta, iters, f, threads=None):
    """MarchingCubesSearchFilter (mc.go:83-155) with the Python filter f,
    called with a Rect (MinVal, MaxVal as Coord3D); iters == 0 is
    MarchingCubesFilter.  Returns dict(tris=(T,9) soup, ...)."""
    from model3d_gb300.geometry import XYZ
    from model3d_gb300.solids import Rect
    calls = [0]

    def cb(r, _user):
        calls[0] += 1
        return 1 if f(Rect(XYZ(r[0], r[1], r[2]), XYZ(r[3], r[4], r[5]))) else 0

    fn = RECT_FILTER(cb)
    L = lib()
    L.oracle_mc_search_filter.restype = ctypes.c_int
    L.oracle_mc_search_filter.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                          ctypes.c_double, ctypes.c_int, ctypes.c_int, RECT_FILTER,
                                          ctypes.c_void_p, ctypes.POINTER(OracleMesh)]
    nodes, arr, keep = _scene(nodes, sets)
    out = OracleMesh()
    st = L.oracle_mc_search_filter(nodes.ctypes.data, len(nodes), ctypes.addressof(arr), len(sets), float(delta),
                                   int(iters), int(threads or os.cpu_count() or 1), fn, None, ctypes.byref(out))
    if st != 0:
        msg = out.error.decode()
        L.oracle_mesh_free(ctypes.byref(out))
        raise OracleError(st, msg)
    T = out.n_triangles
    tris = np.ctypeslib.as_array(out.tris, shape=(max(T, 1) * 9,))[:T * 9].reshape(T, 9).copy()
    res = dict(tris=tris, n_vertices=out.n_vertices, nx=out.nx, ny=out.ny, nz=out.nz, filter_calls=calls[0])
    L.oracle_mesh_free(ctypes.byref(out))
    return res


def encode_stl(tris):
    """EncodeSTL (model3d/export.go) of a (T, 9) triangle soup, as bytes."""
    t = np.ascontiguousarray(tris, dtype=np.float64).reshape(-1, 9)
    out = np.zeros(84 + 50 * len(t), dtype=np.uint8)
    lib().oracle_encode_stl(t.ctypes.data, len(t), out.ctypes.data)
    return out.tobytes()


def group_triangles(tris):
    """GroupTriangles (model3d/bvh.go:118-217) of a (T, 9) triangle soup:
    the permutation SaveGroupedSTL writes the triangles in (ties in the
    midpoint sorts keep the input order)."""
    t = np.ascontiguousarray(tris, dtype=np.float64).reshape(-1, 9)
    out = np.zeros(len(t), dtype=np.int32)
    lib().oracle_group_triangles(t.ctypes.data, len(t), out.ctypes.data)
    return out


def apply_transform(steps, pts, inverse=False):
    """JoinedTransform(steps).Apply -- or its Inverse().Apply -- at each
    point (transform.go); steps are mc_node records of MC_XF_* kinds."""
    steps = np.ascontiguousarray(steps)
    out = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3).copy()
    st = lib().oracle_apply_transform(steps.ctypes.data, len(steps), int(bool(inverse)),
                                      out.ctypes.data, len(out))
    if st != 0:
        raise OracleError(st, "bad transform step")
    return out


def contains(nodes, sets, pts, threads=None):
    nodes, arr, keep = _scene(nodes, sets)
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(len(pts), dtype=np.uint8)
    counts = np.zeros(3, dtype=np.int64)
    st = lib().oracle_contains(nodes.ctypes.data, len(nodes), ctypes.addressof(arr), len(sets),
                               pts.ctypes.data, len(pts), int(threads or os.cpu_count() or 1),
                               out.ctypes.data, counts.ctypes.data)
    if st != 0:
        raise OracleError(st, "contains")
    return out.astype(bool), counts


def bounds(nodes, sets):
    nodes, arr, keep = _scene(nodes, sets)
    mn = np.zeros(3)
    mx = np.zeros(3)
    st = lib().oracle_bounds(nodes.ctypes.data, len(nodes), ctypes.addressof(arr), len(sets),
                             mn.ctypes.data, mx.ctypes.data)
    if st != 0:
        raise OracleError(st, "bounds")
    return mn, mx


def spacer_axis(lo, hi, delta):
    n = ctypes.c_int64()
    lib().oracle_spacer_axis(lo, hi, delta, None, 0, ctypes.byref(n))
    out = np.zeros(n.value)
    st = lib().oracle_spacer_axis(lo, hi, delta, out.ctypes.data, n.value, ctypes.byref(n))
    if st != 0:
        raise OracleError(st, "spacer")
    return out


def case_table():
    counts = np.zeros(256, dtype=np.uint8)
    tris = np.zeros((256, 5, 6), dtype=np.uint8)
    conflicts, covered = ctypes.c_int(), ctypes.c_int()
    lib().oracle_case_table(counts.ctypes.data, tris.ctypes.data, ctypes.byref(conflicts),
                            ctypes.byref(covered))
    return counts, tris, conflicts.value, covered.value


def rotations():
    out = np.zeros((24, 8), dtype=np.uint8)
    n = lib().oracle_rotations(out.ctypes.data)
    return out[:n], n
