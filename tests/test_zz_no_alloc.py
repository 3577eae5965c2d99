"""mc_search_noalloc: the allocation-free entry point, for callers that cannot
allocate device memory when they mesh (their device memory belongs to another
allocator that hands them only their own buffers, or their loop forbids
cudaMalloc/cudaFree after start-up because those can synchronise the device).

Its intermediate arrays live in a fixed device array inside the library; the
caller passes the solid and its own output buffers.  The output must equal
the allocating entry point's (mc_search) bit for bit — the same tolerance as
every parity test here — on consecutive calls, since the shared scratch
array keeps the previous call's contents.

This file is collected last so that a failure here does not hide the others.
"""
import ctypes

import numpy as np
import pytest

from model3d_gb300 import (MarchingCubesSearch, MeshToCollider, NewColliderSolid, Sphere, SubtractedSolid,
                           XYZ, serialize)
from model3d_gb300 import _native as N
from model3d_gb300.workloads import csg_tree, displaced_icosphere, metaball_blob

pytestmark = pytest.mark.gpu


def _noalloc(solid, delta, iters, vcap, tcap, torch, stream=None, opts=None, bufs=None):
    nodes, sets = serialize(solid)
    dv, dt = bufs or (torch.full((max(vcap, 1) * 3,), float("nan"), dtype=torch.float64, device="cuda"),
                      torch.full((max(tcap, 1) * 3,), -1, dtype=torch.int32, device="cuda"))
    torch.cuda.synchronize()
    nv, nt = ctypes.c_int64(), ctypes.c_int64()
    st = N.lib().mc_search_noalloc(nodes.ctypes.data, len(nodes), float(delta), int(iters),
                                   ctypes.byref(opts) if opts is not None else None,
                                   stream.cuda_stream if stream is not None else None,
                                   dv.data_ptr(), vcap, dt.data_ptr(), tcap,
                                   ctypes.byref(nv), ctypes.byref(nt))
    return st, nv.value, nt.value, dv, dt


def _same_as_allocating(ref, st, nv, nt, dv, dt):
    V, T = len(ref.vertices), len(ref.triangles)
    assert st == N.MC_OK, N.status_string(st)
    assert (nv, nt) == (V, T)
    verts = dv[:V * 3].cpu().numpy().reshape(V, 3)
    tris = dt[:T * 3].cpu().numpy().reshape(T, 3)
    assert np.array_equal(verts.view(np.uint64), ref.vertices.view(np.uint64))
    assert np.array_equal(tris, ref.triangles)


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    cases = [(csg_tree(3, 12, 4), 0.015, 8),      # larger grid first ...
             (Sphere(XYZ(0.1, 0.3, -0.2), 0.6), 0.05, 8),  # ... then a smaller one over its leftovers
             (csg_tree(3, 12, 4), 0.015, 8),
             (metaball_blob(4, 16), 0.02, 8)]             # metaball leaves take the same path
    for solid, delta, iters in cases:
        ref = MarchingCubesSearch(solid, delta, iters)
        V, T = len(ref.vertices), len(ref.triangles)
        st, nv, nt, dv, dt = _noalloc(solid, delta, iters, V + 7, T + 5, torch)
        _same_as_allocating(ref, st, nv, nt, dv, dt)
        # nothing written past the mesh
        assert torch.isnan(dv[V * 3:]).all() and (dt[T * 3:] == -1).all()


def test_noalloc_rejects_small_buffers_and_oversized_grids():
    torch = pytest.importorskip("torch")
    solid = Sphere(XYZ(0, 0, 0), 1.0)
    ref = MarchingCubesSearch(solid, 0.05, 8)
    st, nv, nt, _, _ = _noalloc(solid, 0.05, 8, 10, 10, torch)
    assert st == N.MC_ERR_LIMIT
    assert (nv, nt) == (len(ref.vertices), len(ref.triangles))
    # 2000^3 corners cannot fit the fixed scratch array
    st, _, _, _, _ = _noalloc(solid, 0.001, 8, 10, 10, torch)
    assert st == N.MC_ERR_LIMIT


def test_noalloc_on_a_side_stream_and_without_device_allocation():
    """Two calls on a non-default stream equal mc_search; a warm call leaves
    the device's free memory where it was (nothing is allocated)."""
    torch = pytest.importorskip("torch")
    solid = csg_tree(5, 10, 3)
    ref = MarchingCubesSearch(solid, 0.02, 8)
    V, T = len(ref.vertices), len(ref.triangles)
    side = torch.cuda.Stream()
    bufs = (torch.full((V * 3,), float("nan"), dtype=torch.float64, device="cuda"),
            torch.full((T * 3,), -1, dtype=torch.int32, device="cuda"))
    _same_as_allocating(ref, *_noalloc(solid, 0.02, 8, V, T, torch, stream=side, bufs=bufs))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        _same_as_allocating(ref, *_noalloc(solid, 0.02, 8, V, T, torch, stream=side, bufs=bufs))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_refuses_colliders_and_interior_points():
    torch = pytest.importorskip("torch")
    col = SubtractedSolid(NewColliderSolid(MeshToCollider(displaced_icosphere(4))), Sphere(XYZ(0, 0, 0), 0.3))
    st, _, _, _, _ = _noalloc(col, 0.05, 8, 1000, 1000, torch)
    assert st == N.MC_ERR_BAD_PROGRAM
    o = N.MCOpts()
    o.precision = N.MC_PREC_FP32_FILTERED
    o.cull = 1
    o.interior = 1
    st, _, _, _, _ = _noalloc(Sphere(XYZ(0, 0, 0), 1.0), 0.05, 8, 10000, 10000, torch, opts=o)
    assert st == N.MC_ERR_ARG


def test_noalloc_program_beyond_48_kib_of_shared_memory():
    """A 1,700-leaf CSG tree folds into more than 48 KiB of shared memory per
    classification block; the call raises the kernel's limit as mc_search
    does (setting the attribute allocates nothing)."""
    torch = pytest.importorskip("torch")
    solid = csg_tree(8, 1500, 200)
    assert N.lib() and len(serialize(solid)[0]) > 1700
    ref = MarchingCubesSearch(solid, 0.03, 8)
    V, T = len(ref.vertices), len(ref.triangles)
    _same_as_allocating(ref, *_noalloc(solid, 0.03, 8, V, T, torch))
