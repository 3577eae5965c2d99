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

from model3d_gb300 import MarchingCubesSearch, Sphere, XYZ, serialize
from model3d_gb300 import _native as N
from model3d_gb300.workloads import csg_tree, metaball_blob

pytestmark = pytest.mark.gpu


def _noalloc(solid, delta, iters, vcap, tcap, torch):
    nodes, sets = serialize(solid)
    assert not sets
    dv = torch.full((max(vcap, 1) * 3,), float("nan"), dtype=torch.float64, device="cuda")
    dt = torch.full((max(tcap, 1) * 3,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    nv, nt = ctypes.c_int64(), ctypes.c_int64()
    st = N.lib().mc_search_noalloc(nodes.ctypes.data, len(nodes), float(delta), int(iters), None,
                                   None, dv.data_ptr(), vcap, dt.data_ptr(), tcap,
                                   ctypes.byref(nv), ctypes.byref(nt))
    return st, nv.value, nt.value, dv, dt


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
        assert st == N.MC_OK, N.status_string(st)
        assert (nv, nt) == (V, T)
        verts = dv[:V * 3].cpu().numpy().reshape(V, 3)
        tris = dt[:T * 3].cpu().numpy().reshape(T, 3)
        assert np.array_equal(verts.view(np.uint64), ref.vertices.view(np.uint64))
        assert np.array_equal(tris, ref.triangles)
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
