"""Consecutive mc_search_device calls on one context, growing and shrinking:
the context's grow-only buffers and solid pool carry over between calls, and
every result must equal mc_search's bit for bit; a border panic leaves the
context usable.
"""
import ctypes

import numpy as np
import pytest

from model3d_gb300 import (Context, DeviceSolid, MarchingCubesSearch, MCError, MeshToCollider, NewColliderSolid,
                           Sphere, XYZ, serialize)
from model3d_gb300 import _native as N
from model3d_gb300.workloads import csg_tree, displaced_icosphere, metaball_blob

pytestmark = pytest.mark.gpu


def _device(ctx, ds, delta, iters=8, prec=N.MC_PREC_FP32_FILTERED):
    L = N.lib()
    o = N.MCOpts()
    o.precision = prec
    o.cull = 1
    V, T = ctypes.c_int64(), ctypes.c_int64()
    st = N.MCStats()
    s = L.mc_search_device(ctx.ptr, ds.ptr, float(delta), int(iters), ctypes.byref(o), ctypes.byref(V),
                           ctypes.byref(T), ctypes.byref(st))
    if s != N.MC_OK:
        raise MCError(s, L.mc_last_error(ctx.ptr).decode())
    v = np.empty((V.value, 3))
    t = np.empty((T.value, 3), dtype=np.int32)
    assert L.mc_result_copy(ctx.ptr, v.ctypes.data, t.ctypes.data) == N.MC_OK
    return v, t, st


def test_device_calls_grow_shrink_and_match_the_waiting_path():
    ctx = Context(0)
    cases = [(Sphere(XYZ(0, 0, 0), 1.0), 0.1),
             (csg_tree(1, 48, 16), 0.01),   # outgrows the first call's buffers
             (Sphere(XYZ(0.21, -0.03, 0.02), 0.5), 0.05),
             (csg_tree(1, 48, 16), 0.008),  # larger again
             (NewColliderSolid(MeshToCollider(displaced_icosphere(10))), 0.03),
             (metaball_blob(2, 12), 0.02),
             (csg_tree(1, 48, 16), 0.01)]
    for solid, delta in cases:
        ds = DeviceSolid(solid, ctx)
        for prec in (N.MC_PREC_FP32_FILTERED, N.MC_PREC_FP64):
            v, t, st = _device(ctx, ds, delta, prec=prec)
            ref = MarchingCubesSearch(ds, delta, 8, precision="fp64" if prec == N.MC_PREC_FP64 else "fp32")
            assert np.array_equal(v.view(np.uint64), ref.vertices.view(np.uint64))
            assert np.array_equal(t, ref.triangles)
            assert (st.vertices, st.triangles) == (len(ref.vertices), len(ref.triangles))


def test_border_panic_on_a_warm_context(oracle):
    ctx = Context(0)

    class Lying(Sphere):
        def Min(self):
            return XYZ(-0.5, -0.5, -0.5)

        def Max(self):
            return XYZ(0.5, 0.5, 0.5)

    good = DeviceSolid(Sphere(XYZ(0, 0, 0), 1.0), ctx)
    _device(ctx, good, 0.05)
    bad = DeviceSolid(Lying(XYZ(0, 0, 0), 1.0), ctx)
    with pytest.raises(MCError) as e:
        _device(ctx, bad, 0.05)
    assert e.value.status == N.MC_ERR_BOUNDS_INSIDE
    v, t, _ = _device(ctx, good, 0.05)
    ref = MarchingCubesSearch(good, 0.05, 8)
    assert np.array_equal(v.view(np.uint64), ref.vertices.view(np.uint64))
    # Right bounds, but the corner (0.7000000000000001, -6.9e-17, -6.9e-17)
    # of the spacer's last x plane is inside in float64 (its squared distance
    # to the centre rounds to 0.25): the reference panics, and so does every
    # precision here.
    tight = Sphere(XYZ(0.2, 0, 0), 0.5)
    with pytest.raises(RuntimeError, match="outside of bounds"):
        oracle.mc_search(*serialize(tight), 0.05, 8)
    ds = DeviceSolid(tight, ctx)
    for prec in (N.MC_PREC_FP32_FILTERED, N.MC_PREC_FP64):
        with pytest.raises(MCError) as e:
            _device(ctx, ds, 0.05, prec=prec)
        assert e.value.status == N.MC_ERR_BOUNDS_INSIDE
    _device(ctx, good, 0.05)
