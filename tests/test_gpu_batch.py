"""Batched search (mc_search_batch): one launch per phase for many solids.

Every job's mesh must equal the single-solid entry point's bit for bit (same
vertex and triangle layout), on the first call (sizing run) and on a repeated
call (CUDA-graph replay); failing jobs report their own status without
disturbing the others.
"""
import numpy as np
import pytest

from model3d_gb300 import (DeviceSolid, MarchingCubesSearch, MarchingCubesSearchBatch, MCError,
                           NewColliderSolid, MeshToCollider, Sphere, XYZ, canonical)
from model3d_gb300 import _native as N
from model3d_gb300.workloads import csg_batch, csg_tree, displaced_icosphere

pytestmark = pytest.mark.gpu


def _jobs():
    jobs = [(DeviceSolid(s), d, 8) for s, d in csg_batch(5, count=14, grid_lo=16, grid_hi=96)]
    jobs.append((DeviceSolid(Sphere(XYZ(0.1, 0.2, 0.3), 0.7)), 0.05, 0))
    jobs.append((DeviceSolid(NewColliderSolid(MeshToCollider(displaced_icosphere(6)))), 0.04, 8))
    jobs.append((DeviceSolid(csg_tree(9, 3, 1)), 0.03, 2))
    return jobs


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batch_equals_single_calls_and_replay(prec):
    jobs = _jobs()
    refs = [MarchingCubesSearch(ds, d, it, precision=prec) for ds, d, it in jobs]
    for call in range(2):  # second call replays the captured graph
        out = MarchingCubesSearchBatch(jobs, precision=prec)
        assert len(out) == len(jobs)
        for m, r in zip(out, refs):
            assert not isinstance(m, MCError)
            assert np.array_equal(m.vertices.view(np.uint64), r.vertices.view(np.uint64))
            assert np.array_equal(m.triangles, r.triangles)


def test_batch_job_failures_are_per_job():
    class Lying(Sphere):
        def Min(self):
            return XYZ(-0.5, -0.5, -0.5)

        def Max(self):
            return XYZ(0.5, 0.5, 0.5)

    class Inverted(Sphere):
        def Max(self):
            return XYZ(-2, 0, 0)

    good = DeviceSolid(csg_tree(4, 6, 2))
    jobs = [(good, 0.03, 8), (DeviceSolid(Lying(XYZ(0, 0, 0), 1.0)), 0.1, 8),
            (DeviceSolid(Inverted(XYZ(0, 0, 0), 1.0)), 0.1, 8), (good, 0.05, 8)]
    out = MarchingCubesSearchBatch(jobs)
    assert isinstance(out[1], MCError) and out[1].status == N.MC_ERR_BOUNDS_INSIDE
    assert isinstance(out[2], MCError) and out[2].status == N.MC_ERR_INVALID_BOUNDS
    for k in (0, 3):
        ref = MarchingCubesSearch(good, jobs[k][1], 8)
        assert np.array_equal(canonical(out[k].TriangleSoup()), canonical(ref.TriangleSoup()))


def test_autotune_keeps_results_and_peaks_are_positive():
    from model3d_gb300 import autotune, measure_peaks
    ds = DeviceSolid(csg_tree(2, 16, 4))
    ref = MarchingCubesSearch(ds, 0.02, 8)
    ty, tz, ms = autotune(ds, 0.02, 8)
    assert ty * tz <= 32 and ms > 0
    m = MarchingCubesSearch(ds, 0.02, 8)  # tuned shape is now the context default
    assert np.array_equal(m.vertices.view(np.uint64), ref.vertices.view(np.uint64))
    assert np.array_equal(m.triangles, ref.triangles)
    f32, f64, l2 = measure_peaks()
    assert f32 > 0 and f64 > 0 and l2 > 0


def test_solid_outliving_its_context():
    """mc_destroy detaches the context's solids; destroying them afterwards
    frees their device buffers without touching the context."""
    from model3d_gb300 import Context
    ctx = Context(0)
    ds = DeviceSolid(csg_tree(2, 4, 1), ctx)
    m = MarchingCubesSearch(ds, 0.05, 8)
    assert m.NumTriangles() > 0
    ctx.close()
    ds.close()
