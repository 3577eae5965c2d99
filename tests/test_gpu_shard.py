"""The two splits of the path (model3d_gb300/shard.py), run one part after
another on one GPU: every merged result must equal the single call bit for
bit (canonical triangle sort).

* z-slabs of one solid (mc_opts.z_begin / z_end), merged on the host;
* a batch partitioned largest-first, each part as its own batched call.
"""
import numpy as np
import pytest

from model3d_gb300 import (DeviceSolid, MarchingCubesSearch, MarchingCubesSearchBatch, MCError, MeshToCollider,
                           NewColliderSolid, Sphere, XYZ, canonical)
from model3d_gb300 import _native as N
from model3d_gb300.shard import (MarchingCubesSearchSlab, MarchingCubesSearchSlabs, grid_shape, job_costs,
                                 partition_jobs, slab_ranges)
from model3d_gb300.workloads import csg_batch, csg_tree, displaced_icosphere, metaball_blob

pytestmark = pytest.mark.gpu


def _same(a, b, what=""):
    x, y = canonical(a.TriangleSoup()), canonical(b.TriangleSoup())
    assert x.shape == y.shape, (what, x.shape, y.shape)
    assert np.array_equal(x, y), what
    assert len(a.vertices) == len(b.vertices), what


@pytest.mark.parametrize("parts", [2, 3, 7])
@pytest.mark.parametrize("iters", [0, 8])
def test_slabs_merge_to_the_single_call(parts, iters):
    solid = csg_tree(1, 48, 16)
    ds = DeviceSolid(solid)
    for prec in ("fp32", "fp64"):
        whole = MarchingCubesSearch(ds, 0.01, iters, precision=prec)
        merged = MarchingCubesSearchSlabs(ds, 0.01, iters, parts, precision=prec)
        _same(merged, whole, f"{parts} slabs, {prec}")


def test_slabs_of_colliders_metaballs_and_a_sphere():
    cases = [(NewColliderSolid(MeshToCollider(displaced_icosphere(20))), 0.02),
             (metaball_blob(2, 12), 0.02),
             (Sphere(XYZ(0.1, 0.3, -0.2), 1.0), 0.02)]
    for solid, delta in cases:
        ds = DeviceSolid(solid)
        _same(MarchingCubesSearchSlabs(ds, delta, 8, 4), MarchingCubesSearch(ds, delta, 8), type(solid).__name__)


def test_slab_of_one_layer_and_slab_limits():
    solid = Sphere(XYZ(0, 0, 0), 1.0)
    nx, ny, nz = grid_shape(solid, 0.05)
    ranges = [(z, z + 1) for z in range(nz - 1)]  # every cube layer on its own
    parts = [MarchingCubesSearchSlab(solid, 0.05, 8, a, b) for a, b in ranges]
    assert sum(m.NumTriangles() for m in parts) == MarchingCubesSearch(solid, 0.05, 8).NumTriangles()
    for bad in [(-1, 3), (3, 3), (5, 2), (0, nz)]:
        with pytest.raises(MCError) as e:
            MarchingCubesSearchSlab(solid, 0.05, 8, *bad)
        assert e.value.status == N.MC_ERR_ARG


def test_slabs_keep_the_border_panic_of_the_whole_grid():
    """A sphere whose declared bounds cut it at the top (z max 0.5 for a
    sphere reaching 0.8) is true on the grid's top border plane only: the
    slab holding that plane panics ("solid is true outside of bounds",
    mc.go:687-689) and the others do not, as in the reference's ring, which
    checks planes 0 and nz - 1 of the whole grid."""
    class Lying(Sphere):
        def Min(self):
            return XYZ(-0.5, -0.5, -0.5)

        def Max(self):
            return XYZ(0.5, 0.5, 0.5)

    solid = Lying(XYZ(0, 0, 0.5), 0.3)
    ds = DeviceSolid(solid)
    with pytest.raises(MCError) as e:
        MarchingCubesSearch(ds, 0.1, 8)
    assert e.value.status == N.MC_ERR_BOUNDS_INSIDE
    nx, ny, nz = grid_shape(solid, 0.1)
    assert MarchingCubesSearchSlab(ds, 0.1, 8, 0, nz - 2).NumTriangles() > 0
    with pytest.raises(MCError) as e:
        MarchingCubesSearchSlab(ds, 0.1, 8, nz - 3, nz - 1)
    assert e.value.status == N.MC_ERR_BOUNDS_INSIDE


def test_batch_partitioned_largest_first_equals_one_batch():
    items = csg_batch(7, count=40, grid_lo=16, grid_hi=120)
    jobs = [(DeviceSolid(s), d, 8) for s, d in items]
    whole = MarchingCubesSearchBatch(jobs)
    parts = partition_jobs(job_costs(jobs), 3)
    assert sorted(i for p in parts for i in p) == list(range(len(jobs)))
    for p in parts:
        got = MarchingCubesSearchBatch([jobs[i] for i in p])
        for i, m in zip(p, got):
            _same(m, whole[i], f"job {i}")
    # slab ranges cover the cube layers once
    assert slab_ranges(10, 3) == [(0, 3), (3, 6), (6, 10)]
