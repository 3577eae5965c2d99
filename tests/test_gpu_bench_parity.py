"""Parity with the oracle at the sizes the benchmark measures.

Every benchmark configuration is compared bit for bit (canonical triangle
sort, nine float64 bit patterns per triangle, vertex order kept) with the
oracle on the same inputs, in both precisions:

* the 48-minus-16 CSG tree at delta 0.004 (580 x 613 x 606 corners);
* the 1,048,820-triangle displaced icosphere collider on its 256^3 grid;
* the 512-solid CSG batch: its 8 largest and 8 seeded-random jobs, taken
  from the batched call;
* the 64-mesh collider batch: its largest-triangle and largest-grid meshes,
  taken from the batched call.

The oracle runs on all host threads (a few seconds to a minute each).
"""
import numpy as np
import pytest

from model3d_gb300 import (DeviceSolid, MarchingCubesSearch, MarchingCubesSearchBatch, MeshToCollider,
                           NewColliderSolid, canonical, serialize)
from model3d_gb300.workloads import collider_batch, csg_batch, csg_tree, displaced_icosphere

pytestmark = pytest.mark.gpu


def _same(mesh, ref, what):
    a, b = canonical(mesh.TriangleSoup()), canonical(ref["tris"])
    assert a.shape == b.shape, f"{what}: {len(a)} triangles, oracle {len(b)}"
    bad = np.nonzero((a != b).any(1))[0]
    assert len(bad) == 0, f"{what}: {len(bad)} triangles differ"
    assert mesh.stats["vertices"] == ref["n_vertices"], what
    assert (mesh.stats["nx"], mesh.stats["ny"], mesh.stats["nz"]) == (ref["nx"], ref["ny"], ref["nz"]), what


def test_headline_csg_full_size_matches_oracle(oracle):
    solid = csg_tree(1, 48, 16)
    ref = oracle.mc_search(*serialize(solid), 0.004, 8)
    ds = DeviceSolid(solid)
    for prec in ("fp32", "fp64"):
        m = MarchingCubesSearch(ds, 0.004, 8, precision=prec)
        _same(m, ref, prec)
    assert m.stats["corners"] == 580 * 613 * 606


def test_collider_1m_triangles_full_size_matches_oracle(oracle):
    tris = displaced_icosphere(229)
    assert len(tris) == 1048820
    s = NewColliderSolid(MeshToCollider(tris))
    mn, mx = s.Min(), s.Max()
    delta = max(mx.X - mn.X, mx.Y - mn.Y, mx.Z - mn.Z) / 255
    ref = oracle.mc_search(*serialize(s), delta, 8)
    ds = DeviceSolid(s)
    for prec in ("fp32", "fp64"):
        _same(MarchingCubesSearch(ds, delta, 8, precision=prec), ref, prec)


def test_csg_batch_512_sampled_jobs_match_oracle(oracle):
    items = csg_batch(2024, count=512)
    jobs = [(DeviceSolid(s), d, 8) for s, d in items]
    outs = {prec: MarchingCubesSearchBatch(jobs, precision=prec) for prec in ("fp32", "fp64")}
    corners = [m.stats["corners"] for m in outs["fp32"]]
    largest = list(np.argsort(corners)[::-1][:8])
    rng = np.random.default_rng(2024)
    rest = [i for i in range(len(jobs)) if i not in largest]
    picked = largest + list(rng.choice(rest, 8, replace=False))
    assert max(corners) >= 300 ** 3
    for i in picked:
        solid, delta = items[i]
        ref = oracle.mc_search(*serialize(solid), delta, 8)
        for prec in ("fp32", "fp64"):
            _same(outs[prec][i], ref, f"job {i} {prec}")


@pytest.fixture(scope="module")
def collider_batch_64():
    meshes = collider_batch(77, count=64)
    solids, jobs = [], []
    for tris, _, side in meshes:
        s = NewColliderSolid(MeshToCollider(tris))
        mn, mx = s.Min(), s.Max()
        delta = max(mx.X - mn.X, mx.Y - mn.Y, mx.Z - mn.Z) / (side - 3)
        solids.append(s)
        jobs.append((DeviceSolid(s), delta, 8))
    outs = {prec: MarchingCubesSearchBatch(jobs, precision=prec) for prec in ("fp32", "fp64")}
    return meshes, solids, jobs, outs


@pytest.mark.parametrize("which", ["most_triangles", "largest_grid"])
def test_collider_batch_64_jobs_match_oracle(oracle, collider_batch_64, which):
    meshes, solids, jobs, outs = collider_batch_64
    if which == "most_triangles":
        i = int(np.argmax([len(t) for t, _, _ in meshes]))
        assert len(meshes[i][0]) > 1_800_000
    else:
        i = int(np.argmax([m.stats["corners"] for m in outs["fp32"]]))
        assert outs["fp32"][i].stats["corners"] > 400 ** 3
    ref = oracle.mc_search(*serialize(solids[i]), jobs[i][1], 8)
    for prec in ("fp32", "fp64"):
        _same(outs[prec][i], ref, f"job {i} {prec}")
