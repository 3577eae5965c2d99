"""Pins against the reference's own outputs and fixture meshes
(tests/golden/reference_meshes.json and non_intersecting_hook.npz, made by
tests/golden/make_reference_pins.py from model3d/test_data/).

hierarchy_test.stl.gz is a mesh the reference's MarchingCubesSearch wrote
(model3d/mesh_hierarchy_test.go:104-127, delta 0.03, iters 2; STL keeps the
float32 casts of the normal and the vertices).  The oracle must reproduce
it exactly at that resolution, on CPU; the CUDA path must reproduce it in
both precisions and equal the oracle in float64.  Its triangles and the
hook mesh (model3d/primitives_test.go:273-285) then serve as collider
inputs, compared bit for bit with the oracle.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from model3d_gb300 import (DeviceSolid, JoinedSolid, MarchingCubesSearch, MeshToCollider,
                           NewColliderSolid, Sphere, SubtractedSolid, XYZ, canonical, serialize)

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "reference_meshes.json")))


def hierarchy_solid():
    """The solid of model3d/mesh_hierarchy_test.go:107-124."""
    def shell(c, r):
        return SubtractedSolid(Sphere(c, r), Sphere(c, r - 0.05))
    return JoinedSolid([shell(XYZ(0, 0, 0), 1.0), shell(XYZ(0, 0, 0), 0.5), Sphere(XYZ(0, 0, 0), 0.1),
                        shell(XYZ(3, 0, 0), 1.0), Sphere(XYZ(0, 3, 0), 1.0)])


def f32_digests(tris64, stl_bytes=None):
    """SHA-256 of the float32 casts of (T, 9) float64 triangles, rows sorted
    (vertex order kept), and of the float32 normals of the matching binary
    STL records in the same row order."""
    a = np.ascontiguousarray(np.asarray(tris64, dtype=np.float64).reshape(-1, 9).astype(np.float32)).view(np.uint32)
    order = np.lexsort(a.T[::-1])
    tri = hashlib.sha256(np.ascontiguousarray(a[order]).tobytes()).hexdigest()
    if stl_bytes is None:
        return tri, None
    rec = np.frombuffer(stl_bytes[84:], dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")]))
    assert np.array_equal(rec["v"].view(np.uint32), a)
    nrm = hashlib.sha256(np.ascontiguousarray(rec["n"][order]).tobytes()).hexdigest()
    return tri, nrm


def hook_triangles():
    z = np.load(os.path.join(HERE, "golden", "non_intersecting_hook.npz"))
    return z["vertices"][z["faces"]].reshape(-1, 9)


def test_oracle_reproduces_reference_hierarchy_mesh(oracle):
    g = GOLD["hierarchy_test"]
    nodes, sets = serialize(hierarchy_solid())
    m = oracle.mc_search(nodes, sets, g["delta"], g["iters"])
    assert len(m["tris"]) == g["triangles"]
    tri, nrm = f32_digests(m["tris"], oracle.encode_stl(m["tris"]))
    assert tri == g["sha256_f32_triangles"]
    assert nrm == g["sha256_f32_normals"]


def test_hook_fixture_is_the_reference_file():
    t = hook_triangles()
    assert len(t) == GOLD["non_intersecting_hook"]["triangles"]
    h = hashlib.sha256(np.ascontiguousarray(t, dtype="<f4").tobytes()).hexdigest()
    assert h == GOLD["non_intersecting_hook"]["sha256_f32_file_order"]


def test_oracle_hook_collider_matches_brute_force(oracle):
    """Ray-parity containment on the reference's hook mesh, tree traversal
    against every-triangle brute force (collisions_test.go:22-76)."""
    from test_oracle import _brute_force_parity
    tris = hook_triangles().astype(np.float64)
    s = NewColliderSolid(MeshToCollider(tris))
    nodes, sets = serialize(s)
    mn, mx = np.array(s.Min().Array()), np.array(s.Max().Array())
    rng = np.random.default_rng(5)
    pts = mn + (mx - mn) * rng.uniform(-0.05, 1.05, size=(300, 3))
    inside, _ = oracle.contains(nodes, sets, pts)
    inb = ((pts >= mn) & (pts <= mx)).all(1)
    assert (inside == (_brute_force_parity(tris, pts) & inb)).all()
    assert inside.any() and not inside.all()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_reproduces_reference_hierarchy_mesh(oracle, prec):
    g = GOLD["hierarchy_test"]
    solid = hierarchy_solid()
    m = MarchingCubesSearch(solid, g["delta"], g["iters"], precision=prec)
    assert m.NumTriangles() == g["triangles"]
    assert f32_digests(m.TriangleSoup())[0] == g["sha256_f32_triangles"]
    ref = oracle.mc_search(*serialize(solid), g["delta"], g["iters"])
    assert np.array_equal(canonical(m.TriangleSoup()), canonical(ref["tris"]))


def _collider_parity(oracle, tris, delta, iters=8):
    s = NewColliderSolid(MeshToCollider(np.ascontiguousarray(tris, dtype=np.float64)))
    nodes, sets = serialize(s)
    ref = oracle.mc_search(nodes, sets, delta, iters)
    ds = DeviceSolid(s)
    for prec in ("fp64", "fp32"):
        m = MarchingCubesSearch(ds, delta, iters, precision=prec)
        a, b = canonical(m.TriangleSoup()), canonical(ref["tris"])
        assert a.shape == b.shape, (prec, a.shape, b.shape)
        assert np.array_equal(a, b), prec
        assert m.stats["vertices"] == ref["n_vertices"]
    return len(ref["tris"])


@pytest.mark.gpu
def test_gpu_hook_collider_matches_oracle(oracle):
    """The reference's hook fixture as MeshToCollider input (delta 0.003, a
    272 x 358 x 70 grid over its 1.06-unit extent, iters 8)."""
    assert _collider_parity(oracle, hook_triangles(), 0.003) > 0


@pytest.mark.gpu
def test_gpu_hierarchy_mesh_collider_matches_oracle(oracle):
    """The reference's 220,180-triangle hierarchy mesh (regenerated by the
    oracle and checked against the fixture's digest first) as a collider:
    three nested shells, so rays cross up to ten surfaces."""
    g = GOLD["hierarchy_test"]
    ref = oracle.mc_search(*serialize(hierarchy_solid()), g["delta"], g["iters"])
    tris = ref["tris"].astype(np.float32).astype(np.float64)
    assert f32_digests(tris)[0] == g["sha256_f32_triangles"]
    assert _collider_parity(oracle, tris, 0.02) > 0
