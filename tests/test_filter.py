"""MarchingCubesFilter / SearchFilter / C2F (model3d/mc.go:73-180).

CPU: the oracle's restatement of the block pruning (per-block corner caches,
oracle/mc_oracle.cpp) against the reference's own tests (mc_test.go:44-94:
a collider's RectCollision as the filter gives MarchingCubes' mesh, and
MarchingCubesC2F gives MarchingCubesSearch's); the host block recursion of
model3d_gb300/filter.py visits the same blocks with the same bounds as the
oracle's; RectCollider (the tree's parent-box pruning) answers as brute force
over every triangle.

GPU: the library's filtered meshes equal the oracle's bit for bit, for the
reference's conservative filters and for filters that drop cubes the
surface crosses.
"""
import math

import numpy as np
import pytest

from model3d_gb300 import (DeviceSolid, MarchingCubesC2F, MarchingCubesFilter, MarchingCubesSearchFilter,
                           MeshToCollider, NewColliderSolid, Rect, RectCollider, Sphere, XYZ, canonical, serialize,
                           spacer_axis)
from model3d_gb300.filter import kept_cubes
from model3d_gb300.workloads import box_triangles, csg_tree, icosphere_triangles


def _icosphere():
    """An icosphere of radius 1 centred at (0.1, 0.3, -0.2), as mc_test.go:46."""
    t = icosphere_triangles(20).reshape(-1, 3, 3) + np.array([0.1, 0.3, -0.2])
    return t.reshape(-1, 9)


def _boxes(gap=0.1):
    """The two-box mesh of mc_test.go:55-57 (0.3 for C2F, mc_test.go:82-84)."""
    return np.concatenate([box_triangles((-1, -1, -1), (0, 0, 0)), box_triangles((gap, 0, 0), (1, 1, 1))])


def _same(a, b):
    x, y = canonical(a), canonical(b)
    return x.shape == y.shape and np.array_equal(x, y)


@pytest.mark.parametrize("mesh", ["icosphere", "boxes"])
def test_oracle_filter_with_rect_collision_is_marching_cubes(oracle, mesh):
    """mc_test.go:44-67."""
    tris = _icosphere() if mesh == "icosphere" else _boxes()
    solid = NewColliderSolid(MeshToCollider(tris))
    nodes, sets = serialize(solid)
    base = oracle.mc_search(nodes, sets, 0.1, 0)
    rc = oracle.mc_search_filter(nodes, sets, 0.1, 0, RectCollider(tris).RectCollision)
    assert _same(rc["tris"], base["tris"])
    assert rc["filter_calls"] > 0


def _oracle_c2f(oracle, solid, big, small, extra, iters):
    """MarchingCubesC2F (mc.go:165-180) over the oracle: coarse mesh, its
    collider, the filtered fine search."""
    nodes, sets = serialize(solid)
    coarse = oracle.mc_search(nodes, sets, big, iters)
    col = RectCollider(coarse["tris"])
    e = extra + 2 * big * math.sqrt(3)
    return oracle.mc_search_filter(nodes, sets, small, iters, lambda r: col.RectCollision(r.Expand(e)))


@pytest.mark.parametrize("mesh", ["sphere", "boxes"])
def test_oracle_c2f_is_marching_cubes_search(oracle, mesh):
    """mc_test.go:69-94."""
    if mesh == "sphere":
        solid, big, small = Sphere(XYZ(0.1, 0.3, -0.2), 1.0), 0.1, 0.05
    else:
        solid, big, small = NewColliderSolid(MeshToCollider(_boxes(0.3))), 0.2, 0.1
    nodes, sets = serialize(solid)
    full = oracle.mc_search(nodes, sets, small, 8)
    assert _same(_oracle_c2f(oracle, solid, big, small, 0, 8)["tris"], full["tris"])


def test_host_block_recursion_visits_the_oracles_blocks(oracle):
    """kept_cubes calls f on the same blocks, with the same bounds bit for
    bit, in the same order, as the oracle's Pieces."""
    solid = csg_tree(4, 10, 3)
    nodes, sets = serialize(solid)
    delta = 0.025

    def f(r):
        return r.MinVal.X + r.MaxVal.Y < 0.4 or r.MaxVal.Z > 0.5

    seen_o, seen_h = [], []
    oracle.mc_search_filter(nodes, sets, delta, 0, lambda r: seen_o.append(r.MinVal.Array() + r.MaxVal.Array()) or f(r))
    mn, mx = solid.Min(), solid.Max()
    xs, ys, zs = (spacer_axis(a, b, delta) for a, b in ((mn.X, mx.X), (mn.Y, mx.Y), (mn.Z, mx.Z)))
    mask = kept_cubes(lambda r: seen_h.append(r.MinVal.Array() + r.MaxVal.Array()) or f(r), xs, ys, zs, delta)
    assert len(seen_h) == len(seen_o) > 100
    assert np.array_equal(np.array(seen_h).view(np.uint64), np.array(seen_o).view(np.uint64))
    assert 0 < mask.sum() < mask.size


def test_rect_collider_matches_brute_force():
    tris = _icosphere()
    col = RectCollider(tris)
    brute = RectCollider.__new__(RectCollider)
    brute.tris, brute.root_only, brute.pbox = col.tris, True, None  # every triangle, no box pruning
    rng = np.random.default_rng(3)
    hits = 0
    for _ in range(300):
        c = rng.uniform(-1.3, 1.3, 3)
        h = rng.uniform(0.01, 0.4, 3)
        r = Rect(XYZ(*(c - h)), XYZ(*(c + h)))
        a, b = col.RectCollision(r), brute.RectCollision(r)
        assert a == b
        hits += a
    assert 0 < hits < 300


@pytest.mark.gpu
@pytest.mark.parametrize("mesh", ["icosphere", "boxes"])
def test_gpu_filter_with_rect_collision(oracle, mesh):
    tris = _icosphere() if mesh == "icosphere" else _boxes()
    solid = NewColliderSolid(MeshToCollider(tris))
    nodes, sets = serialize(solid)
    base = oracle.mc_search(nodes, sets, 0.1, 0)
    for prec in ("fp64", "fp32"):
        m = MarchingCubesFilter(solid, RectCollider(tris).RectCollision, 0.1, precision=prec)
        assert _same(m.TriangleSoup(), base["tris"]), prec


@pytest.mark.gpu
@pytest.mark.parametrize("iters", [0, 8])
def test_gpu_filter_that_drops_surface_cubes_matches_oracle(oracle, iters):
    """Filters that break the reference's contract: the kept cubes' triangles
    and their searched vertices are still the reference's."""
    solid = csg_tree(4, 10, 3)
    nodes, sets = serialize(solid)
    ds = DeviceSolid(solid)
    filters = [lambda r: r.MinVal.X < 0.1,
               lambda r: r.MinVal.X + r.MaxVal.Y < 0.4 or r.MaxVal.Z > 0.5,
               lambda r: (int((r.MinVal.X + 2) * 37) + int((r.MinVal.Z + 2) * 11)) % 3 != 0]
    for f in filters:
        ref = oracle.mc_search_filter(nodes, sets, 0.025, iters, f)
        for prec in ("fp64", "fp32"):
            m = MarchingCubesSearchFilter(ds, f, 0.025, iters, precision=prec)
            assert _same(m.TriangleSoup(), ref["tris"]), prec
            assert len(m.vertices) == ref["n_vertices"]


@pytest.mark.gpu
@pytest.mark.parametrize("mesh", ["sphere", "boxes"])
def test_gpu_c2f(oracle, mesh):
    if mesh == "sphere":
        solid, big, small = Sphere(XYZ(0.1, 0.3, -0.2), 1.0), 0.1, 0.05
    else:
        solid, big, small = NewColliderSolid(MeshToCollider(_boxes(0.3))), 0.2, 0.1
    nodes, sets = serialize(solid)
    full = oracle.mc_search(nodes, sets, small, 8)
    m = MarchingCubesC2F(solid, big, small, 0, 8)
    assert _same(m.TriangleSoup(), full["tris"])
    assert _same(m.TriangleSoup(), _oracle_c2f(oracle, solid, big, small, 0, 8)["tris"])
    # a coarse pass that misses a thin feature: the fine mesh loses it exactly as the reference's
    thin = csg_tree(6, 14, 0)
    ref = _oracle_c2f(oracle, thin, 0.3, 0.03, 0, 8)
    assert _same(MarchingCubesC2F(thin, 0.3, 0.03, 0, 8).TriangleSoup(), ref["tris"])
