"""GroupTriangles (model3d/bvh.go:118-217) and SaveGroupedSTL
(model3d/mesh.go:724-742).

The reference's grouped order is not deterministic: it sorts a slice taken
in Go map order (mesh.go:757-763) with the unstable sort.Slice
(bvh.go:236-250), so midpoint ties land in any order.  The oracle and the
library both sort stably over their input order, and the library's device
order must equal the oracle's bit for bit on the same input.  The oracle is
pinned to the reference's own grouped file (model3d/test_data/
hierarchy_test.stl.gz) at the top of the hierarchy, which ties do not move:
the separating axes of the nodes above depth 3 and the depth-3 midpoint
centroids.

CPU: the oracle against the reference's file, the hierarchy invariant, and
permutation checks.  GPU: mc_mesh_group / mc_result_group /
mc_result_stl_grouped / Mesh.SaveGroupedSTL against the oracle, on soups
with many ties, sizes on both sides of every kernel switch, degenerate
meshes and a searched mesh.
"""
import json
import os

import numpy as np
import pytest

from model3d_gb300 import serialize

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "reference_meshes.json")))


def _mids(tris):
    t = np.asarray(tris, dtype=np.float64).reshape(-1, 3, 3)
    return (t.min(1) + t.max(1)) * 0.5


def _check_hierarchy(tris, order):
    """Every node of more than two triangles has halves separated by
    midpoint along some axis (splitBounders cuts one axis' sorted order at
    n/2), and the order is a permutation."""
    assert np.array_equal(np.sort(order), np.arange(len(tris)))
    mid = _mids(tris)[order]
    stack = [(0, len(order))]
    while stack:
        lo, n = stack.pop()
        if n <= 2:
            continue
        h = n // 2
        a, b = mid[lo:lo + h], mid[lo + h:lo + n]
        assert any(a[:, k].max() <= b[:, k].min() for k in range(3)), (lo, n)
        stack += [(lo, h), (lo + h, n - h)]


def _signature(tris, order, depth):
    mid = _mids(np.asarray(tris, dtype=np.float64).astype(np.float32))[order]
    axes, cents = [], []

    def rec(lo, n, d):
        if d == depth:
            cents.append(mid[lo:lo + n].mean(0))
            return
        h = n // 2
        axes.append([a for a in range(3) if mid[lo:lo + h, a].max() <= mid[lo + h:lo + n, a].min()])
        rec(lo, h, d + 1)
        rec(lo + h, n - h, d + 1)

    rec(0, len(order), 0)
    return axes, np.array(cents)


def _tied_soup(n, seed, grid=0.125):
    """Triangles with vertices on a coarse lattice: many equal midpoints."""
    rng = np.random.default_rng(seed)
    c = np.round(rng.uniform(-2, 2, (n, 1, 3)) / grid) * grid
    d = np.round(rng.uniform(-0.3, 0.3, (n, 3, 3)) / grid) * grid
    return (c + d).reshape(-1, 9)


def test_oracle_grouping_matches_the_reference_file_top(oracle):
    from test_reference_pins import hierarchy_solid
    g = GOLD["hierarchy_test_grouping"]
    m = oracle.mc_search(*serialize(hierarchy_solid()), 0.03, 2)
    tris = m["tris"]
    order = oracle.group_triangles(tris)
    axes, cents = _signature(tris, order, g["depth"])
    assert axes == g["separating_axes"]
    assert np.abs(cents - np.array(g["centroids"])).max() < 0.02
    _check_hierarchy(tris, order)


@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 33, 1000])
def test_oracle_grouping_hierarchy(oracle, n):
    tris = _tied_soup(n, n)
    order = oracle.group_triangles(tris)
    _check_hierarchy(tris, order)
    if n <= 2:
        assert list(order) == list(np.argsort(_mids(tris)[:, 0], kind="stable"))


def test_oracle_grouping_ties_keep_input_order(oracle):
    """All midpoints equal: every sort keeps the input order, so every
    node's halves are its input halves and the order is the identity."""
    tri = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], dtype=np.float64)
    order = oracle.group_triangles(np.repeat(tri, 37, axis=0))
    assert list(order) == list(range(37))


def _indexed(tris):
    t = np.ascontiguousarray(tris, dtype=np.float64).reshape(-1, 9)
    return t.reshape(-1, 3), np.arange(3 * len(t), dtype=np.int32).reshape(-1, 3)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 3, 31, 32, 33, 64, 65, 1023, 1024, 1025, 2049, 4097, 5000, 70001, 300000])
def test_gpu_group_equals_oracle(oracle, n):
    from model3d_gb300 import GroupTriangles, Mesh
    for seed, grid in ((n, 0.125), (n + 1, 1e-3)):
        tris = _tied_soup(n, seed, grid)
        v, t = _indexed(tris)
        got = GroupTriangles(Mesh(v, t))
        assert np.array_equal(got, oracle.group_triangles(tris)), (n, grid)


@pytest.mark.gpu
def test_gpu_group_degenerate_meshes(oracle):
    from model3d_gb300 import GroupTriangles, Mesh
    flat = _tied_soup(3000, 7)
    flat[:, 2::3] = 0.25  # every z equal: the z sort's passes are all skipped
    same = np.repeat(_tied_soup(1, 8), 5000, axis=0)  # every triangle equal
    shared = _tied_soup(2000, 9)
    v = shared.reshape(-1, 3)[:500]
    t = np.random.default_rng(1).integers(0, 500, (4000, 3)).astype(np.int32)  # shared, repeated vertices
    for tris, mesh in ((flat, None), (same, None), (None, Mesh(v, t))):
        if mesh is None:
            mesh = Mesh(*_indexed(tris))
        else:
            tris = v[t].reshape(-1, 9)
        assert np.array_equal(GroupTriangles(mesh), oracle.group_triangles(tris))
    assert list(GroupTriangles(Mesh(*_indexed(same)))) == list(range(5000))
    assert len(GroupTriangles(Mesh(np.zeros((0, 3)), np.zeros((0, 3), dtype=np.int32)))) == 0


@pytest.mark.gpu
def test_gpu_group_rejects_bad_indices():
    from model3d_gb300 import GroupTriangles, MCError, Mesh
    v, t = _indexed(_tied_soup(10, 3))
    t[4, 1] = len(v)
    with pytest.raises(MCError):
        GroupTriangles(Mesh(v, t))
    t[4, 1] = -1
    with pytest.raises(MCError):
        GroupTriangles(Mesh(v, t))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_gpu_grouped_stl_of_a_search(oracle, prec, tmp_path):
    """MarchingCubesSearch + SaveGroupedSTL: the device result's grouped
    STL is the oracle's GroupTriangles of the library's triangles, encoded
    by the oracle's EncodeSTL; Mesh.SaveGroupedSTL writes the same bytes."""
    from model3d_gb300 import DeviceSolid, MarchingCubesSearch, MarchingCubesSearchGroupedSTL, canonical
    from model3d_gb300.workloads import csg_tree
    from test_reference_pins import hierarchy_solid
    for solid, delta, iters in ((hierarchy_solid(), 0.03, 2), (csg_tree(3, 24, 8), 0.01, 8)):
        ds = DeviceSolid(solid)
        mesh = MarchingCubesSearch(ds, delta, iters, precision=prec)
        soup = mesh.TriangleSoup()
        ref_tris = oracle.mc_search(*serialize(solid), delta, iters)["tris"]
        assert np.array_equal(canonical(soup), canonical(ref_tris))
        order = oracle.group_triangles(soup)
        want = oracle.encode_stl(soup[order])
        assert MarchingCubesSearchGroupedSTL(ds, delta, iters, precision=prec) == want
        p = tmp_path / "m.stl"
        mesh.SaveGroupedSTL(str(p))
        assert p.read_bytes() == want
        _check_hierarchy(soup, order)


@pytest.mark.gpu
def test_gpu_result_group_headline_mesh(oracle):
    """The 48-minus-16 CSG tree at delta 0.004 (4.17M triangles): the
    device order of the search result equals the oracle's."""
    import ctypes
    from model3d_gb300 import Context, DeviceSolid
    from model3d_gb300 import _native as N
    from model3d_gb300.workloads import csg_tree
    ctx = Context(0)
    ds = DeviceSolid(csg_tree(1, 48, 16), ctx)
    L = N.lib()
    o = N.MCOpts()
    o.precision = N.MC_PREC_FP32_FILTERED
    o.cull = 1
    V, T = ctypes.c_int64(), ctypes.c_int64()
    st = N.MCStats()
    assert L.mc_search_device(ctx.ptr, ds.ptr, 0.004, 8, ctypes.byref(o), ctypes.byref(V), ctypes.byref(T),
                              ctypes.byref(st)) == N.MC_OK
    v = np.empty((V.value, 3))
    t = np.empty((T.value, 3), dtype=np.int32)
    assert L.mc_result_copy(ctx.ptr, v.ctypes.data, t.ctypes.data) == N.MC_OK
    order = np.empty(T.value, dtype=np.int32)
    assert L.mc_result_group(ctx.ptr, order.ctypes.data) == N.MC_OK
    assert np.array_equal(order, oracle.group_triangles(v[t].reshape(-1, 9)))
