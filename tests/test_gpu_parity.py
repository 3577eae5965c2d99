"""Parity of the CUDA path with the oracle, through the C ABI.

Bit-exact: every mesh is compared as the sorted list of its triangles' nine
float64 bit patterns (triangle vertex order kept), for both precision modes
(FP64 and FP32-filtered) and with tile culling on and off.
"""
import numpy as np
import pytest

from model3d_gb300 import (CacheSolidBounds, Capsule, Contains, Cylinder, DeviceSolid,
                           GroupedTrianglesToCollider, IntersectedSolid, JoinedSolid,
                           JoinedTransform, MarchingCubesSearch, MCError, MeshToCollider,
                           NewColliderSolid, NotLowerable, Rect, Rotation, Scale, Sphere,
                           SubtractedSolid, Torus, TransformSolid, Translate, VecScale, XYZ,
                           canonical, serialize)
from model3d_gb300 import _native as N
from model3d_gb300.workloads import (SplitMix64, box_triangles, csg_tree, displaced_icosphere,
                                     random_primitive)

pytestmark = pytest.mark.gpu

MODES = [("fp64", True), ("fp32", True), ("fp32", False)]


def _same(mesh, ref):
    a = canonical(mesh.TriangleSoup())
    b = canonical(ref["tris"])
    assert a.shape == b.shape, f"triangle count {len(a)} != oracle {len(b)}"
    diff = np.nonzero((a != b).any(1))[0]
    assert len(diff) == 0, f"{len(diff)} triangles differ, first at {diff[:3]}"


def _check(oracle, solid, delta, iters, modes=MODES):
    nodes, sets = serialize(solid)
    ref = oracle.mc_search(nodes, sets, delta, iters)
    ds = DeviceSolid(solid)
    for prec, cull in modes:
        m = MarchingCubesSearch(ds, delta, iters, precision=prec, cull=cull)
        _same(m, ref)
        assert m.stats["vertices"] == ref["n_vertices"]
        assert (m.stats["nx"], m.stats["ny"], m.stats["nz"]) == (ref["nx"], ref["ny"], ref["nz"])
    return m


def test_sphere_full_size(oracle):
    """Plain sphere at delta 0.01 (202^3 corners), iters 8."""
    m = _check(oracle, Sphere(XYZ(0, 0, 0), 1.0), 0.01, 8)
    assert m.stats["corners"] == 202 ** 3


@pytest.mark.parametrize("iters", [0, 1, 2, 8])
def test_sphere_iters(oracle, iters):
    _check(oracle, Sphere(XYZ(0.1, 0.3, -0.2), 0.7), 0.05, iters)


@pytest.mark.parametrize("seed", range(6))
def test_single_primitives(oracle, seed):
    rng = SplitMix64(1000 + seed)
    for _ in range(4):
        _check(oracle, random_primitive(rng), 0.02, 8)


def test_reference_benchmark_cylinder(oracle):
    """BenchmarkMarchingCubes' cylinder (mc_test.go:98-106) at delta 0.025."""
    _check(oracle, Cylinder(XYZ(1, 2, 3), XYZ(3, 1, 4), 0.5), 0.025, 8)


@pytest.mark.parametrize("seed", range(4))
def test_csg_trees(oracle, seed):
    _check(oracle, csg_tree(seed, 24, 8), 0.015, 8)


def test_csg_config_shape_reduced_delta(oracle):
    """The 48-minus-16 CSG tree of the headline workload at delta 0.01."""
    _check(oracle, csg_tree(1, 48, 16), 0.01, 8)


def test_torus(oracle):
    _check(oracle, Torus(XYZ(0.1, -0.2, 0.3), XYZ(0.3, 1, -0.2), 0.6, 0.2), 0.02, 8)
    _check(oracle, Torus(XYZ(0, 0, 0), XYZ(0, 0, 1), 0.5, 0.25), 0.02, 8)


def test_transforms_and_combinators(oracle):
    base = SubtractedSolid(Cylinder(XYZ(0, 0, -0.5), XYZ(0.2, 0.1, 0.5), 0.4),
                           Sphere(XYZ(0.1, 0, 0.3), 0.25))
    solids = [
        TransformSolid(Translate(XYZ(0.3, -0.2, 0.1)), base),
        TransformSolid(Scale(1.7), base),
        TransformSolid(VecScale(XYZ(1.3, -0.7, 0.9)), base),
        TransformSolid(Rotation(XYZ(0, 0.6, 0.8), 0.7), base),
        TransformSolid(JoinedTransform([Scale(1.2), Rotation(XYZ(1, 0, 0), 0.3),
                                        Translate(XYZ(0.1, 0.2, 0.3))]), base),
        IntersectedSolid([Sphere(XYZ(0, 0, 0), 1), Rect(XYZ(-0.5, -2, -2), XYZ(2, 0.4, 2))]),
        JoinedSolid([random_primitive(SplitMix64(i)) for i in range(10)]).Optimize(),
        CacheSolidBounds(TransformSolid(Translate(XYZ(1, 0, 0)),
                                        TransformSolid(Scale(0.5), base))),
    ]
    for s in solids:
        _check(oracle, s, 0.02, 8)


def test_collider_icosphere(oracle):
    s = NewColliderSolid(MeshToCollider(displaced_icosphere(8)))
    _check(oracle, s, 0.03, 8)


def test_collider_boxes(oracle):
    """The two-box collider of mc_test.go:51-60 / BenchmarkMarchingCubes."""
    tris = np.concatenate([box_triangles((-1, -1, -1), (0, 0, 0)), box_triangles((0.1, 0, 0), (1, 1, 1))])
    _check(oracle, NewColliderSolid(MeshToCollider(tris)), 0.1, 8)
    _check(oracle, NewColliderSolid(GroupedTrianglesToCollider(tris)), 0.05, 8)


def test_collider_single_triangle_and_csg_mix(oracle):
    tris = displaced_icosphere(3)
    col = NewColliderSolid(MeshToCollider(tris))
    s = SubtractedSolid(col, Sphere(XYZ(0.5, 0.5, 0.5), 0.5))
    _check(oracle, s, 0.04, 8)


def test_empty_and_degenerate(oracle):
    # smaller than one grid cell: no corner inside, empty mesh
    m = _check(oracle, Sphere(XYZ(0.0123, 0.0456, 0.0789), 0.001), 0.1, 8)
    assert m.NumTriangles() == 0
    # flat box (zero extent in z) and a zero-length capsule
    _check(oracle, Rect(XYZ(-0.3, -0.2, 0.1), XYZ(0.4, 0.5, 0.1)), 0.05, 8)
    _check(oracle, Capsule(XYZ(0.1, 0.1, 0.1), XYZ(0.1, 0.1, 0.1), 0.3), 0.05, 8)


def test_border_inside_raises(oracle):
    nodes, sets = serialize(Sphere(XYZ(0, 0, 0), 1.0))
    s = Sphere(XYZ(0, 0, 0), 1.0)

    class Lying(Sphere):
        def Min(self):
            return XYZ(-0.5, -0.5, -0.5)

        def Max(self):
            return XYZ(0.5, 0.5, 0.5)

    with pytest.raises(MCError) as e:
        MarchingCubesSearch(Lying(XYZ(0, 0, 0), 1.0), 0.1, 8)
    assert e.value.status == N.MC_ERR_BOUNDS_INSIDE
    assert "solid is true outside of bounds" in str(e.value)
    with pytest.raises(Exception):
        oracle.mc_search(*serialize(Lying(XYZ(0, 0, 0), 1.0)), 0.1, 8)


def test_invalid_bounds_raise():
    class Inverted(Sphere):
        def Max(self):
            return XYZ(-2, 0, 0)

    with pytest.raises(MCError) as e:
        MarchingCubesSearch(Inverted(XYZ(0, 0, 0), 1.0), 0.1, 8)
    assert e.value.status == N.MC_ERR_INVALID_BOUNDS


def test_unlowerable_solid_raises():
    class Custom:
        def Min(self):
            return XYZ(0, 0, 0)

        def Max(self):
            return XYZ(1, 1, 1)

    with pytest.raises(NotLowerable):
        MarchingCubesSearch(Custom(), 0.1, 8)


def _near_surface_points(solid, n, rng):
    mn, mx = np.array(solid.Min().Array()), np.array(solid.Max().Array())
    pad = 0.1 * (mx - mn + 1e-3)
    p = mn - pad + (mx - mn + 2 * pad) * rng.random((n, 3))
    return p


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_contains_parity(oracle, prec):
    """Solid.Contains at random points, incl. points on grid values of the
    reference spacer and points nudged by one ulp off a surface."""
    rng = np.random.default_rng(7)
    solids = [random_primitive(SplitMix64(50 + i)) for i in range(16)]
    solids += [Torus(XYZ(0.1, -0.2, 0.3), XYZ(0.3, 1, -0.2), 0.6, 0.2), csg_tree(3, 12, 4)]
    for s in solids:
        nodes, sets = serialize(s)
        pts = _near_surface_points(s, 20000, rng)
        ref, _ = oracle.contains(nodes, sets, pts)
        got = Contains(s, pts, precision=prec)
        assert (got == ref).all()
    # points exactly on a sphere surface and one ulp either side
    s = Sphere(XYZ(0.25, -0.5, 0.125), 0.75)
    d = rng.normal(size=(5000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p = np.array(s.Center.Array()) + 0.75 * d
    pts = np.concatenate([p, np.nextafter(p, np.inf), np.nextafter(p, -np.inf)])
    ref, _ = oracle.contains(*serialize(s), pts)
    assert (Contains(s, pts, precision=prec) == ref).all()


def test_filter_escalation_rate_is_small():
    for s in (csg_tree(1, 48, 16), Torus(XYZ(0.1, -0.2, 0.3), XYZ(0.3, 1, -0.2), 0.6, 0.2)):
        st = MarchingCubesSearch(s, 0.01, 8, precision="fp32").stats
        assert st["leaf_evals"] > 0
        assert st["escalations"] <= 0.01 * st["leaf_evals"]


def _closed_oriented(tris):
    e = tris[:, [0, 1, 1, 2, 2, 0]].reshape(-1, 2).astype(np.int64)
    V = int(e.max()) + 1 if len(e) else 1
    k = e[:, 0] * V + e[:, 1]
    r = e[:, 1] * V + e[:, 0]
    assert len(np.unique(k)) == len(k)
    assert np.array_equal(np.sort(k), np.sort(r))


def test_headline_csg_full_size_properties():
    """The headline workload at full size (delta 0.004): the FP32-filtered and
    FP64 meshes are bit-identical, closed and consistently oriented."""
    s = csg_tree(1, 48, 16)
    ds = DeviceSolid(s)
    a = MarchingCubesSearch(ds, 0.004, 8, precision="fp32")
    b = MarchingCubesSearch(ds, 0.004, 8, precision="fp64")
    assert a.stats["corners"] > 1.0e8
    assert np.array_equal(canonical(a.TriangleSoup()), canonical(b.TriangleSoup()))
    _closed_oriented(a.triangles)


def test_collider_fp32_filter_larger_mesh(oracle):
    """32k-triangle displaced icosphere: FP32-filtered box and triangle tests
    with float64 escalation give the float64 mesh."""
    s = NewColliderSolid(MeshToCollider(displaced_icosphere(40)))
    m = _check(oracle, s, 0.02, 8)
    assert m.stats["bvh_nodes"] > 0 and m.stats["bvh_tris"] > 0


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_collider_contains_parity(oracle, prec):
    rng = np.random.default_rng(17)
    tris = displaced_icosphere(12)
    s = NewColliderSolid(MeshToCollider(tris))
    nodes, sets = serialize(s)
    # random points, and points on the mesh's vertices and edges (hardest cases)
    pts = [rng.uniform(-1.3, 1.3, size=(20000, 3))]
    t = tris.reshape(-1, 3, 3)
    w = rng.dirichlet([1, 1, 1], size=len(t))
    pts.append((t * w[:, :, None]).sum(1))
    pts.append(t[:, 0] * 0.5 + t[:, 1] * 0.5)
    pts = np.concatenate(pts)
    ref, _ = oracle.contains(nodes, sets, pts)
    assert (Contains(s, pts, precision=prec) == ref).all()


RAY_D = np.array([0.5224892708603626, 0.10494477243214506, 0.43558938446126527])


def _grazing_mesh(rng):
    """Triangles that stress the ray grid: a displaced icosphere, slivers
    nearly parallel to the containment ray, tiny triangles and a duplicate."""
    tris = [displaced_icosphere(5)]
    d = RAY_D / np.linalg.norm(RAY_D)
    for k in range(40):
        p0 = rng.uniform(-0.8, 0.8, 3)
        side = np.cross(d, rng.normal(size=3))
        side /= np.linalg.norm(side)
        tilt = 10.0 ** rng.uniform(-7.5, -2)  # angle off the ray direction
        p1 = p0 + 0.3 * (d + tilt * np.cross(d, side))
        p2 = p0 + 0.2 * side
        tris.append(np.concatenate([p0, p1, p2])[None])
    for k in range(40):
        p0 = rng.uniform(-0.8, 0.8, 3)
        tris.append(np.concatenate([p0, p0 + 1e-6 * rng.normal(size=3), p0 + 1e-6 * rng.normal(size=3)])[None])
    t = np.concatenate(tris)
    return np.concatenate([t, t[:3]])


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_collider_grazing_rays(oracle, prec):
    """Rays aimed exactly at triangle vertices, edge points and sliver
    triangles nearly parallel to the ray: the ray-grid candidates and the
    parent-box test reproduce the reference's traversal count."""
    rng = np.random.default_rng(23)
    tris = _grazing_mesh(rng)
    s = NewColliderSolid(MeshToCollider(tris))
    nodes, sets = serialize(s)
    t = tris.reshape(-1, 3, 3)
    targets = [t.reshape(-1, 3),                                   # vertices
               0.5 * (t[:, 0] + t[:, 1]), 0.5 * (t[:, 1] + t[:, 2]),  # edge midpoints
               (t * rng.dirichlet([1, 1, 1], size=len(t))[:, :, None]).sum(1)]
    targets = np.concatenate(targets)
    s_back = rng.uniform(0.0, 0.6, size=(len(targets), 1))
    pts = targets - s_back * RAY_D[None]
    pts = np.concatenate([pts, np.nextafter(pts, np.inf), np.nextafter(pts, -np.inf), targets])
    ref, _ = oracle.contains(nodes, sets, pts)
    got = Contains(s, pts, precision=prec)
    bad = np.nonzero(got != ref)[0]
    assert len(bad) == 0, f"{len(bad)} of {len(pts)} differ, first {pts[bad[:3]]}"
    _check(oracle, s, 0.05, 8, modes=[(prec, True)])


@pytest.mark.parametrize("iters", [0, 3, 8])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_marching_cubes_interior(oracle, iters, prec):
    """MarchingCubesInterior (mc.go:55-60): same mesh as the oracle and, per
    vertex, the oracle's interior point, bit for bit; every interior point is
    inside the solid."""
    from model3d_gb300 import MarchingCubesInterior
    solids = [Sphere(XYZ(0.1, 0.0, -0.1), 0.8), csg_tree(2, 12, 4),
              TransformSolid(Rotation(XYZ(0.3, 1, 0.2), 0.5), Cylinder(XYZ(0, 0, -0.4), XYZ(0.1, 0, 0.5), 0.3))]
    for s in solids:
        nodes, sets = serialize(s)
        ref = oracle.mc_search(nodes, sets, 0.04, iters, interior=True)
        mesh, inner = MarchingCubesInterior(s, 0.04, iters, precision=prec)
        _same(mesh, ref)
        want = {}
        for c, ip in zip(ref["tris"].reshape(-1, 3).view(np.uint64), ref["interior"].reshape(-1, 3)):
            want[c.tobytes()] = ip
        got_v = mesh.vertices.view(np.uint64)
        for i in range(len(mesh.vertices)):
            assert np.array_equal(want[got_v[i].tobytes()].view(np.uint64), inner[i].view(np.uint64))
        assert Contains(s, inner, precision="fp64").all()


def test_interior_points_of_a_chunked_search(oracle):
    """A mesh large enough (>= 2^17 vertices) that mc_search runs the search
    in vertex ranges whose read-back overlaps the next range: vertices and
    interior points still match the oracle's."""
    from model3d_gb300 import MarchingCubesInterior
    s = Sphere(XYZ(0.05, -0.02, 0.01), 1.0)
    ref = oracle.mc_search(*serialize(s), 0.01, 8, interior=True)
    mesh, inner = MarchingCubesInterior(s, 0.01, 8)
    assert len(mesh.vertices) >= 1 << 17
    _same(mesh, ref)
    want = dict(zip(map(bytes, ref["tris"].reshape(-1, 3).view(np.uint64)),
                    map(bytes, ref["interior"].reshape(-1, 3).view(np.uint64))))
    got = [want[bytes(v)] for v in mesh.vertices.view(np.uint64)]
    assert got == list(map(bytes, inner.view(np.uint64)))


def test_marching_cubes_conj(oracle):
    """MarchingCubesConj (mc.go:66-71): search in the transformed space, then
    the inverse transform on the device; equals the oracle's mesh mapped by
    JoinedTransform(xforms).Inverse()."""
    from model3d_gb300 import JoinedTransform, MarchingCubesConj
    from model3d_gb300.solids import transform_records
    base = SubtractedSolid(Capsule(XYZ(-0.4, 0.1, 0), XYZ(0.5, -0.2, 0.3), 0.35), Sphere(XYZ(0.2, 0.1, 0.2), 0.3))
    for xforms in ([Scale(1.3), Rotation(XYZ(0.2, 1, 0.3), 0.4), Translate(XYZ(0.1, -0.2, 0.05))],
                   [VecScale(XYZ(1.5, 0.8, 1.1))], [Translate(XYZ(0.25, 0, -0.5))]):
        joined = JoinedTransform(xforms)
        for prec in ("fp64", "fp32"):
            mesh = MarchingCubesConj(base, 0.03, 8, *xforms, precision=prec)
            ref = oracle.mc_search(*serialize(TransformSolid(joined, base)), 0.03, 8)
            back = oracle.apply_transform(transform_records(joined), ref["tris"].reshape(-1, 3), inverse=True)
            _same(mesh, {"tris": back.reshape(-1, 9)})


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_stl_encoding(oracle, prec):
    """EncodeSTL on the device (mc_result_stl): header and the multiset of
    50-byte records equal the oracle's encoding of the oracle's mesh."""
    from model3d_gb300 import MarchingCubesSearchSTL
    for s, d in ((csg_tree(4, 10, 3), 0.02), (NewColliderSolid(MeshToCollider(displaced_icosphere(6))), 0.05)):
        nodes, sets = serialize(s)
        ref = oracle.encode_stl(oracle.mc_search(nodes, sets, d, 8)["tris"])
        got = MarchingCubesSearchSTL(s, d, 8, precision=prec)
        assert len(got) == len(ref) and got[:84] == ref[:84]
        def recs(b):
            a = np.frombuffer(b[84:], dtype=np.uint8).reshape(-1, 50)
            return a[np.lexsort(a.T[::-1])]
        assert np.array_equal(recs(got), recs(ref))


def test_filter_and_c2f_match_reference_tests(oracle):
    """The properties of mc_test.go:44-94: MarchingCubesFilter with a
    collider's RectCollision equals MarchingCubes, MarchingCubesC2F equals
    MarchingCubesSearch (sphere and two-box solids), here against the
    oracle's MarchingCubes / MarchingCubesSearch."""
    from model3d_gb300 import MarchingCubesC2F, MarchingCubesFilter, MarchingCubesSearchFilter
    from model3d_gb300.workloads import icosphere_triangles
    ico = icosphere_triangles(6).reshape(-1, 3, 3) + np.array([0.1, 0.3, -0.2])
    col = NewColliderSolid(MeshToCollider(ico.reshape(-1, 9)))
    boxes = np.concatenate([box_triangles((-1, -1, -1), (0, 0, 0)), box_triangles((0.1, 0, 0), (1, 1, 1))])
    bcol = NewColliderSolid(MeshToCollider(boxes))
    for s in (col, bcol):
        ref = oracle.mc_search(*serialize(s), 0.1, 0)
        _same(MarchingCubesFilter(s, lambda r: True, 0.1), ref)
        ref8 = oracle.mc_search(*serialize(s), 0.1, 8)
        _same(MarchingCubesSearchFilter(s, lambda r: True, 0.1, 8), ref8)
    sph = Sphere(XYZ(0.1, 0.3, -0.2), 1.0)
    _same(MarchingCubesC2F(sph, 0.1, 0.05, 0, 8), oracle.mc_search(*serialize(sph), 0.05, 8))
    boxes2 = np.concatenate([box_triangles((-1, -1, -1), (0, 0, 0)), box_triangles((0.3, 0, 0), (1, 1, 1))])
    b2 = NewColliderSolid(MeshToCollider(boxes2))
    _same(MarchingCubesC2F(b2, 0.2, 0.1, 0, 8), oracle.mc_search(*serialize(b2), 0.1, 8))
    with pytest.raises(MCError):
        MarchingCubesC2F(sph, 0.05, 0.1, 0, 8)


def test_grid_at_the_corner_limit():
    """A grid just under the 2^31-corner limit meshes (FP32-filtered and FP64
    identical; Euler characteristic 2 of a sphere); one just over it is
    refused with MC_ERR_GRID, not truncated."""
    s = Sphere(XYZ(0, 0, 0), 1.0)
    a = MarchingCubesSearch(s, 2.0 / 1275, 2, precision="fp32")
    assert 1.9e9 < a.stats["corners"] < 2 ** 31
    b = MarchingCubesSearch(s, 2.0 / 1275, 2, precision="fp64")
    assert np.array_equal(a.vertices.view(np.uint64), b.vertices.view(np.uint64))
    assert np.array_equal(a.triangles, b.triangles)
    V, T = len(a.vertices), len(a.triangles)
    assert V - T // 2 == 2  # closed triangle mesh of genus 0: V - E + F = V - 3T/2 + T
    with pytest.raises(MCError) as e:
        MarchingCubesSearch(s, 2.0 / 1295, 2)
    assert e.value.status == N.MC_ERR_GRID


def test_long_thin_grid_near_the_key_limit(oracle):
    """An x-extent of about 600k grid values (keys hold 20-bit indices) with a
    solid thinner than one cell in y and z."""
    s = Rect(XYZ(-1, 0, 0), XYZ(1, 1.5e-6, 1.5e-6))
    _check(oracle, s, 2.0 / 600000, 8, modes=[("fp32", True), ("fp64", True)])


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_torus_contains_near_surface_and_axis(oracle, prec):
    """The FP32 torus filter: points on the tube surface and one ulp off it,
    points on and next to the symmetry axis (the reference's on == 0 case),
    and random points; all equal the oracle."""
    rng = np.random.default_rng(31)
    for center, axis, R, r in ((XYZ(0.1, -0.2, 0.3), XYZ(0.3, 1, -0.2), 0.6, 0.2),
                               (XYZ(0, 0, 0), XYZ(0, 0, 1), 0.5, 0.25),
                               (XYZ(0.2, 0.1, 0), XYZ(1, 1, 1), 0.3, 0.35)):
        s = Torus(center, axis, R, r)
        c = np.array(center.Array())
        a = np.array(axis.Array()) / np.linalg.norm(axis.Array())
        u = np.cross(a, [0.3, 0.5, 0.7])
        u /= np.linalg.norm(u)
        v = np.cross(a, u)
        th, ph = rng.uniform(0, 2 * np.pi, (2, 4000))
        ring = c + R * (np.cos(th)[:, None] * u + np.sin(th)[:, None] * v)
        surf = ring + r * (np.cos(ph)[:, None] * (ring - c) / R + np.sin(ph)[:, None] * a)
        on_axis = c + rng.uniform(-1, 1, (500, 1)) * a
        pts = np.concatenate([surf, np.nextafter(surf, np.inf), np.nextafter(surf, -np.inf), on_axis,
                              on_axis + 1e-9 * u, rng.uniform(-1.5, 1.5, (4000, 3)) + c])
        ref, _ = oracle.contains(*serialize(s), pts)
        assert (Contains(s, pts, precision=prec) == ref).all()


def test_result_entry_errors():
    """Misuse of the result entry points returns statuses, not crashes."""
    import ctypes
    from model3d_gb300 import Context, DeviceSolid, MarchingCubesSearch
    ctx = Context(0)
    L = N.lib()
    ds = DeviceSolid(Sphere(XYZ(0, 0, 0), 0.5), ctx)
    MarchingCubesSearch(ds, 0.1, 8, ctx=ctx)   # no interior points requested
    buf = np.zeros((10, 3))
    assert L.mc_result_interior_copy(ctx.ptr, buf.ctypes.data) == N.MC_ERR_ARG
    n = ctypes.c_size_t()
    assert L.mc_result_stl(ctx.ptr, None, 0, ctypes.byref(n)) == N.MC_OK and n.value > 84
    small = np.zeros(16, dtype=np.uint8)
    assert L.mc_result_stl(ctx.ptr, small.ctypes.data, 16, ctypes.byref(n)) == N.MC_ERR_ARG
    bad = np.zeros(1, dtype=serialize(Sphere(XYZ(0, 0, 0), 1.0))[0].dtype)
    bad[0]["kind"] = 99
    assert L.mc_result_transform(ctx.ptr, bad.ctypes.data, 1, 0) == N.MC_ERR_BAD_PROGRAM
