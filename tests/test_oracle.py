"""Pins of the oracle (the CPU restatement of the reference path) against the
reference's own tests and known answers.  CPU only.

The reference ships no golden meshes, so these restate its property tests:
  mc_test.go:9-25        lookup table deterministic (and covering all 256 cases)
  mc_test.go:27-42       random solids give valid (closed, oriented) meshes
  measurements_test.go   sphere volume within 1e-2 at delta = 0.02
  shapes_test.go:98-118  no point just outside a solid's bounds is contained
  collisions_test.go:22  collider ray counts equal brute force over triangles
"""
import math

import numpy as np
import pytest

from model3d_gb300 import (Capsule, Cylinder, IntersectedSolid, JoinedSolid, JoinedTransform,
                           MeshToCollider, NewColliderSolid, Rect, Rotation, Scale, Sphere, Torus,
                           TransformSolid, Translate, VecScale, XYZ, serialize)
from model3d_gb300.workloads import SplitMix64, csg_tree, displaced_icosphere, random_primitive


def test_table_deterministic_and_complete(oracle):
    counts, tris, conflicts, covered = oracle.case_table()
    assert conflicts == 0, "two base cases map to one case: Go map order would matter"
    assert covered == 256
    rots, n = oracle.rotations()
    assert n == 24
    assert list(rots[0]) == list(range(8))
    assert all(tuple(rots[i]) < tuple(rots[i + 1]) for i in range(23))
    for _ in range(3):
        c2, t2, _, _ = oracle.case_table()
        assert (c2 == counts).all() and (t2 == tris).all()
    assert counts[0] == 0 and counts[255] == 0 and counts.max() == 5
    # every triangle joins three distinct cube edges
    for c in range(256):
        for t in range(counts[c]):
            e = tris[c, t]
            for k in range(3):
                a, b = e[2 * k], e[2 * k + 1]
                assert bin(a ^ b).count("1") == 1
                assert ((c >> a) & 1) != ((c >> b) & 1), "edge must cross the surface"


def _mc_from_bits(bits, counts, tris):
    """Cube loop of MarchingCubes over a boolean corner grid [z][y][x],
    vertices as edge keys; used to check the table on arbitrary bit grids."""
    nz, ny, nx = bits.shape
    out = []
    for z in range(nz - 1):
        for y in range(ny - 1):
            for x in range(nx - 1):
                k = 0
                for i in range(8):
                    dx, dy, dz = i & 1, (i >> 1) & 1, i >> 2
                    k |= int(bits[z + dz, y + dy, x + dx]) << i
                for t in range(counts[k]):
                    tri = []
                    for v in range(3):
                        a, b = tris[k, t, 2 * v], tris[k, t, 2 * v + 1]
                        pa = (x + (a & 1), y + ((a >> 1) & 1), z + (a >> 2))
                        pb = (x + (b & 1), y + ((b >> 1) & 1), z + (b >> 2))
                        tri.append(tuple(sorted([pa, pb])))
                    out.append(tri)
    return out


def _assert_closed_oriented(tris):
    edges = {}
    for t in tris:
        assert len(set(t)) == 3
        for i in range(3):
            e = (t[i], t[(i + 1) % 3])
            edges[e] = edges.get(e, 0) + 1
    for (a, b), n in edges.items():
        assert n == 1, "directed edge used twice (flipped normals)"
        assert edges.get((b, a), 0) == 1, "mesh not closed"


def test_table_gives_manifold_meshes_on_random_solids(oracle):
    """mc_test.go:27-42: 30 random solids (each corner inside with p=1/4)."""
    counts, tris, _, _ = oracle.case_table()
    rng = np.random.default_rng(1337)
    for _ in range(30):
        bits = rng.random((9, 9, 9)) < 0.25
        bits[0, :, :] = bits[-1, :, :] = bits[:, 0, :] = bits[:, -1, :] = False
        bits[:, :, 0] = bits[:, :, -1] = False
        _assert_closed_oriented(_mc_from_bits(bits, counts, tris))


def test_spacer_known_answer(oracle):
    """newSquareSpacer for the unit sphere at delta 0.01: 202 values ending at
    1.0000000000000013 (the nominal max+delta point is dropped)."""
    xs = oracle.spacer_axis(-1.0, 1.0, 0.01)
    assert len(xs) == 202
    assert xs[0] == -1.01
    assert xs[-1] == 1.0000000000000013
    x = -1.0 - 0.01
    for v in xs:
        assert v == x
        x += 0.01


def _soup_edges(soup):
    t = [tuple(tuple(r) for r in tri.reshape(3, 3)) for tri in soup]
    return t


def test_sphere_volume(oracle):
    """measurements_test.go: |volume - 4/3 pi r^3| <= 1e-2 at delta 0.02."""
    rng = np.random.default_rng(5)
    for _ in range(3):
        s = Sphere(XYZ(*rng.normal(size=3)), rng.random() * 1.5 + 0.1)
        nodes, sets = serialize(s)
        m = oracle.mc_search(nodes, sets, 0.02, 8)
        t = m["tris"].reshape(-1, 3, 3)
        vol = abs(np.linalg.det(t).sum() / 6)
        assert abs(vol - 4 / 3 * math.pi * s.Radius ** 3) <= 1e-2


def test_search_vertices_lie_on_the_surface(oracle):
    """The SDF tests' solid (sdf_test.go:189-196, the torus of
    TestMeshSDFVertices / TestMeshSDFConsistency at delta 0.02, iters 8): every
    searched vertex lies within the last bisection step of the true surface,
    |SDF| <= delta * 2^-8 (a crossing is bracketed on its edge to 2^-iters of
    the edge, and the SDF is 1-Lipschitz); a sphere and a capsule likewise."""
    ax = XYZ(1, 2, -0.5).Normalize()
    torus = Torus(XYZ(0, 0, 0), ax, 0.7, 0.2)
    a = np.array(ax.Array())

    def torus_sdf(v):
        h = v @ a
        ring = np.linalg.norm(v - h[:, None] * a, axis=1)
        return 0.2 - np.sqrt((ring - 0.7) ** 2 + h ** 2)

    def sphere_sdf(v):
        return 0.55 - np.linalg.norm(v - np.array([0.1, -0.2, 0.05]), axis=1)

    p1, p2 = np.array([-0.3, 0.1, 0.0]), np.array([0.4, -0.2, 0.3])

    def capsule_sdf(v):
        d = p2 - p1
        t = np.clip((v - p1) @ d / (d @ d), 0, 1)
        return 0.25 - np.linalg.norm(v - (p1 + t[:, None] * d), axis=1)

    for s, sdf in ((torus, torus_sdf), (Sphere(XYZ(0.1, -0.2, 0.05), 0.55), sphere_sdf),
                   (Capsule(XYZ(*p1), XYZ(*p2), 0.25), capsule_sdf)):
        m = oracle.mc_search(*serialize(s), 0.02, 8)
        v = m["tris"].reshape(-1, 3)
        assert np.abs(sdf(v)).max() <= 0.02 / 256 * 1.001


def test_search_mesh_is_closed(oracle):
    for seed in range(3):
        s = csg_tree(seed, 6, 2)
        nodes, sets = serialize(s)
        m = oracle.mc_search(nodes, sets, 0.05, 4)
        tris = [tuple(tuple(v) for v in t.reshape(3, 3)) for t in m["tris"]]
        _assert_closed_oriented(tris)


def _random_solids():
    rng = SplitMix64(99)
    out = [random_primitive(rng) for _ in range(12)]
    out.append(Torus(XYZ(0.1, -0.2, 0.3), XYZ(0.3, 1, -0.2), 0.6, 0.2))
    out.append(Torus(XYZ(0, 0, 0), XYZ(0, 0, 1), 0.5, 0.1))
    return out


def test_bounds_never_exceeded(oracle):
    """shapes_test.go:98-118 testSolidBounds, per primitive kind."""
    rng = np.random.default_rng(3)
    for s in _random_solids():
        nodes, sets = serialize(s)
        mn, mx = np.array(s.Min().Array()), np.array(s.Max().Array())
        pts = []
        for _ in range(2000):
            ax = rng.integers(3)
            p = mn + (mx - mn) * rng.random(3)
            p[ax] = mn[ax] - 1e-4 if rng.integers(2) == 0 else mx[ax] + 1e-4
            pts.append(p)
        inside, _ = oracle.contains(nodes, sets, np.array(pts))
        assert not inside.any()


def test_python_bounds_match_oracle(oracle):
    solids = _random_solids()
    solids.append(csg_tree(5, 10, 4))
    solids.append(IntersectedSolid([Sphere(XYZ(0, 0, 0), 1), Rect(XYZ(-0.5, -2, -2), XYZ(2, 2, 2))]))
    solids.append(TransformSolid(JoinedTransform([Scale(1.5), Rotation(XYZ(0, 0.6, 0.8), 0.7),
                                                  Translate(XYZ(0.1, 0.2, 0.3))]),
                                 Cylinder(XYZ(0, 0, -0.5), XYZ(0.2, 0.1, 0.5), 0.3)))
    solids.append(TransformSolid(VecScale(XYZ(1, -2, 0.5)), Capsule(XYZ(0, 0, 0), XYZ(1, 0, 0), 0.2)))
    solids.append(JoinedSolid([random_primitive(SplitMix64(i)) for i in range(9)]).Optimize())
    tris = displaced_icosphere(3)
    solids.append(NewColliderSolid(MeshToCollider(tris)))
    for s in solids:
        nodes, sets = serialize(s)
        mn, mx = oracle.bounds(nodes, sets)
        assert (mn.view(np.uint64) == np.array(s.Min().Array()).view(np.uint64)).all()
        assert (mx.view(np.uint64) == np.array(s.Max().Array()).view(np.uint64)).all()


def _brute_force_parity(tris, pts):
    """Triangle.rayCollision over every triangle (primitives.go:207-249),
    float64 in the reference operation order, vectorised over triangles."""
    D = np.array([0.5224892708603626, 0.10494477243214506, 0.43558938446126527])
    T = tris.reshape(-1, 3, 3)
    t0, t1, t2 = T[:, 0], T[:, 1], T[:, 2]

    def cross(a, b):
        return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                         a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                         a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)

    def dot(a, b):
        return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]

    def normalize(a):
        n = np.sqrt(a[..., 0] * a[..., 0] + a[..., 1] * a[..., 1] + a[..., 2] * a[..., 2])
        return a * (1 / n)[..., None]

    v1, v2 = t1 - t0, t2 - t0
    d = dot(normalize(cross(v1, v2)), normalize(D))
    parallel = (d < 1e-8) & (d > -1e-8)
    c1 = cross(np.broadcast_to(D, v2.shape), v2)
    det = dot(c1, v1)
    with np.errstate(all="ignore"):
        inv = 1 / det
    out = []
    for p in pts:
        o = p[None] - t0
        with np.errstate(all="ignore"):
            b1 = inv * dot(o, c1)
            c2 = cross(o, v1)
            b2 = inv * dot(np.broadcast_to(D, c2.shape), c2)
            sc = inv * dot(v2, c2)
        hit = ~parallel & (det != 0) & ~((b1 < 0) | (b1 > 1)) & ~((b2 < 0) | (b1 + b2 > 1)) & ~(sc < 0)
        out.append(hit.sum() % 2 == 1)
    return np.array(out)


def test_collider_matches_brute_force(oracle):
    """collisions_test.go:22-76: the BVH collider counts what brute force counts."""
    tris = displaced_icosphere(4)
    s = NewColliderSolid(MeshToCollider(tris))
    nodes, sets = serialize(s)
    rng = np.random.default_rng(11)
    pts = rng.normal(size=(400, 3)) * 0.7
    inside, counts = oracle.contains(nodes, sets, pts)
    mn, mx = np.array(s.Min().Array()), np.array(s.Max().Array())
    inb = ((pts >= mn) & (pts <= mx)).all(1)
    brute = _brute_force_parity(tris, pts) & inb
    assert (inside == brute).all()
    assert counts[1] > 0 and counts[2] > 0


def test_oracle_threads_deterministic(oracle):
    from model3d_gb300 import canonical
    s = csg_tree(2, 8, 3)
    nodes, sets = serialize(s)
    a = oracle.mc_search(nodes, sets, 0.03, 8, threads=1)
    b = oracle.mc_search(nodes, sets, 0.03, 8, threads=8)
    assert (canonical(a["tris"]) == canonical(b["tris"])).all()


def test_border_inside_panics(oracle):
    """FetchZ panics "solid is true outside of bounds" (mc.go:687-689) when the
    caller's Min()/Max() are smaller than the set the solid contains."""
    nodes, sets = serialize(Sphere(XYZ(0, 0, 0), 1.0))
    nodes["min"][0] = [-0.5, -0.5, -0.5]
    nodes["max"][0] = [0.5, 0.5, 0.5]
    with pytest.raises(oracle.OracleError) as e:
        oracle.mc_search(nodes, sets, 0.1, 8)
    assert e.value.status == 2


def test_invalid_bounds_panic(oracle):
    """validateBounds (bounder.go:48-52): inverted or non-finite bounds."""
    nodes, sets = serialize(Sphere(XYZ(0, 0, 0), 1.0))
    nodes["max"][0][0] = -2.0
    with pytest.raises(oracle.OracleError) as e:
        oracle.mc_search(nodes, sets, 0.1, 8)
    assert e.value.status == 1


def test_coord_min_max_follow_go_math():
    """Coord3D.Min/Max take a strict comparison first; on ties (+0 / -0), NaN
    and infinities they must still give math.Min / math.Max's answers
    (coords.go:440-448)."""
    from model3d_gb300.geometry import Coord3D, go_max, go_min
    vals = [0.0, -0.0, 1.0, -1.0, math.inf, -math.inf, math.nan, 2.5, -3.0, 5e-324]

    def same(a, b):
        return (math.isnan(a) and math.isnan(b)) or (a == b and math.copysign(1, a) == math.copysign(1, b))

    for x in vals:
        for y in vals:
            a, b = Coord3D(x, y, x), Coord3D(y, x, y)
            m, M = a.Min(b), a.Max(b)
            for got, want in ((m.X, go_min(x, y)), (m.Y, go_min(y, x)), (M.X, go_max(x, y)), (M.Y, go_max(y, x))):
                assert same(got, want), (x, y, got, want)
