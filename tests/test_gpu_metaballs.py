"""Metaball solids on the GPU, bit-exact against the oracle: meshes in both
precision modes with tile culling on and off, containment next to the
threshold surface, metaballs inside CSG trees, transforms and batches, and
the float64 corner cases of the weighted sum (infinite and NaN terms)."""
import numpy as np
import pytest

from model3d_gb300 import (Capsule, Contains, Cylinder, CubicMetaballFalloffFunc, DeviceSolid,
                           InversePowerMetaballFalloffFunc, JoinedSolid, LinearMetaballFalloffFunc,
                           MarchingCubesSearch, MarchingCubesSearchBatch, MetaballSolid, Rect,
                           RotateMetaball, ScaleMetaball, SDFToMetaball, SignedMetaballSolid, Sphere,
                           SubtractedSolid, Torus, TransformSolid, TranslateMetaball, Translate,
                           VecScaleMetaball, WeightedMetaballSolid, WyvillMetaballFalloffFunc, XYZ,
                           canonical, serialize)
from model3d_gb300.workloads import metaball_blob

pytestmark = pytest.mark.gpu

MODES = [("fp64", True), ("fp32", True), ("fp32", False)]


def _check(oracle, solid, delta, iters=8, modes=MODES):
    nodes, sets = serialize(solid)
    ref = oracle.mc_search(nodes, sets, delta, iters)
    ds = DeviceSolid(solid)
    out = None
    for prec, cull in modes:
        m = MarchingCubesSearch(ds, delta, iters, precision=prec, cull=cull)
        a, b = canonical(m.TriangleSoup()), canonical(ref["tris"])
        assert a.shape == b.shape, f"{prec}: {len(a)} triangles, oracle {len(b)}"
        assert np.array_equal(a, b), f"{prec}: {np.count_nonzero((a != b).any(1))} triangles differ"
        if prec == "fp32" and cull:
            out = m
    return out


CAPS = [Capsule(XYZ(0, 0, 0), XYZ(0.5, 0.2, 0.1), 0.2),
        Cylinder(XYZ(0.3, -0.4, 0.1), XYZ(0.1, 0.5, -0.2), 0.15),
        Rect(XYZ(-0.5, -0.4, -0.3), XYZ(-0.2, 0.1, 0.2)),
        Torus(XYZ(0.2, 0.3, -0.4), XYZ(0, 0.6, 0.8), 0.3, 0.08)]


@pytest.mark.parametrize("kind", range(4))
def test_single_primitive_balls(oracle, kind):
    _check(oracle, MetaballSolid(None, 0.1, CAPS[kind]), 0.01)


def test_quartic_blob_64(oracle):
    m = _check(oracle, metaball_blob(3, 64), 0.012)
    assert m.stats["escalations"] <= 0.02 * m.stats["leaf_evals"]


def test_many_balls(oracle):
    """200 balls: classification tiles near the middle have more near balls
    than the far-field split lists, and fall back to the full sum."""
    _check(oracle, metaball_blob(21, 200), 0.03)


@pytest.mark.parametrize("f", [LinearMetaballFalloffFunc, CubicMetaballFalloffFunc,
                               InversePowerMetaballFalloffFunc(7), WyvillMetaballFalloffFunc(0.4),
                               WyvillMetaballFalloffFunc(0.15)])
def test_falloffs(oracle, f):
    _check(oracle, WeightedMetaballSolid(f, 0.1, CAPS, [1.0, 0.7, 1.3, 0.5]), 0.01)


def test_signed_and_weighted(oracle):
    """Negative balls, a zero weight and non-float weights."""
    _check(oracle, SignedMetaballSolid(None, 0.12, CAPS[:3], [Sphere(XYZ(0.1, 0.1, 0.0), 0.1)]), 0.01)
    _check(oracle, WeightedMetaballSolid(None, 0.1, CAPS + [Sphere(XYZ(0.4, 0.4, 0.4), 0.1)],
                                         [0.3, 1 / 3, 0.7, 1.1, 0.0]), 0.01)


def test_transformed_balls(oracle):
    s = MetaballSolid(None, 0.2, TranslateMetaball(RotateMetaball(CAPS[0], XYZ(0, 0, 1), 0.7), XYZ(0.1, 0.2, 0.3)),
                      ScaleMetaball(CAPS[1], 1.5), SDFToMetaball(CAPS[3]),
                      VecScaleMetaball(CAPS[2], XYZ(1.2, -0.8, 0.9)))
    _check(oracle, s, 0.01)


def test_metaballs_in_csg_and_transforms(oracle):
    mb = metaball_blob(7, 16)
    _check(oracle, SubtractedSolid(JoinedSolid([mb, Sphere(XYZ(0.9, 0.9, 0.9), 0.3)]),
                                   Capsule(XYZ(-1, 0, 0), XYZ(1, 0, 0), 0.15)), 0.015)
    _check(oracle, TransformSolid(Translate(XYZ(0.3, 0.1, -0.2)), mb), 0.015)
    # two metaball leaves: the search's far-field region serves the first only
    _check(oracle, JoinedSolid([metaball_blob(8, 12), TransformSolid(Translate(XYZ(0.4, 0, 0)), metaball_blob(9, 12))]),
           0.015)


def test_infinite_and_nan_terms(oracle):
    """Inside a positive ball the term is +Inf (contained); inside a positive
    and a negative ball at once Inf - Inf is NaN (not contained); a zero
    weight times +Inf is NaN too."""
    pos = Sphere(XYZ(0, 0, 0), 0.4)
    neg = Sphere(XYZ(0.3, 0, 0), 0.2)
    _check(oracle, SignedMetaballSolid(None, 0.2, [pos], [neg]), 0.01)
    _check(oracle, WeightedMetaballSolid(None, 0.2, [pos, neg], [1.0, 0.0]), 0.01)


def test_contains_near_the_threshold_surface(oracle):
    """Vertices of the mesh (on the threshold surface to 8 bisection steps)
    and points one and two float ulps around them, in both modes."""
    for s in (metaball_blob(5, 24), WeightedMetaballSolid(WyvillMetaballFalloffFunc(0.3), 0.05, CAPS,
                                                          [1.0, 0.8, 1.2, 0.9])):
        ref_mesh = oracle.mc_search(*serialize(s), 0.02, 8)
        v = np.unique(ref_mesh["tris"].reshape(-1, 3), axis=0)[:20000]
        f = np.float32
        jitter = [v, np.nextafter(v, np.inf), np.nextafter(v, -np.inf),
                  v + np.spacing(v.astype(f)).astype(float), v - np.spacing(v.astype(f)).astype(float)]
        pts = np.ascontiguousarray(np.concatenate(jitter))
        ref, _ = oracle.contains(*serialize(s), pts)
        for prec in ("fp64", "fp32"):
            assert (Contains(s, pts, precision=prec) == ref).all()


def test_metaball_batch(oracle):
    jobs = [(metaball_blob(11 + i, 8 + 4 * i), 0.02 + 0.005 * i) for i in range(4)]
    jobs.append((Sphere(XYZ(0, 0, 0), 0.5), 0.03))
    meshes = MarchingCubesSearchBatch([(DeviceSolid(s), d, 8) for s, d in jobs])
    for (s, d), m in zip(jobs, meshes):
        ref = oracle.mc_search(*serialize(s), d, 8)
        assert np.array_equal(canonical(m.TriangleSoup()), canonical(ref["tris"]))


def test_empty_threshold(oracle):
    """radiusThreshold <= 0 makes the threshold +Inf: nothing is contained."""
    m = MarchingCubesSearch(DeviceSolid(MetaballSolid(None, 0.0, CAPS[0])), 0.05, 8)
    assert m.NumTriangles() == 0


def _random_metaball(seed):
    """A metaball solid mixing every primitive kind and wrapper, negative and
    non-float weights, and one of the lowerable falloffs."""
    from model3d_gb300.workloads import SplitMix64
    rng = SplitMix64(seed)
    balls, weights = [], []
    for i in range(6 + seed % 7):
        c = XYZ(rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5))
        r = rng.uniform(0.05, 0.2)
        k = rng.next_u64() % 5
        axis = rng.unit_vector()
        if k == 0:
            b = Sphere(c, r)
        elif k == 1:
            h = XYZ(rng.uniform(0.03, 0.15), rng.uniform(0.03, 0.15), rng.uniform(0.03, 0.15))
            b = Rect(c.Sub(h), c.Add(h))
        elif k == 2:
            b = Capsule(c.Sub(axis.Scale(0.1)), c.Add(axis.Scale(0.1)), r)
        elif k == 3:
            b = Cylinder(c.Sub(axis.Scale(0.1)), c.Add(axis.Scale(0.1)), r)
        else:
            b = Torus(c, axis, 0.15, r * 0.5)
        w = rng.next_u64() % 4
        if w == 0:
            b = TranslateMetaball(RotateMetaball(b, rng.unit_vector(), rng.uniform(0, 3)), XYZ(0.05, -0.02, 0.01))
        elif w == 1:
            b = VecScaleMetaball(ScaleMetaball(b, rng.uniform(0.7, 1.3)), XYZ(1.1, 0.9, rng.uniform(0.8, 1.2)))
        balls.append(b)
        weights.append(-rng.uniform(0.1, 0.5) if i % 4 == 3 else rng.uniform(0.4, 1.6))
    f = [None, CubicMetaballFalloffFunc, LinearMetaballFalloffFunc, WyvillMetaballFalloffFunc(0.3)][seed % 4]
    return WeightedMetaballSolid(f, 0.08 if f is None or f is CubicMetaballFalloffFunc else 0.12, balls, weights)


@pytest.mark.parametrize("seed", range(12))
def test_filter_is_sound_on_random_metaballs(oracle, seed):
    """FP32-filtered Contains equals the float64 kernel at every point on and
    a few float ulps around the threshold surface of random metaball solids
    (the filter never decides a point the float64 sum would decide the other
    way), and both equal the oracle on a subset."""
    s = _random_metaball(seed)
    ds = DeviceSolid(s)
    mesh = MarchingCubesSearch(ds, 0.02, 8, precision="fp64")
    if mesh.NumTriangles() == 0:
        pytest.skip("empty solid")
    v = np.unique(mesh.vertices, axis=0)
    sp = np.spacing(v.astype(np.float32)).astype(float)
    pts = np.ascontiguousarray(np.concatenate(
        [v, np.nextafter(v, np.inf), np.nextafter(v, -np.inf), v + sp, v - sp, v + 3 * sp, v - 3 * sp]))
    a = Contains(s, pts, precision="fp32")
    b = Contains(s, pts, precision="fp64")
    assert (a == b).all(), f"{np.count_nonzero(a != b)} of {len(pts)} points differ"
    sub = pts[::7]
    ref, _ = oracle.contains(*serialize(s), np.ascontiguousarray(sub))
    assert (b[::7] == ref).all()


def test_power_and_parameter_extremes(oracle):
    """Powers past the fast bracket's k <= 64, and Wyvill radii whose d^2
    leaves the float range (every corner then takes the float64 sum)."""
    s1 = Sphere(XYZ(0, 0, 0), 0.3)
    s2 = Capsule(XYZ(0.1, -0.2, 0.05), XYZ(0.35, 0.1, -0.1), 0.12)
    _check(oracle, MetaballSolid(InversePowerMetaballFalloffFunc(20), 0.1, s1, s2), 0.02)
    _check(oracle, MetaballSolid(InversePowerMetaballFalloffFunc(100), 0.1, s1, s2), 0.02)
    # d^2 = 9e-32: every corner in the box takes the float64 sum.  Inside a
    # ball the Wyvill falloff is +Inf, so the solid is the balls' union.
    _check(oracle, WeightedMetaballSolid(WyvillMetaballFalloffFunc(3e-16), 1e-16, [s1, s2], [1.0, 0.5]), 0.02)


def test_metaball_with_collider_and_intersection(oracle):
    """Metaball leaves next to a collider leaf (both rare kinds in one
    program) and under an intersection."""
    from model3d_gb300 import IntersectedSolid, MeshToCollider, NewColliderSolid
    from model3d_gb300.workloads import displaced_icosphere
    col = NewColliderSolid(MeshToCollider(displaced_icosphere(6) * 0.4 + 0.5))
    mb = metaball_blob(13, 10)
    _check(oracle, JoinedSolid([mb, col]), 0.02)
    _check(oracle, IntersectedSolid([mb, Rect(XYZ(-0.5, -0.6, -0.4), XYZ(0.4, 0.3, 0.5))]), 0.015)
