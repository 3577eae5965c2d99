"""Metaball solids on the CPU: the restated math.Pow, the bounds of
WeightedMetaballSolid against the oracle's own restatement, the reference's
metaball tests (model3d/metaball_test.go) as properties of oracle meshes, and
the solids that must refuse to lower."""
import math
from fractions import Fraction

import numpy as np
import pytest

from model3d_gb300 import (Capsule, Cylinder, CubicMetaballFalloffFunc, ExponentialMetaballFalloffFunc,
                           GaussianMetaballFalloffFunc, InversePowerMetaballFalloffFunc, JoinedSolid,
                           MetaballSolid, NotLowerable, QuarticMetaballFalloffFunc, Rect, RotateMetaball,
                           ScaleMetaball, SDFToMetaball, SignedMetaballSolid, Sphere, SubtractedSolid,
                           Torus, TransformMetaball, TranslateMetaball, VecScale, VecScaleMetaball,
                           VecScaleSolid, WeightedMetaballSolid, WyvillMetaballFalloffFunc, XYZ,
                           serialize)
from model3d_gb300.metaballs import go_ldexp, go_pow_int
from model3d_gb300.workloads import metaball_blob


def test_go_pow_matches_exact_powers():
    """Pow(x, -k) by repeated squaring: squaring doubles the relative error,
    so the result is within (k + 2 log2 k + 2) 2^-53 of the exact power;
    exactly 1/x for k = 1, exact for powers of two."""
    rng = np.random.default_rng(5)
    for x in rng.uniform(1e-3, 1e3, 300):
        x = float(x)
        assert go_pow_int(x, -1) == 1 / x
        for k in (2, 3, 4, 5, 7, 16, 33):
            got = Fraction(go_pow_int(x, -k))
            exact = Fraction(x) ** -k
            err = abs(got - exact) / exact
            assert err <= (k + 2 * math.ceil(math.log2(k)) + 2) * Fraction(1, 2 ** 53)
    for e in range(-30, 30):
        assert go_pow_int(2.0 ** e, -4) == 2.0 ** (-4 * e)
    assert go_pow_int(1.0, -4) == 1.0


def test_go_ldexp_rounds_subnormals_once():
    assert go_ldexp(0.75, -1074) == 5e-324 * 1  # 0.75 * 2^-1074 rounds to 2^-1074
    assert go_ldexp(0.5, -1074) == 0.0          # exactly half the smallest subnormal: ties to even
    assert go_ldexp(1.5, 1024) == math.inf
    assert go_ldexp(-0.0, 5) == 0.0 and math.copysign(1, go_ldexp(-0.0, 5)) < 0
    for f, e in [(0.6, -1030), (0.9, -1060), (0.51, 100), (0.999, -1022)]:
        assert go_ldexp(f, e) == math.ldexp(f, e)


def _solids():
    caps = [Capsule(XYZ(0, 0, 0), XYZ(0.5, 0.2, 0.1), 0.2),
            Cylinder(XYZ(0.3, -0.4, 0.1), XYZ(0.1, 0.5, -0.2), 0.15),
            Rect(XYZ(-0.5, -0.4, -0.3), XYZ(-0.2, 0.1, 0.2)),
            Torus(XYZ(0.2, 0.3, -0.4), XYZ(0, 0.6, 0.8), 0.3, 0.08)]
    return {
        "overlaid": MetaballSolid(QuarticMetaballFalloffFunc, 1.0, Sphere(XYZ(1, 2, 0), 1.73),
                                  Sphere(XYZ(1, 2, 0), 1.73)),
        "mixed_cubic": MetaballSolid(CubicMetaballFalloffFunc, 0.1, *caps),
        "signed": SignedMetaballSolid(None, 0.12, caps[:3], [Sphere(XYZ(0.1, 0.1, 0.0), 0.1)]),
        "wyvill": WeightedMetaballSolid(WyvillMetaballFalloffFunc(0.4), 0.1, caps, [1.0, 0.7, 1.3, 0.5]),
        "transformed": MetaballSolid(None, 0.2,
                                     TranslateMetaball(RotateMetaball(caps[0], XYZ(0, 0, 1), 0.7),
                                                       XYZ(0.1, 0.2, 0.3)),
                                     ScaleMetaball(caps[1], 1.5), SDFToMetaball(caps[3]),
                                     VecScaleMetaball(caps[2], XYZ(1.2, -0.8, 0.9))),
        "blob64": metaball_blob(3, 64),
        "linear": MetaballSolid(InversePowerMetaballFalloffFunc(1), 0.3, *caps[:2]),
        "power7": MetaballSolid(InversePowerMetaballFalloffFunc(7), 0.15, *caps),
    }


@pytest.mark.parametrize("name", sorted(_solids()))
def test_bounds_equal_the_oracle(oracle, name):
    """Min()/Max() of the Python mirror equal the oracle's restatement of the
    outset search bit for bit (the spacer depends on them)."""
    s = _solids()[name]
    mn, mx = oracle.bounds(*serialize(s))
    assert list(mn) == s.Min().Array() and list(mx) == s.Max().Array()


def test_metaball_overlaid_bounds():
    """TestMetaballOverlaid (model3d/metaball_test.go:74-96): two overlaid
    quartic spheres outset by 2^(1/4), conservatively, within 1e-4."""
    sphere = Sphere(XYZ(1, 2, 0), 1.73)
    mb = MetaballSolid(QuarticMetaballFalloffFunc, 1.0, sphere, sphere)
    e = 1.18920711500272106671
    exp_min, exp_max = sphere.Min().AddScalar(-e), sphere.Max().AddScalar(e)
    assert mb.Min().Dist(exp_min) <= 1e-4 and mb.Max().Dist(exp_max) <= 1e-4
    assert mb.Min().Min(exp_min) == mb.Min() and mb.Max().Max(exp_max) == mb.Max()


def test_metaball_equivalence(oracle):
    """TestMetaballEquivalence (metaball_test.go:10-40): a quartic sphere
    metaball of radius 1 at threshold 0.5 is the sphere of radius 1.5; the
    mesh's vertices lie on it to within the grid spacing."""
    c = XYZ(1.7, -0.3, 0)
    m = oracle.mc_search(*serialize(MetaballSolid(None, 0.5, Sphere(c, 1.0))), 0.02, 8)
    v = m["tris"].reshape(-1, 3)
    r = np.linalg.norm(v - np.array(c.Array()), axis=1)
    assert np.abs(r - 1.5).max() < 0.02


def test_metaball_equivalence_vecscale(oracle):
    """TestMetaballEquivalenceVecScale (metaball_test.go:42-72): a VecScale'd
    radius-1 sphere solid and the VecScaleMetaball of a radius-0.3 sphere at
    threshold 0.7 are one ellipsoid; both meshes' vertices lie on it."""
    obj = Sphere(XYZ(1, 2, 0), 1.0)
    scale = XYZ(0.25, 0.5, 1.0)
    mb = MetaballSolid(None, 0.7, VecScaleMetaball(Sphere(XYZ(1, 2, 0), 0.3), scale))
    for s in (VecScaleSolid(obj, scale), mb):
        v = oracle.mc_search(*serialize(s), 0.02, 8)["tris"].reshape(-1, 3)
        q = v / np.array(scale.Array()) - np.array([1, 2, 0])
        assert np.abs(np.linalg.norm(q, axis=1) - 1).max() < 0.02 / 0.25


def test_metaball_mesh_is_closed(oracle):
    """Random-solid manifoldness (mc_test.go:27-42) for a 64-ball blob."""
    tris = oracle.mc_search(*serialize(metaball_blob(3, 64)), 0.03, 8)["tris"]
    v = tris.reshape(-1, 3, 3)
    edges = {}
    for t in v:
        for a, b in ((0, 1), (1, 2), (2, 0)):
            k = (tuple(t[a]), tuple(t[b]))
            edges[k] = edges.get(k, 0) + 1
    for (a, b), n in edges.items():
        assert n == 1 and edges.get((b, a)) == 1


def test_not_lowerable_and_reference_panics():
    s = Sphere(XYZ(0, 0, 0), 1)
    with pytest.raises(NotLowerable):
        MetaballSolid(ExponentialMetaballFalloffFunc, 0.5, s)
    with pytest.raises(NotLowerable):
        MetaballSolid(GaussianMetaballFalloffFunc, 0.5, s)
    with pytest.raises(NotLowerable):
        MetaballSolid(InversePowerMetaballFalloffFunc(2.5), 0.5, s)
    with pytest.raises(TypeError):  # VecScale's inverse is not a DistTransform
        TransformMetaball(VecScale(XYZ(1, 2, 3)), s)
    with pytest.raises(ValueError):
        WeightedMetaballSolid(None, 0.5, [s, s], [1.0])
    with pytest.raises(ValueError):
        InversePowerMetaballFalloffFunc(0)
    with pytest.raises(ValueError):
        WyvillMetaballFalloffFunc(-1)
    with pytest.raises(NotLowerable):
        MetaballSolid(None, 0.5, JoinedSolid([s]))
    # No positive weight: NewRect(Origin, Origin) (metaball.go:186-188).
    r = SignedMetaballSolid(None, 0.5, [], [s])
    assert isinstance(r, Rect) and r.Min().Array() == [0, 0, 0] == r.Max().Array()


def test_serialised_records(oracle):
    """One METABALL record, then per ball a BALL record with the weight, the
    forward steps innermost first and the primitive; metaballs nest under CSG
    nodes like any leaf."""
    ball = TranslateMetaball(ScaleMetaball(Sphere(XYZ(0, 0, 0), 0.2), 2.0), XYZ(0.1, 0, 0))
    mb = WeightedMetaballSolid(None, 0.1, [ball, Capsule(XYZ(0, 0, 0), XYZ(0.3, 0, 0), 0.1)], [1.0, -0.5])
    nodes, _ = serialize(SubtractedSolid(mb, Sphere(XYZ(0.5, 0.5, 0.5), 0.1)))
    kinds = list(nodes["kind"])
    assert kinds == [17, 7, 8, 33, 32, 1, 8, 4, 1]
    assert nodes[1]["n_children"] == 2 and list(nodes[1]["p"][:3]) == [0.1, 1, 4]
    assert nodes[2]["p"][0] == 1.0 and nodes[2]["n_steps"] == 2 and nodes[6]["p"][0] == -0.5
    assert list(nodes[1]["min"]) == mb.Min().Array()
    oracle.bounds(nodes, [])  # parses


def _records(s):
    nodes, _ = serialize(s)
    return nodes.copy()


def test_library_lowering_on_the_host():
    """mc_program_check lowers without a GPU: the library's own restatement of
    math.Pow gives the same threshold bits as the Python mirror's, the root
    bounds are the serialised ones, and the program has one leaf per metaball."""
    from model3d_gb300 import check_program
    for name, s in _solids().items():
        info = check_program(s)
        assert info["n_metaballs"] == 1 and info["n_leaves"] == 1, name
        assert info["n_balls"] == len(s.balls)
        assert info["threshold"] == s.falloff(s.radiusThreshold), name
        assert info["root_min"] == s.Min().Array() and info["root_max"] == s.Max().Array()
    for k in range(1, 9):
        for rt in (0.05, 0.1, 0.37, 1.0, 3.3):
            s = MetaballSolid(InversePowerMetaballFalloffFunc(k), rt, Sphere(XYZ(0, 0, 0), 0.3))
            assert check_program(s)["threshold"] == go_pow_int(rt, -k)
    info = check_program(JoinedSolid([metaball_blob(1, 5), Sphere(XYZ(2, 0, 0), 0.2)]))
    assert info["n_metaballs"] == 1 and info["n_leaves"] == 2


def test_library_lowering_errors():
    """Malformed or unlowerable metaball records return statuses on the host."""
    import ctypes
    from model3d_gb300 import _native as N
    L = N.lib()
    base = _records(MetaballSolid(None, 0.1, Sphere(XYZ(0, 0, 0), 0.3), Capsule(XYZ(0, 0, 0), XYZ(0.2, 0, 0), 0.1)))

    def status(nodes):
        err = ctypes.create_string_buffer(256)
        return L.mc_program_check(nodes.ctypes.data, len(nodes), None, 0, None, err, 256), err.value.decode()

    assert status(base)[0] == N.MC_OK
    bad = base.copy()
    bad[0]["p"][1] = 3  # unknown falloff kind
    assert status(bad)[0] == N.MC_ERR_NOT_LOWERABLE
    bad = base.copy()
    bad[0]["p"][2] = 2.5  # non-integer power
    assert status(bad)[0] == N.MC_ERR_NOT_LOWERABLE
    bad = base.copy()
    bad[0]["p"][1], bad[0]["p"][2] = 2, -1.0  # Wyvill needs d > 0
    assert status(bad)[0] == N.MC_ERR_BAD_PROGRAM
    bad = base.copy()
    bad[1]["kind"] = 1  # a ball record replaced by a primitive
    assert status(bad)[0] == N.MC_ERR_BAD_PROGRAM
    bad = base.copy()
    bad[2]["kind"] = 16  # a ball's primitive replaced by a combinator
    assert status(bad)[0] == N.MC_ERR_BAD_PROGRAM
    assert status(base[:3])[0] == N.MC_ERR_BAD_PROGRAM  # truncated
    many = _records(MetaballSolid(None, 0.1, *[Sphere(XYZ(i * 0.01, 0, 0), 0.1) for i in range(4097)]))
    assert status(many)[0] == N.MC_ERR_LIMIT
