"""Host lowering of CSG, transformed, checked and collider solids, with no GPU.

`mc_program_check` runs the same lowering as `mc_solid_create` (CSG bytecode,
leaf tables, bound boxes, collider trees) and reports the program's shape.
The root bounds it reports are the serialised `Min()/Max()` of the root
(`model3d/mc.go:594-608` builds the grid from them), so they must match the
Python mirror bit for bit.  Malformed record arrays come back as statuses.
"""
import ctypes
import math

import numpy as np
import pytest

from model3d_gb300 import (XYZ, CacheSolidBounds, Capsule, Cylinder, ForceSolidBounds, IntersectedSolid,
                           JoinedSolid, JoinedTransform, MeshToCollider, NewColliderSolid, NotLowerable, Rect,
                           Rotation, Scale, Solid, Sphere, SubtractedSolid, Torus, TransformSolid, Translate,
                           check_program, serialize)
from model3d_gb300 import _native as N
from model3d_gb300.mc import _tri_sets
from model3d_gb300.workloads import box_triangles, csg_batch, csg_tree, icosphere_triangles


def _bits(v):
    return np.asarray(v, dtype=np.float64).view(np.uint64).tolist()


def _assert_root_bounds(info, solid):
    assert _bits(info["root_min"]) == _bits(solid.Min().Array())
    assert _bits(info["root_max"]) == _bits(solid.Max().Array())


def _primitives(s):
    """Leaf count of a CSG tree as the reference walks it."""
    if isinstance(s, (JoinedSolid, IntersectedSolid)):
        return sum(_primitives(c) for c in s.solids)
    if isinstance(s, SubtractedSolid):
        return _primitives(s.Positive) + _primitives(s.Negative)
    return 1


def test_headline_tree_lowers_to_one_leaf_per_primitive():
    s = csg_tree(1)
    info = check_program(s)
    assert info["n_leaves"] == 64 == _primitives(s)
    assert info["n_colliders"] == info["n_metaballs"] == info["n_boxes"] == 0
    assert info["n_ops"] >= 1 and info["max_stack"] >= 1
    assert np.isnan(info["threshold"])
    _assert_root_bounds(info, s)


def test_batch_solids_lower_with_their_own_bounds():
    for s, _delta in csg_batch(2024, count=24):
        info = check_program(s)
        assert info["n_leaves"] == _primitives(s)
        _assert_root_bounds(info, s)


def test_every_primitive_and_combinator():
    prims = [Sphere(XYZ(0.1, 0.2, 0.3), 0.7), Rect(XYZ(-1, -0.5, -0.25), XYZ(0.5, 1, 0.75)),
             Cylinder(XYZ(0, 0, -1), XYZ(0.3, 0.2, 1), 0.4), Capsule(XYZ(-1, 0, 0), XYZ(1, 0.5, 0), 0.3),
             Torus(XYZ(0, 0, 0), XYZ(0.2, 0.9, 0.1).Normalize(), 1.0, 0.25)]
    for p in prims:
        info = check_program(p)
        assert info["n_leaves"] == 1 and info["n_ops"] == 1
        _assert_root_bounds(info, p)
    for s in (JoinedSolid(prims), IntersectedSolid(prims[:3]), SubtractedSolid(JoinedSolid(prims[:2]), prims[4])):
        info = check_program(s)
        assert info["n_leaves"] == _primitives(s)
        _assert_root_bounds(info, s)


def test_transforms_and_checked_solids_add_one_bound_box_each():
    inner = csg_tree(2, 6, 2)
    t = TransformSolid(JoinedTransform([Translate(XYZ(1, 2, 3)), Scale(2.0),
                                        Rotation(XYZ(0, 0, 1), 0.3)]), inner)
    info = check_program(t)
    assert info["n_leaves"] == 8 and info["n_boxes"] == 1
    _assert_root_bounds(info, t)
    c = CacheSolidBounds(csg_tree(3, 5, 1))
    info = check_program(c)
    assert info["n_leaves"] == 6 and info["n_boxes"] == 1
    _assert_root_bounds(info, c)
    f = ForceSolidBounds(Sphere(XYZ(0, 0, 0), 1), XYZ(-2, -2, -2), XYZ(2, 2, 2))
    info = check_program(f)
    assert info["root_min"] == [-2.0] * 3 and info["root_max"] == [2.0] * 3
    nested = TransformSolid(Translate(XYZ(0.5, 0, 0)), CacheSolidBounds(t))
    info = check_program(nested)
    assert info["n_leaves"] == 8 and info["n_boxes"] == 3
    _assert_root_bounds(info, nested)


def test_colliders_lower_to_one_leaf_per_collider():
    ico = NewColliderSolid(MeshToCollider(icosphere_triangles(2)))
    info = check_program(ico)
    assert info["n_colliders"] == 1 and info["n_leaves"] == 1
    _assert_root_bounds(info, ico)
    box = NewColliderSolid(MeshToCollider(box_triangles((2.0, -0.5, -0.5), (3.0, 0.5, 0.5))))
    mixed = JoinedSolid([ico, box, Sphere(XYZ(0, 3, 0), 0.5)])
    info = check_program(mixed)
    assert info["n_colliders"] == 2 and info["n_leaves"] == 3
    _assert_root_bounds(info, mixed)


def _status(nodes, sets=()):
    arr, keep = _tri_sets(list(sets))
    err = ctypes.create_string_buffer(256)
    info = N.MCProgramInfo()
    st = N.lib().mc_program_check(nodes.ctypes.data if len(nodes) else None, len(nodes),
                                  ctypes.addressof(arr), len(sets), ctypes.byref(info), err, len(err))
    return st, err.value.decode()


def test_collider_bounds_follow_math_min_max():
    """MeshCollider.Min/Max equal the fold of math.Min / math.Max over every
    vertex coordinate (Triangle.Min and the joined colliders' bounds,
    model3d/primitives.go:36-42, collisions.go:217-253): -Inf wins over NaN,
    NaN over numbers, -0 over +0 in Min and +0 over -0 in Max."""
    import functools
    from model3d_gb300.geometry import go_max, go_min
    from model3d_gb300.solids import MeshCollider
    rng = np.random.default_rng(5)
    specials = [0.0, -0.0, math.nan, math.inf, -math.inf, 1.5, -2.25]
    for trial in range(300):
        n = int(rng.integers(1, 6))
        t = rng.choice([0.0, -0.0, 0.5, -0.5], size=(n, 9))
        for _ in range(int(rng.integers(0, 4))):
            t[rng.integers(0, n), rng.integers(0, 9)] = specials[rng.integers(0, len(specials))]
        c = MeshCollider(t, grouped=False)
        v = t.reshape(-1, 3)
        for got, op in ((c.Min(), go_min), (c.Max(), go_max)):
            for a, g in enumerate(got.Array()):
                want = functools.reduce(op, [float(x) for x in v[:, a]])
                assert (g != g and want != want) or (g == want and math.copysign(1, g) == math.copysign(1, want)), \
                    (trial, a, g, want)


def test_malformed_records_are_rejected():
    nodes, _ = serialize(JoinedSolid([Sphere(XYZ(0, 0, 0), 1), Sphere(XYZ(1, 0, 0), 0.5)]))
    assert _status(nodes) == (N.MC_OK, "")
    assert _status(nodes[:0])[0] == N.MC_ERR_ARG
    assert _status(nodes[:2])[0] == N.MC_ERR_BAD_PROGRAM
    assert _status(np.concatenate([nodes, nodes[1:2]]))[0] == N.MC_ERR_BAD_PROGRAM
    bad = nodes.copy()
    bad[0]["kind"] = 99
    assert _status(bad)[0] == N.MC_ERR_NOT_LOWERABLE
    bad = nodes.copy()
    bad[0]["n_children"] = 5
    assert _status(bad)[0] == N.MC_ERR_BAD_PROGRAM
    bad = nodes.copy()
    bad[0]["n_children"] = -1
    assert _status(bad)[0] == N.MC_ERR_BAD_PROGRAM


def test_collider_records_need_their_triangle_set():
    nodes, sets = serialize(NewColliderSolid(MeshToCollider(icosphere_triangles(1))))
    assert _status(nodes, sets)[0] == N.MC_OK
    assert _status(nodes, [])[0] == N.MC_ERR_BAD_PROGRAM
    bad = nodes.copy()
    bad[0]["mesh"] = 3
    assert _status(bad, sets)[0] == N.MC_ERR_BAD_PROGRAM


def test_user_defined_solids_are_not_lowerable():
    class Custom(Solid):
        def Min(self):
            return XYZ(-1, -1, -1)

        def Max(self):
            return XYZ(1, 1, 1)

        def Contains(self, c):
            return c.Norm() < 1

    with pytest.raises(NotLowerable):
        check_program(Custom())
    with pytest.raises(NotLowerable):
        check_program(JoinedSolid([Sphere(XYZ(0, 0, 0), 1), Custom()]))


def test_lowering_matches_golden_digests():
    """Every array of the lowered program is byte-identical to the lowering
    that the GPU parity tests passed with (tests/golden/lowering.json, made by
    tests/golden/make_lowering_golden.py)."""
    import json
    import os
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    import make_lowering_golden as G
    gold = json.load(open(os.path.join(here, "lowering.json")))
    assert G.digests() == gold


def test_digest_follows_every_byte():
    """One ulp in one parameter, or one triangle moved, changes the digest."""
    import math
    a = check_program(Sphere(XYZ(0, 0, 0), 1.0))["digest"]
    assert check_program(Sphere(XYZ(0, 0, 0), 1.0))["digest"] == a
    assert check_program(Sphere(XYZ(0, 0, 0), math.nextafter(1.0, 2.0)))["digest"] != a
    tris = icosphere_triangles(4)
    d0 = check_program(NewColliderSolid(MeshToCollider(tris)))["digest"]
    moved = tris.copy()
    moved[7, 4] = math.nextafter(moved[7, 4], 9.0)
    assert check_program(NewColliderSolid(MeshToCollider(moved)))["digest"] != d0


def test_overridden_bounds_are_serialised():
    """A subclass that overrides Min/Max (as the batch's border-panic test
    does) is serialised with its own bounds, inside a tree as at the root."""
    class Lying(Sphere):
        def Min(self):
            return XYZ(-0.5, -0.5, -0.5)

        def Max(self):
            return XYZ(0.5, 0.5, 0.5)

    for s in (Lying(XYZ(0, 0, 0), 1.0), JoinedSolid([Lying(XYZ(0, 0, 0), 1.0), Sphere(XYZ(0, 0, 0), 0.2)]),
              SubtractedSolid(Lying(XYZ(0.1, 0, 0), 1.0), Sphere(XYZ(0, 0, 0), 0.2))):
        _assert_root_bounds(check_program(s), s)
        assert s.Max().Array() == [0.5, 0.5, 0.5]
