"""Digests of the host lowering (tests/golden/lowering.json).

For each scene below, `check_program` lowers the solid on the host and
returns `digest`, an FNV-1a hash of every array the library would upload
(CSG bytecode, leaf tables, bound boxes, collider trees and ray grids,
metaball tables).  The fixture pins the lowering that the GPU parity tests
passed with.  Regenerate it only for an intended change of the device
program, after the GPU tests pass with that change:

    python tests/golden/make_lowering_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from model3d_gb300 import (XYZ, CacheSolidBounds, Cylinder, JoinedSolid, JoinedTransform,  # noqa: E402
                           MeshToCollider, NewColliderSolid, Rotation, Scale, Sphere, SubtractedSolid,
                           Torus, TransformSolid, Translate, WyvillMetaballFalloffFunc, check_program)
from model3d_gb300.workloads import (box_triangles, csg_tree, displaced_icosphere,  # noqa: E402
                                     icosphere_triangles, metaball_blob)


def _soup(n, seed, scale=0.05):
    """n random small triangles around points of [-1, 1]^3 (seeded)."""
    r = np.random.default_rng(seed)
    c = r.uniform(-1, 1, (n, 1, 3))
    return (c + r.normal(0, scale, (n, 3, 3))).reshape(-1, 9)


def _degenerate(n, seed):
    """A soup with every 7th triangle's second vertex repeated (det 0) and
    every 11th (from the 2nd) collinear."""
    t = _soup(n, seed)
    t[::7, 3:6] = t[::7, 0:3]
    t[1::11, 6:9] = 2 * t[1::11, 3:6] - t[1::11, 0:3]
    return t


def scenes():
    """name -> solid.  Sizes stay small enough to lower in a few seconds in all."""
    ico = NewColliderSolid(MeshToCollider(icosphere_triangles(40)))
    return {
        "csg_tree_48_16": csg_tree(1),
        "csg_tree_6_2_transformed": TransformSolid(
            JoinedTransform([Translate(XYZ(1, 2, 3)), Scale(2.0), Rotation(XYZ(0, 0, 1), 0.3)]),
            csg_tree(2, 6, 2)),
        "torus_minus_cylinder_cached": CacheSolidBounds(SubtractedSolid(
            Torus(XYZ(0, 0, 0), XYZ(0.2, 0.9, 0.1).Normalize(), 1.0, 0.25),
            Cylinder(XYZ(0, 0, -2), XYZ(0.1, 0, 2), 0.3))),
        "collider_icosphere_32000": ico,
        # 72,000 triangles: above the size at which grouping runs on threads.
        "collider_displaced_icosphere_72000": NewColliderSolid(MeshToCollider(displaced_icosphere(60, seed=3))),
        "collider_box_with_csg": JoinedSolid([
            NewColliderSolid(MeshToCollider(box_triangles((2.0, -0.5, -0.5), (3.0, 0.5, 0.5)))),
            ico, Sphere(XYZ(0, 3, 0), 0.5)]),
        # Just above the size at which the ray grid is counted and filled in
        # bands of cell rows; degenerate triangles; many equal midpoints.
        "collider_soup_65537": NewColliderSolid(MeshToCollider(_soup(65537, 65537))),
        "collider_degenerate_70000": NewColliderSolid(MeshToCollider(_degenerate(70000, 1))),
        "collider_lattice_90000": NewColliderSolid(MeshToCollider(np.round(_soup(90000, 3) * 8) / 8)),
        "metaball_blob_12": metaball_blob(2, 12),
        "metaball_blob_wyvill_8": metaball_blob(4, 8, falloff=WyvillMetaballFalloffFunc(0.6)),
    }


def digests():
    return {name: check_program(s)["digest"] for name, s in scenes().items()}


if __name__ == "__main__":
    out = os.path.join(HERE, "lowering.json")
    with open(out, "w") as f:
        json.dump(digests(), f, indent=1, sort_keys=True)
        f.write("\n")
    print(out)
