#!/usr/bin/env python3
"""Generate tests/golden/meshes.json: SHA-256 digests of canonical meshes
(triangles as nine float64 bit patterns, rows sorted) of small seeded
workloads, computed by the oracle (oracle/mc_oracle.cpp).

The reference is Go and cannot run here, so these digests pin the oracle
against future changes of itself and give the GPU path a fixed target; the
oracle's agreement with the reference rests on the reference's property
tests restated in tests/test_oracle.py.

    python tests/golden/make_golden.py      # rewrites meshes.json
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from model3d_gb300 import (Cylinder, MeshToCollider, NewColliderSolid, Rotation, Sphere,  # noqa: E402
                           SubtractedSolid, TransformSolid, XYZ, canonical, serialize)
from model3d_gb300.workloads import box_triangles, csg_tree, displaced_icosphere, metaball_blob  # noqa: E402


def cases():
    boxes = np.concatenate([box_triangles((-1, -1, -1), (0, 0, 0)), box_triangles((0.1, 0, 0), (1, 1, 1))])
    return {
        "sphere_r1_delta0.1_iters8": (Sphere(XYZ(0, 0, 0), 1.0), 0.1, 8),
        "sphere_offset_delta0.05_iters0": (Sphere(XYZ(0.1, 0.3, -0.2), 0.7), 0.05, 0),
        "benchmark_cylinder_delta0.05_iters8": (Cylinder(XYZ(1, 2, 3), XYZ(3, 1, 4), 0.5), 0.05, 8),
        "csg_tree_1_12_4_delta0.04_iters8": (csg_tree(1, 12, 4), 0.04, 8),
        "rotated_subtraction_delta0.04_iters8": (
            TransformSolid(Rotation(XYZ(0, 0.6, 0.8), 0.7),
                           SubtractedSolid(Cylinder(XYZ(0, 0, -0.5), XYZ(0.2, 0.1, 0.5), 0.4),
                                           Sphere(XYZ(0.1, 0, 0.3), 0.25))), 0.04, 8),
        "collider_two_boxes_delta0.1_iters8": (NewColliderSolid(MeshToCollider(boxes)), 0.1, 8),
        "collider_icosphere8_delta0.05_iters8": (NewColliderSolid(MeshToCollider(displaced_icosphere(8))), 0.05, 8),
        "metaball_blob_2_12_delta0.04_iters8": (metaball_blob(2, 12), 0.04, 8),
    }


def digest(tris):
    return hashlib.sha256(np.ascontiguousarray(canonical(tris)).tobytes()).hexdigest()


def main():
    from oracle import oracle as O
    out = {}
    for name, (solid, delta, iters) in cases().items():
        nodes, sets = serialize(solid)
        m = O.mc_search(nodes, sets, delta, iters)
        out[name] = {"delta": delta, "iters": iters, "triangles": int(len(m["tris"])),
                     "vertices": int(m["n_vertices"]), "sha256": digest(m["tris"])}
    counts, tris = O.case_table()[:2]
    out["case_table"] = {"sha256": hashlib.sha256(np.ascontiguousarray(counts, dtype=np.uint8).tobytes() +
                                                  np.ascontiguousarray(tris, dtype=np.uint8).tobytes()).hexdigest()}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "meshes.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
