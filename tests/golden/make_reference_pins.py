#!/usr/bin/env python3
"""Generate the fixtures that pin the oracle to the reference's own outputs.

model3d ships two meshes under model3d/test_data/, and this script turns
them into the small fixtures the tests use (the reference tree is read here,
in the build container, and never at test time):

* hierarchy_test.stl.gz is an OUTPUT of the reference path.  Its generator is
  recorded in model3d/mesh_hierarchy_test.go:104-127:
      solid := JoinedSolid{shell((0,0,0), 1), shell((0,0,0), 0.5),
                           &Sphere{Radius: 0.1}, shell((3,0,0), 1),
                           &Sphere{Center: Y(3), Radius: 1}}
      mesh = MarchingCubesSearch(solid, 0.03, 2); mesh.SaveGroupedSTL(...)
  with shell(c, r) = &SubtractedSolid{&Sphere{c, r}, &Sphere{c, r - 0.05}}.
  Binary STL stores float32 casts of Triangle.Normal() and of the three
  vertices (model3d/export.go:20-66), so this pins MarchingCubesSearch (both
  phases: cube classification and the bisection search) at float32
  resolution.  reference_meshes.json keeps the triangle count, the SHA-256 of
  the 9 x float32 vertex bit patterns with rows sorted (vertex order inside a
  triangle kept), and the SHA-256 of the float32 normals in that row order.
  The file's record order is SaveGroupedSTL's GroupTriangles order, which
  the reference leaves to Go map order and an unstable sort on ties; what
  it fixes is the top of the hierarchy: the axes along which the halves of
  the nodes above depth 3 are separated by triangle midpoint, and the
  midpoint centroids of the eight depth-3 nodes (file coordinates).
* non_intersecting_hook.stl is a 19,584-triangle INPUT mesh
  (model3d/primitives_test.go:273-285).  It is stored as an indexed float32
  mesh in non_intersecting_hook.npz (unique vertices + faces); expanding it
  gives the file's triangle soup, in the file's order, exactly.

    python tests/golden/make_reference_pins.py [REFERENCE_ROOT]
"""
import gzip
import hashlib
import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
STL_RECORD = np.dtype([("normal", "<f4", 3), ("v", "<f4", 9), ("attr", "<u2")])


def read_stl(data: bytes) -> np.ndarray:
    n = struct.unpack("<I", data[80:84])[0]
    return np.frombuffer(data[84:84 + 50 * n], dtype=STL_RECORD)


def canonical_f32(tris: np.ndarray):
    """(sorted 9 x uint32 rows, the sorting permutation) of float32 triangles."""
    a = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9).view(np.uint32)
    order = np.lexsort(a.T[::-1])
    return a[order], order


def f32_digests(tris: np.ndarray, normals: np.ndarray):
    rows, order = canonical_f32(tris)
    nrm = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)[order]
    return (hashlib.sha256(rows.tobytes()).hexdigest(),
            hashlib.sha256(np.ascontiguousarray(nrm).tobytes()).hexdigest())


def grouping_signature(tris, depth=3):
    """Top of a GroupTriangles hierarchy of (T, 9) triangles in grouped
    order: per node above `depth` (preorder), the axes whose midpoints
    separate its halves; per node at `depth`, its midpoint centroid."""
    t = tris.reshape(-1, 3, 3)
    mid = (t.min(1) + t.max(1)) * 0.5
    axes, cents = [], []

    def rec(lo, n, d):
        if d == depth:
            cents.append([float(x) for x in mid[lo:lo + n].mean(0)])
            return
        h = n // 2
        axes.append([a for a in range(3) if mid[lo:lo + h, a].max() <= mid[lo + h:lo + n, a].min()])
        rec(lo, h, d + 1)
        rec(lo + h, n - h, d + 1)

    rec(0, len(mid), 0)
    return {"depth": depth, "separating_axes": axes, "centroids": cents}


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    data = os.path.join(ref, "model3d", "test_data")
    out = {}

    h = read_stl(gzip.open(os.path.join(data, "hierarchy_test.stl.gz")).read())
    tri_sha, nrm_sha = f32_digests(h["v"], h["normal"])
    out["hierarchy_test"] = {
        "source": "model3d/test_data/hierarchy_test.stl.gz",
        "made_by": "MarchingCubesSearch(solid, 0.03, 2) + SaveGroupedSTL (model3d/mesh_hierarchy_test.go:104-127)",
        "delta": 0.03, "iters": 2, "triangles": int(len(h)),
        "sha256_f32_triangles": tri_sha, "sha256_f32_normals": nrm_sha,
    }

    out["hierarchy_test_grouping"] = grouping_signature(np.ascontiguousarray(h["v"]).astype(np.float64))

    k = read_stl(open(os.path.join(data, "non_intersecting_hook.stl"), "rb").read())
    v = np.ascontiguousarray(k["v"]).reshape(-1, 3)
    uniq, inv = np.unique(v.view(np.dtype((np.void, 12))).ravel(), return_inverse=True)
    verts = np.frombuffer(uniq.tobytes(), dtype="<f4").reshape(-1, 3)
    faces = inv.reshape(-1, 3).astype(np.int32)
    assert np.array_equal(verts[faces].reshape(-1, 9).view(np.uint32), k["v"].view(np.uint32))
    np.savez_compressed(os.path.join(HERE, "non_intersecting_hook.npz"), vertices=verts, faces=faces)
    out["non_intersecting_hook"] = {
        "source": "model3d/test_data/non_intersecting_hook.stl",
        "triangles": int(len(k)),
        "sha256_f32_file_order": hashlib.sha256(np.ascontiguousarray(k["v"]).tobytes()).hexdigest(),
    }

    with open(os.path.join(HERE, "reference_meshes.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
