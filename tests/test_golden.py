"""Golden fixtures (tests/golden/meshes.json, made by
tests/golden/make_golden.py from the oracle): SHA-256 digests of canonical
meshes of small seeded workloads and of the case table.  The oracle must
reproduce them (CPU), and so must the CUDA path in both precisions (GPU)."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

GOLD = json.load(open(os.path.join(HERE, "golden", "meshes.json")))
CASES = G.cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(oracle, name):
    solid, delta, iters = CASES[name]
    m = oracle.mc_search(*G.serialize(solid), delta, iters)
    assert len(m["tris"]) == GOLD[name]["triangles"]
    assert m["n_vertices"] == GOLD[name]["vertices"]
    assert G.digest(m["tris"]) == GOLD[name]["sha256"]


def test_case_table_golden(oracle):
    from model3d_gb300 import case_table
    for counts, tris in (oracle.case_table()[:2], case_table()):
        h = hashlib.sha256(np.ascontiguousarray(counts, dtype=np.uint8).tobytes() +
                           np.ascontiguousarray(tris, dtype=np.uint8).tobytes()).hexdigest()
        assert h == GOLD["case_table"]["sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_reproduces_golden(prec):
    from model3d_gb300 import MarchingCubesSearch
    for name, (solid, delta, iters) in sorted(CASES.items()):
        m = MarchingCubesSearch(solid, delta, iters, precision=prec)
        assert m.NumTriangles() == GOLD[name]["triangles"], name
        assert G.digest(m.TriangleSoup()) == GOLD[name]["sha256"], name
