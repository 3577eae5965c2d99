"""The C ABI library: loads without a GPU, exports what include/mcgpu.h
declares, and its host-only entry points agree with the oracle.  CPU only."""
import os
import re

import numpy as np
import pytest

from model3d_gb300 import _native as N
from model3d_gb300 import case_table, spacer_axis, MCError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "mcgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mc_[a-z_]+)\s*\(", src)))


def test_library_loads_and_exports_header_symbols():
    L = N.lib()
    names = _declared()
    assert "mc_search" in names and "mc_solid_create" in names
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/mcgpu.h but not exported"
    assert set(names) <= set(N.EXPORTS) | set(names)
    assert L.mc_version().decode().startswith("mcgpu")


def test_case_table_matches_oracle(oracle):
    c1, t1 = case_table()
    c2, t2, conflicts, covered = oracle.case_table()
    assert (c1 == c2).all()
    assert (t1 == t2).all()


def test_spacer_matches_oracle(oracle):
    rng = np.random.default_rng(2)
    cases = [(-1.0, 1.0, 0.01), (-1.3, 1.27, 0.004), (0.0, 0.0, 0.1), (-5.1, 3.7, 0.033)]
    for _ in range(20):
        lo = rng.normal() * 3
        cases.append((lo, lo + abs(rng.normal()) * 2, 10 ** rng.uniform(-3, -1)))
    for lo, hi, d in cases:
        a = spacer_axis(lo, hi, d)
        b = oracle.spacer_axis(lo, hi, d)
        assert len(a) == len(b)
        assert (a.view(np.uint64) == b.view(np.uint64)).all()


def test_spacer_rejects_non_terminating_loops():
    for lo, hi, d in [(0.0, 1.0, 0.0), (0.0, 1.0, -0.1), (1e17, 1e17 + 10, 1.0), (0.0, 1.0, float("nan"))]:
        with pytest.raises(MCError) as e:
            spacer_axis(lo, hi, d)
        assert e.value.status == N.MC_ERR_GRID


def test_status_strings_carry_reference_panics():
    assert N.status_string(N.MC_ERR_BOUNDS_INSIDE) == "solid is true outside of bounds"
    assert N.status_string(N.MC_ERR_NOT_ON_EDGE) == "vertex not on edge"
