"""Host logic of the device program: constant folding of culled leaves.

tests/csrc/fold_check.cpp lowers 3000 random Solid trees with the library's
own lowering (mc_lower.cpp), folds each under 20 random active-leaf sets and
checks that the folded program evaluates like the full program.  CPU only.
"""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fold_matches_full_program(tmp_path):
    exe = tmp_path / "fold_check"
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-o", str(exe),
                    os.path.join(ROOT, "tests", "csrc", "fold_check.cpp"),
                    os.path.join(ROOT, "model3d_gb300", "csrc", "mc_lower.cpp")], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout


def test_bisection_bit_arithmetic(tmp_path):
    """mid_bits / float_bits_of (integer midpoint and float rounding used by
    the search) equal IEEE (f + t) * 0.5 and (float)x on 5.5M cases."""
    exe = tmp_path / "bits_check"
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-o", str(exe),
                    os.path.join(ROOT, "tests", "csrc", "bits_check.cpp")], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " bad 0" in r.stdout
