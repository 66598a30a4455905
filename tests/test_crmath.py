"""Host check of the correctly rounded float exp/log of the LBP normalisation
(bp-layers_gb300/csrc/bpl_crmath.cuh): whenever the float-float fast path
returns a value it equals the reference expression (float)exp((double)x) /
(float)log((double)s); undecided roundings fall back to that expression."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fast_exp_log_match_double_rounding(tmp_path):
    exe = str(tmp_path / "crmath_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                           os.path.join(ROOT, "tests", "crmath", "crmath_check.cpp")])
    r = subprocess.run([exe, "400000", "7"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
