"""The FP32 screen of the flux rejection test (puncpp_gb300/csrc/pg_screen.h)
never contradicts the exact FP64 test, also at the acceptance boundary, and
leaves almost every random candidate decided (so the FP64 path is rare)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_screen_agrees_with_the_fp64_test(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = tmp_path / "screen_check"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                        "-I" + os.path.join(ROOT, "puncpp_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cpp", "screen_check.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    total, bad, undecided, rnd, rnd_undecided = (int(x) for x in out.stdout.split())
    assert out.returncode == 0 and bad == 0, out.stdout
    assert total > 5_000_000 and rnd >= 700_000
    assert rnd_undecided < 1e-4 * rnd
