"""The host graph build (structure.cpp build_window) against a brute-force restatement on seeded
random windows: active edges and their point-major order, free cameras and points, and the Schur
pair and block counts that size the device work (CPU only: the C++ checker is compiled here)."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "nav24_gb300" / "csrc"


def test_build_window_matches_brute_force(tmp_path):
    from nav24_gb300.build import cuda_home
    exe = tmp_path / "structure_check"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(CSRC), "-I", str(ROOT / "include"),
           "-I", str(cuda_home() / "include"), str(ROOT / "tests" / "host" / "structure_check.cpp"),
           str(CSRC / "structure.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("compile failed:\n" + r.stderr[-2000:])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok 2000", out.stdout
