"""The reverse of the two-shock Riemann solver that the MUSCL-Riemann
adjoint kernel runs (amrsolver_gb300/csrc/riemann_vjp.cuh, host- and
device-callable) against the oracle's forward-mode dual numbers, on the CPU:
100k random Riemann problems, every branch of the solver (shock or
rarefaction each side, sign of u*, supersonic side state, star state,
transonic fan)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_riemann_vjp_matches_dual_numbers(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "riemann_vjp_check")
    src = os.path.join(ROOT, "tests", "cpp", "riemann_vjp_check.cpp")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe, src], check=True)
    out = subprocess.run([exe, "100000"], capture_output=True, text=True, check=True).stdout.split()
    worst, nbad = float(out[0]), int(out[1])
    assert nbad == 0 and worst <= 1e-11, (worst, nbad)
