"""The integer-pipe division (amrsolver_gb300/csrc/ddiv.cuh) on the host:
compiled with g++ and compared bit for bit with the host's IEEE division
over random operands (the WENO weight and normalisation ranges, arbitrary
bit patterns, significands near all-ones and powers of two, quotients next
to rounding boundaries) and special values.  The device build of the same
header is checked against CUDA's division in tests/test_gpu_ddiv.py."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("ddiv") / "ddiv_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-o", out, os.path.join(HERE, "cpp", "ddiv_check.cpp")])
    return out


@pytest.mark.parametrize("seed", [11, 12])
def test_ddiv_matches_ieee_division(exe, seed):
    r = subprocess.run([exe, "10000000", str(seed)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0 checked" in r.stdout
