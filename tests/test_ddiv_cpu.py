"""The integer-pipe division, square root and product
(amrsolver_gb300/csrc/ddiv.cuh) on the host: compiled with g++ and compared
bit for bit with the host's IEEE division, square root and multiplication
over random operands (for the division: the WENO weight and normalisation
ranges, arbitrary bit patterns, significands near all-ones and powers of
two, quotients next to rounding boundaries; for the square root: arbitrary
bits, the whole exponent range, squares and their neighbours; for the
product: arbitrary bits, short significands whose products fall on rounding
ties, exponent sums at the edges of underflow and overflow, zeros,
subnormals and specials) and special values.  The device build of the same
header is checked against CUDA's division, square root and product in
tests/test_gpu_ddiv.py."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exes(tmp_path_factory):
    d = tmp_path_factory.mktemp("ddiv")
    out = {}
    for name in ("ddiv_check", "dsqrt_check", "dmul_check"):
        out[name] = str(d / name)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-o", out[name], os.path.join(HERE, "cpp", name + ".cpp")])
    return out


@pytest.mark.parametrize("seed", [11, 12])
def test_ddiv_matches_ieee_division(exes, seed):
    r = subprocess.run([exes["ddiv_check"], "10000000", str(seed)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0 checked" in r.stdout


@pytest.mark.parametrize("seed", [13, 14])
def test_dsqrt_matches_ieee_sqrt(exes, seed):
    r = subprocess.run([exes["dsqrt_check"], "10000000", str(seed)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0 checked" in r.stdout


@pytest.mark.parametrize("seed", [15, 16])
def test_dmul_matches_ieee_product(exes, seed):
    r = subprocess.run([exes["dmul_check"], "10000000", str(seed)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0 checked" in r.stdout
