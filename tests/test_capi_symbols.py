"""The C-ABI library loads and exports every entry point its header declares
(no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

from amrsolver_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "amrs_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(amrs_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = header_symbols()
    assert "amrs_rhs_box" in syms and "amrs_rk_stage_box" in syms and len(syms) >= 15


def test_library_exports_every_header_symbol(lib):
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    assert set(header_symbols()) == set(capi.SIGNATURES)


def test_rk_program_matches_oracle_stage_counts():
    # host-only entry point: no device work
    for (o, s, n) in [(3, 3, 3), (3, 4, 4), (2, 5, 5), (1, 1, 1), (0, 1, 1), (-2, 2, 2)]:
        assert len(capi.rk_program(o, s, 0.1)) == n
    with pytest.raises(capi.AmrsError):
        capi.rk_program(3, 5, 0.1)
    with pytest.raises(capi.AmrsError):
        capi.rk_program(4, 1, 0.1)
