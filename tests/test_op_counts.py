"""The committed op-count polynomials (tests/golden/op_counts.json, read by
bench.py for the roofline) equal the oracle's op-counting scalar at box
sizes outside the fit."""
import json
import os

import pytest

from amrsolver_gb300 import problems as P
from tests.golden import make_op_counts as M

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("n", [7, 16])
def test_op_count_polynomials_match_oracle(orc, n):
    data = json.load(open(os.path.join(HERE, "golden", "op_counts.json")))
    for name, ent in data["schemes"].items():
        got = M.counts(orc, ent["switches"], n)
        for ph, c in ent["phases"].items():
            assert c[0] * n ** 3 + c[1] * n ** 2 + c[2] * n + c[3] == got[ph], (name, ph)


def test_op_count_schemes_cover_bench():
    data = json.load(open(os.path.join(HERE, "golden", "op_counts.json")))
    assert {"keep4_visc", "weno_visc"} <= set(data["schemes"])
    assert P.Scheme(**data["schemes"]["weno_visc"]["switches"]).flux_euler == 2


def test_data_dependent_counts_match_oracle(orc):
    """The Riemann-solver schemes' counts depend on the data; the committed
    figures are the oracle's counts of the bench input's first RHS."""
    data = json.load(open(os.path.join(HERE, "golden", "op_counts.json")))
    assert {"muscl_visc", "weno_riemann_visc"} <= set(data["data_dependent"])
    for name, ent in data["data_dependent"].items():
        assert P.Scheme(**ent["switches"]).flux_euler not in (1, 2), name  # the Riemann path
        got = M.tgv_counts(orc, ent["switches"], ent["n"], ent["tgv_mach"], ent["mu"])
        assert got == ent["phases"], name
