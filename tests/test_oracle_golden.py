"""The CPU oracle against golden vectors produced by the reference build.

The golden vectors in tests/golden/ were written by tests/golden/make_golden.py
from oracle/_ref, i.e. from the reference's own src/tim/CNS_advance.cpp and
kernel headers compiled here.  On x86-64 with glibc the restatement matches
them bit for bit; elsewhere libm differences (pow in the WENO weights) may
move the last bit, hence the 1e-13 bound.
"""
import numpy as np
import pytest

from amrsolver_gb300 import problems as P
from tests import golden_io as G

TOL = 1e-13


@pytest.mark.parametrize("case", G.rhs_cases(), ids=lambda c: c["name"])
def test_rhs_golden(orc, case):
    R = orc.rhs(case["scheme"], case["closures"], case["U"], case["dxinv"], lo=case["lo"])
    assert G.relmax(R, case["dSdt"]) <= TOL


@pytest.mark.parametrize("case", G.wall_cases(), ids=lambda c: c["name"])
def test_rhs_walls_golden(orc, case):
    R = orc.rhs(case["scheme"], case["closures"], case["U"], case["dxinv"], lo=case["lo"], walls=case["walls"])
    assert G.relmax(R, case["dSdt"]) <= TOL


@pytest.mark.parametrize("case", G.adv_cases(), ids=lambda c: c["name"])
def test_advance_golden(orc, case):
    cl = G.closures("const")
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    S2 = orc.advance(sc, cl, case["U"], case["dxinv"], (-1, -1, -1), (-1, -1, -1), case["dt"], case["order_rk"],
                     case["stages_rk"])
    assert G.relmax(P.valid(S2), case["S2"]) <= TOL


def test_sod_step_golden(orc):
    z = np.load(G.HERE + "/sod_step.npz")
    cl = G.closures("suth")
    dt = orc.est_timestep(cl, z["U"], z["dx"], 0.3)
    assert dt == pytest.approx(float(z["dt"]), rel=1e-15)
    sc = P.Scheme(flux_euler=2, rhs_visc=0)
    S2 = orc.advance(sc, cl, z["U"], [1.0 / h for h in z["dx"]], (2, -1, -1), (2, -1, -1), float(z["dt"]), 3, 3)
    assert G.relmax(P.valid(S2), z["S2"]) <= TOL


def test_halo_golden(orc):
    z = np.load(G.HERE + "/halo.npz")
    for tag in ("outflow", "walls", "periodic"):
        A = z["V"].copy()
        bc = z["bc_" + tag]
        orc.fill_halo(A, tuple(bc[0]), tuple(bc[1]))
        np.testing.assert_array_equal(A, z["U_" + tag])
