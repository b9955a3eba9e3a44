"""Opt-in non-finite detection (amrs_set_check_nonfinite).

The reference carries NaNs on silently (its printTotal shows -nan and the
run goes on).  With the check on, a NaN written into the state from the host
makes the next stage's output non-finite, and amrs_sync_check reports
AMRS_ERR_NONFINITE once; the flag is then clear.  With the check off nothing
is reported, and with it on a clean run gives the same bits as without.
"""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def _tgv_level(n=16):
    U, dx = P.tgv(n, mach=0.1)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    return cns.CNSLevel(sc, P.Closures.nondimensional(1.0 / 400.0), U, dx), U, dx


def test_per_box_steps_report_nan_once():
    lev, U, _ = _tgv_level()
    lev.h.set_check_nonfinite(True)
    lev.advance(lev.time, 1e-3)
    lev.h.sync_check()  # clean
    # a NaN written into one valid cell from the host
    lev.S[2, 8, 9, 10] = float("nan")
    lev.advance(lev.time, 1e-3)
    with pytest.raises(capi.AmrsError, match="non-finite value"):
        lev.h.sync_check()
    lev.h.sync_check()  # reported once, then clear
    # without the check the same NaN goes by silently, as in the reference
    lev2, _, _ = _tgv_level()
    lev2.S[2, 8, 9, 10] = float("nan")
    lev2.advance(lev2.time, 1e-3)
    lev2.h.sync_check()
    assert not bool(torch.isfinite(lev2.valid()).all())


def test_check_does_not_change_bits():
    a, _, _ = _tgv_level(24)
    b, _, _ = _tgv_level(24)
    b.h.set_check_nonfinite(True)
    for _ in range(3):
        a.advance(a.time, 1e-3)
        b.advance(b.time, 1e-3)
    a.h.sync_check()
    b.h.sync_check()
    assert torch.equal(a.valid(), b.valid())


@pytest.mark.parametrize("scheme", [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=2, rhs_visc=1)])
def test_box_list_graph_reports_nan(scheme):
    specs, fields, dx = P.batched_boxes(nboxes=6, seed=5, edges=(8, 16))
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(**scheme)
    dxinv = [1.0 / v for v in dx]
    h = capi.Handle(sc, cl)
    slots = [[torch.from_numpy(U).cuda() for _ in range(3)] for U in fields]
    bl = capi.BoxList(h, [s.lo for s in specs], slots, dxinv)
    bl.step(3, 3, 1e-4, use_graph=True)  # recorded without the check
    h.sync_check()
    h.set_check_nonfinite(True)
    bl.step(3, 3, 1e-4, use_graph=True)  # re-recorded with it
    h.sync_check()
    slots[4][0][1, 5, 5, 5] = float("inf")
    bl.step(3, 3, 1e-4, use_graph=True)
    with pytest.raises(capi.AmrsError, match="non-finite value"):
        h.sync_check()
    h.sync_check()
    bl.close()
    h.close()
