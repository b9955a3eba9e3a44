"""CNS::printTotal's primitive extrema and convective CFL table on the device
(amrs_boxlist_prim_stats, amrs_prim_stats_box) against the oracle, whose
table is pinned to the reference's own pointCFL (src/cls/CNS_K.h:49-59).

A level's statistics combine its boxes' exactly: min of the minima, max of
the maxima and of the table entries (the CFL entry max(A0, A1) dt / dx of
the global maxima equals the maximum of the boxes' entries because rounding
is monotonic).
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


def combine(stats):
    s = np.array(stats)
    return np.concatenate([s[:, :6].min(axis=0), s[:, 6:12].max(axis=0), s[:, 12:].max(axis=0)])


def test_box_list_stats_bitexact(orc):
    specs, fields, dx = P.batched_boxes(nboxes=12, seed=31, edges=(8, 16, 24))
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    h = capi.Handle(sc, cl)
    slots = [[torch.from_numpy(U).cuda() for _ in range(3)] for U in fields]
    bl = capi.BoxList(h, [s.lo for s in specs], slots, [1.0 / v for v in dx])
    dt = 2.5e-3
    out = torch.empty(21, dtype=torch.float64, device="cuda")
    bl.prim_stats(0, dx, dt, out)
    h.sync_check()
    ref = combine([orc.prim_stats(cl, U, dx, dt, lo=s.lo) for s, U in zip(specs, fields)])
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    # slot -1: the primitives of the stage input the last RHS read
    prog = capi.rk_program(3, 3, dt)[0]
    bl.stage(prog, 0, 0, 1)
    got = bl.prim_stats(-1, dx, dt, torch.empty_like(out)).cpu().numpy()
    np.testing.assert_array_equal(got, ref)
    # and of the stage's output state
    out1 = bl.prim_stats(1, dx, dt, torch.empty_like(out)).cpu().numpy()
    h.sync_check()
    valid1 = [slots[b][1].cpu().numpy() for b in range(len(specs))]
    ref1 = combine([orc.prim_stats(cl, U, dx, dt, lo=s.lo) for s, U in zip(specs, valid1)])
    np.testing.assert_array_equal(out1, ref1)
    bl.close()


def test_ensemble_per_member_closures(orc):
    members = P.ensemble_members(5, seed=9)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    fields, cls, los, slots = [], [], [], []
    for b, (m, re) in enumerate(members):
        U, dx = P.tgv(12, mach=m)
        cl = P.Closures.nondimensional(1.0 / re)
        cl.gamma = 1.3 + 0.05 * b  # the sound speed uses each member's own gas
        cl.cv = cl.Rspec / (cl.gamma - 1.0)
        cl.cp = cl.cv + cl.Rspec
        fields.append(U)
        cls.append(cl)
        los.append((b * 40, 0, 0))
        slots.append([torch.from_numpy(U).cuda() for _ in range(3)])
    h = capi.Handle(sc, cls[0])
    bl = capi.BoxList(h, los, slots, [1.0 / v for v in dx], closure_index=list(range(5)), closures=cls)
    out = bl.prim_stats(0, dx, 1e-3, torch.empty(21, dtype=torch.float64, device="cuda")).cpu().numpy()
    h.sync_check()
    ref = combine([orc.prim_stats(c, U, dx, 1e-3, lo=lo) for c, U, lo in zip(cls, fields, los)])
    np.testing.assert_array_equal(out, ref)
    bl.close()


def test_level_print_total(orc):
    U, dx = P.tgv(24, mach=0.2)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    lev = cns.CNSLevel(P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1), cl, U, dx)
    for _ in range(2):
        lev.advance(lev.time, 2e-3)
    rep = lev.print_total(2e-3)
    lev.h.sync_check()
    ref = orc.prim_stats(cl, lev.state_host(), dx, 2e-3)
    np.testing.assert_array_equal(np.array([rep[k] for k in capi.PRIM_STATS_KEYS]), ref)
    assert rep["cfl_x"] < 1.0 and len(rep["totals"]) == 5
