"""The reference's main loop as one device launch (amrs_rk_run_boxlist): a
conditional WHILE graph node repeats one RK step with the reference's dt
control computed on the device; and the conserved totals reduction."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import problems as P
from tests import golden_io as G

pytestmark = pytest.mark.gpu
NG = P.NGHOST


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def one_box_list(sc, cl, U, dx, bc):
    h = capi.Handle(sc, cl)
    t = torch.from_numpy(U).cuda()
    slots = [[t, t.clone(), t.clone()]]
    bl = capi.BoxList(h, [(0, 0, 0)], slots, [1.0 / v for v in dx])
    n = (U.shape[3] - 2 * NG, U.shape[2] - 2 * NG, U.shape[1] - 2 * NG)
    bl.set_domain((0, 0, 0), n, bc, bc)
    return h, bl, slots


def test_run_fixed_dt_equals_single_steps():
    U, dx = P.tgv(24, mach=0.2)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    bc = (-1, -1, -1)
    h, bl, slots = one_box_list(sc, cl, U, dx, bc)
    bl.run(3, 3, stop_time=1e9, max_steps=5, dt=1e-3)
    t, dt, steps = bl.run_state()
    assert steps == 5 and dt == 1e-3
    tt = 0.0
    for _ in range(5):
        tt = tt + 1e-3
    assert t == tt
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=bc, bc_hi=bc)
    for _ in range(5):
        lev.advance(lev.time, 1e-3)
    h.sync_check()
    np.testing.assert_array_equal(slots[0][0][:, NG:-NG, NG:-NG, NG:-NG].cpu().numpy(), lev.valid().cpu().numpy())


def test_run_sod_cfl_to_stop_time_matches_oracle(orc):
    """Sod tube to t = 0.2 at CFL 0.3 with the reference's dt control, all
    on the device, against the oracle's loop."""
    cl = P.Closures.air_sutherland()
    sc = P.Scheme(flux_euler=2, rhs_visc=0)
    U, dx = P.sod(256, 8, 8)
    bc = (2, -1, -1)
    h, bl, slots = one_box_list(sc, cl, U, dx, bc)
    stop, cfl = 0.2, 0.3
    bl.run(3, 3, stop_time=stop, max_steps=2000, cfl=cfl)
    t, dt_last, steps = bl.run_state()
    h.sync_check()
    dxinv = [1.0 / v for v in dx]
    S, tt = U, 0.0
    odt = orc.est_timestep(cl, S, dx, cfl)
    nst = 0
    while tt < stop and nst < 2000:
        S = orc.advance(sc, cl, S, dxinv, bc, bc, odt, nthreads=8)
        tt = tt + odt
        nst += 1
        Sv = S.copy()
        orc.fill_halo(Sv, bc, bc)
        dt_min = min(orc.est_timestep(cl, Sv, dx, cfl), 1.1 * odt)
        eps = 0.001 * dt_min
        odt = stop - tt if tt + dt_min > stop - eps else dt_min
    assert steps == nst
    assert t == tt
    assert G.relmax(slots[0][0][:, NG:-NG, NG:-NG, NG:-NG].cpu().numpy(), P.valid(S)) <= 1e-13


def test_run_resumes_and_stops_at_max_steps():
    U, dx = P.tgv(16, mach=0.2)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    bc = (-1, -1, -1)
    ha, bla, sla = one_box_list(sc, cl, U, dx, bc)
    bla.run(3, 3, stop_time=1.0, max_steps=7, cfl=0.5)
    ta, _, na = bla.run_state()
    hb, blb, slb = one_box_list(sc, cl, U, dx, bc)
    blb.run(3, 3, stop_time=1.0, max_steps=3, cfl=0.5)
    tb, dtb, nb = blb.run_state()
    assert nb == 3
    # resuming restarts the dt control (computeInitialDt), as a restarted reference run would
    blb.run(3, 3, stop_time=1.0, max_steps=4, cfl=0.5, time=tb)
    tb2, _, nb2 = blb.run_state()
    assert na == 7 and nb2 == 4
    ha.sync_check()
    hb.sync_check()
    a = sla[0][0][:, NG:-NG, NG:-NG, NG:-NG].cpu().numpy()
    b = slb[0][0][:, NG:-NG, NG:-NG, NG:-NG].cpu().numpy()
    assert np.isfinite(a).all() and np.isfinite(b).all()
    # an inactive run (time already at the stop) changes nothing
    before = slb[0][0].clone()
    blb.run(3, 3, stop_time=tb2, max_steps=10, cfl=0.5, time=tb2)
    assert blb.run_state()[2] == 0
    assert torch.equal(before, slb[0][0])


def test_level_run_and_totals():
    """A periodic level of 8 uneven boxes: the device loop against one box,
    and the totals reduction against numpy, conserved to round-off."""
    n = 32
    U, dx = P.tgv(n, mach=0.2)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    bc = (-1, -1, -1)
    h = capi.Handle(sc, cl)
    edges = [(0, 12, 32), (0, 20, 32), (0, 9, 32)]
    los, slots = [], []
    for z0, z1 in zip(edges[2][:-1], edges[2][1:]):
        for y0, y1 in zip(edges[1][:-1], edges[1][1:]):
            for x0, x1 in zip(edges[0][:-1], edges[0][1:]):
                B = np.ascontiguousarray(U[:, z0:z1 + 2 * NG, y0:y1 + 2 * NG, x0:x1 + 2 * NG])
                t = torch.from_numpy(B).cuda()
                slots.append([t, t.clone(), t.clone()])
                los.append((x0, y0, z0))
    bl = capi.BoxList(h, los, slots, [1.0 / v for v in dx])
    bl.set_domain((0, 0, 0), (n, n, n), bc, bc)
    vol = (2 * np.pi) ** 3
    tot0 = bl.totals(0, vol, torch.zeros(5, dtype=torch.float64, device="cuda")).cpu().numpy()
    ref0 = P.valid(U).reshape(5, -1).sum(axis=1) * vol
    np.testing.assert_allclose(tot0, ref0, rtol=1e-13, atol=1e-13 * np.abs(ref0).max())
    bl.run(3, 3, stop_time=1e9, max_steps=4, dt=2e-3)
    lev = cns.CNSLevel(sc, cl, U, dx)
    for _ in range(4):
        lev.advance(lev.time, 2e-3)
    ref = lev.valid().cpu().numpy()
    out = np.empty_like(ref)
    for lo, sl in zip(los, slots):
        V = sl[0][:, NG:-NG, NG:-NG, NG:-NG].cpu().numpy()
        x0, y0, z0 = lo
        out[:, z0:z0 + V.shape[1], y0:y0 + V.shape[2], x0:x0 + V.shape[3]] = V
    np.testing.assert_array_equal(out, ref)
    tot1 = bl.totals(0, vol, torch.zeros(5, dtype=torch.float64, device="cuda")).cpu().numpy()
    scale = np.abs(P.valid(U)).reshape(5, -1).sum(axis=1) * vol
    # momentum components share one scale (w is zero initially)
    scale[1:4] = scale[1:4].max()
    assert np.all(np.abs(tot1 - tot0) <= 1e-13 * scale), (tot1 - tot0, scale)
    h.sync_check()


def test_step_graph_serves_changing_dt():
    """The step graph reads dt from device memory: one capture, three dts."""
    U, dx = P.tgv(16, mach=0.2)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    bc = (-1, -1, -1)
    h, bl, slots = one_box_list(sc, cl, U, dx, bc)
    lev = cns.CNSLevel(sc, cl, U, dx)
    s1, w1, w2 = 0, 1, 2
    for dt in (1e-3, 2.5e-3, 7e-4, 1e-3):
        r = bl.step(3, 3, dt, s1, w1, w2, use_graph=True)
        # copy the result back so that the same graph (same slots) is replayed
        slots[0][s1][:] = slots[0][r]
        lev.advance(lev.time, dt)
    h.sync_check()
    np.testing.assert_array_equal(slots[0][s1][:, NG:-NG, NG:-NG, NG:-NG].cpu().numpy(), lev.valid().cpu().numpy())
