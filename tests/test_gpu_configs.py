"""Whole-run checks of the configurations the path is measured on.

* Sod tube 256x8x8 (outflow x, periodic y/z), WENO5-JS LLF inviscid, SSPRK3,
  CFL 0.3 with the reference's dynamic dt control, to t = 0.2: every dt and
  the final per-cell state against the CPU oracle run the same way.
* Taylor-Green 64^3 (M=0.1, Re=1600), KEEP4 + viscous, 100 SSPRK3 steps:
  kinetic-energy and enstrophy series and the final state against the oracle.
* Autotuner: tuned tiles on a box list keep the bits.
"""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import autotune, capi, cns
from amrsolver_gb300 import problems as P
from tests import golden_io as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def test_sod_to_t02(orc):
    cl = P.Closures.air_sutherland()
    sc = P.Scheme(flux_euler=2, rhs_visc=0)
    U, dx = P.sod(256, 8, 8)
    bc = (2, -1, -1)
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=bc, bc_hi=bc)
    stop, cfl = 0.2, 0.3
    # GPU run with the reference's dt control (src/CNS.cpp:282-377)
    dts = []
    dt = lev.compute_initial_dt(cfl)
    while lev.time < stop and len(dts) < 2000:
        dts.append(dt)
        lev.advance(lev.time, dt)
        dt = lev.compute_new_dt(cfl, dt, stop)
    gpu = lev.valid().cpu().numpy()
    # oracle run, same control flow
    dxinv = [1.0 / h for h in dx]
    S = U
    t = 0.0
    odt = orc.est_timestep(cl, S, dx, cfl)
    odts = []
    while t < stop and len(odts) < 2000:
        odts.append(odt)
        S = orc.advance(sc, cl, S, dxinv, bc, bc, odt, nthreads=8)
        t = t + odt
        g = 3
        Sv = S.copy()
        orc.fill_halo(Sv, bc, bc)
        dt_min = min(orc.est_timestep(cl, Sv, dx, cfl), 1.1 * odt)
        eps = 0.001 * dt_min
        odt = stop - t if t + dt_min > stop - eps else dt_min
    assert len(dts) == len(odts)
    np.testing.assert_allclose(dts, odts, rtol=1e-12, atol=0)
    assert abs(lev.time - 0.2) < 1e-12
    assert G.relmax(gpu, P.valid(S)) <= 1e-10
    # the shock has formed: density jump of the Sod solution present
    rho = gpu[0, 4, 4, :]
    assert rho.max() > 0.9 and rho.min() < 0.2


def ke_enstrophy(Uv, dx):
    rho = Uv[0]
    u, v, w = Uv[1] / rho, Uv[2] / rho, Uv[3] / rho
    ke = np.mean(0.5 * rho * (u * u + v * v + w * w))

    def d(f, axis, h):  # axes of the (z, y, x) array; periodic central difference
        return (np.roll(f, -1, axis) - np.roll(f, 1, axis)) / (2 * h)

    ox = d(w, 1, dx[1]) - d(v, 0, dx[2])
    oy = d(u, 0, dx[2]) - d(w, 2, dx[0])
    oz = d(v, 2, dx[0]) - d(u, 1, dx[1])
    ens = np.mean(0.5 * rho * (ox * ox + oy * oy + oz * oz))
    return ke, ens


def test_tgv_ke_enstrophy_series(orc):
    n, steps, dt = 64, 100, 2e-3
    U, dx = P.tgv(n, mach=0.1)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    lev = cns.CNSLevel(sc, cl, U, dx)
    dxinv = [1.0 / h for h in dx]
    S = U
    series_gpu, series_orc = [], []
    for s in range(steps):
        lev.advance(lev.time, dt)
        S = orc.advance(sc, cl, S, dxinv, (-1, -1, -1), (-1, -1, -1), dt, nthreads=8)
        if s % 10 == 9:
            series_gpu.append(ke_enstrophy(lev.valid().cpu().numpy(), dx))
            series_orc.append(ke_enstrophy(P.valid(S), dx))
    lev.h.sync_check()
    assert series_gpu == series_orc
    np.testing.assert_array_equal(lev.valid().cpu().numpy(), P.valid(S))
    # decay of kinetic energy, growth of enstrophy early in the TGV
    assert series_gpu[-1][0] < series_gpu[0][0] and series_gpu[-1][1] > series_gpu[0][1]


def test_autotuner_keeps_bits(orc, tmp_path):
    specs, fields, dx = P.batched_boxes(nboxes=6, seed=21, edges=(8, 24, 48))
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / v for v in dx]
    h = capi.Handle(sc, cl)
    slots_a = [[torch.from_numpy(U).cuda() for _ in range(3)] for U in fields]
    slots_b = [[torch.from_numpy(U).cuda() for _ in range(3)] for U in fields]
    bl_a = capi.BoxList(h, [s.lo for s in specs], slots_a, dxinv)
    bl_b = capi.BoxList(h, [s.lo for s in specs], slots_b, dxinv)
    choice = autotune.tune_boxlist(bl_b, specs, cache_path=str(tmp_path / "tune.json"), nz_probe=16)
    assert set(choice) == {(s.shape[0], s.shape[1]) for s in specs}
    ra = bl_a.step(3, 3, 1e-3, use_graph=True)
    rb = bl_b.step(3, 3, 1e-3, use_graph=True)
    h.sync_check()
    for b in range(len(specs)):
        np.testing.assert_array_equal(slots_a[b][ra][:, 3:-3, 3:-3, 3:-3].cpu().numpy(),
                                      slots_b[b][rb][:, 3:-3, 3:-3, 3:-3].cpu().numpy())
