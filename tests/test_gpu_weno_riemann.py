"""WENO5-Riemann (riemann_weno = 1): WENO5-JS reconstructed primitive states
fed to the reference's two-shock Riemann solver.  The reference has no such
scheme (it pairs WENO5 with the Lax-Friedrichs split only), so parity is
against the oracle's restatement of the extension (unpinned against the
reference), and the physics is checked on the Sod tube against the exact
Riemann solution."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import problems as P
from tests import golden_io as G

pytestmark = pytest.mark.gpu
WENO_TOL = 1e-13  # weno5js squares with pow(x, 2) in the oracle and x*x here


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def gpu_rhs(scheme, closures, U, dxinv, lo=(0, 0, 0)):
    h = capi.Handle(scheme, closures)
    n = tuple(s - 6 for s in U.shape[1:])
    out = torch.full((5,) + n, float("nan"), dtype=torch.float64, device="cuda")
    h.rhs_box(torch.from_numpy(np.ascontiguousarray(U)).cuda(), dxinv, out, lo=lo)
    h.sync_check()
    return out.cpu().numpy()


@pytest.mark.parametrize("visc", [0, 1])
@pytest.mark.parametrize("n", [(8, 8, 8), (13, 7, 5), (37, 19, 11)])
def test_weno_riemann_vs_oracle(orc, n, visc):
    sc = P.Scheme(flux_euler=0, riemann_weno=1, rhs_visc=visc)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    U = P.random_state(n, seed=sum(n) + 11 * visc, amp=0.3)
    lo = (n[0] % 5 - 2, -n[1], 7)
    dxinv = (1.7, 2.9, 0.8)
    R = gpu_rhs(sc, cl, U, dxinv, lo)
    ref = orc.rhs(sc, cl, U, dxinv, lo=lo)
    assert np.isfinite(ref).all()
    assert G.relmax(R, ref) <= WENO_TOL


def test_weno_riemann_uniform_flow_has_zero_rhs():
    """Every face of a uniform moving state sees the same stencils, so every
    flux is the same number and the divergence is exactly zero."""
    n = (12, 10, 9)
    shape = (n[2] + 6, n[1] + 6, n[0] + 6)
    one = np.ones(shape)
    U = P.prims_to_cons(1.3 * one, 0.4 * one, -0.2 * one, 0.7 * one, 0.9 * one, 1.4)
    R = gpu_rhs(P.Scheme(flux_euler=0, riemann_weno=1, rhs_visc=1), P.Closures.nondimensional(1e-2), U, (3.0, 2.0, 1.0))
    assert np.all(R == 0.0)


def sod_exact(x, t, gamma=1.4, left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1), x0=0.5):
    """Exact solution (rho, u, p) of a Riemann problem with a two-wave
    pressure function solved by Newton's method (Toro, Riemann Solvers and
    Numerical Methods for Fluid Dynamics, ch. 4)."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = np.sqrt(gamma * pl / rl), np.sqrt(gamma * pr / rr)

    def f(p, rk, pk, ck):
        if p > pk:  # shock
            a, b = 2.0 / ((gamma + 1) * rk), (gamma - 1) / (gamma + 1) * pk
            return (p - pk) * np.sqrt(a / (p + b)), np.sqrt(a / (b + p)) * (1 - 0.5 * (p - pk) / (b + p))
        q = (p / pk) ** ((gamma - 1) / (2 * gamma))  # rarefaction
        return 2 * ck / (gamma - 1) * (q - 1), 1.0 / (rk * ck) * (p / pk) ** (-(gamma + 1) / (2 * gamma))

    p = 0.5 * (pl + pr)
    for _ in range(60):
        fl, dl = f(p, rl, pl, cl)
        fr, dr = f(p, rr, pr, cr)
        p = max(p - (fl + fr + ur - ul) / (dl + dr), 1e-12)
    fl, _ = f(p, rl, pl, cl)
    fr, _ = f(p, rr, pr, cr)
    us = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    s = (x - x0) / t
    rho, u, pres = np.empty_like(x), np.empty_like(x), np.empty_like(x)
    # left rarefaction (pl > p for the Sod data)
    rsl = rl * (p / pl) ** (1 / gamma)
    csl = cl * (p / pl) ** ((gamma - 1) / (2 * gamma))
    head, tail = ul - cl, us - csl
    # right shock
    sr = ur + cr * np.sqrt((gamma + 1) / (2 * gamma) * p / pr + (gamma - 1) / (2 * gamma))
    rsr = rr * (p / pr + (gamma - 1) / (gamma + 1)) / ((gamma - 1) / (gamma + 1) * p / pr + 1)
    for m, sv in enumerate(s):
        if sv < head:
            rho[m], u[m], pres[m] = rl, ul, pl
        elif sv < tail:
            uu = 2 / (gamma + 1) * (cl + (gamma - 1) / 2 * ul + sv)
            cc = 2 / (gamma + 1) * (cl + (gamma - 1) / 2 * (ul - sv))
            rho[m] = rl * (cc / cl) ** (2 / (gamma - 1))
            u[m], pres[m] = uu, pl * (cc / cl) ** (2 * gamma / (gamma - 1))
        elif sv < us:
            rho[m], u[m], pres[m] = rsl, us, p
        elif sv < sr:
            rho[m], u[m], pres[m] = rsr, us, p
        else:
            rho[m], u[m], pres[m] = rr, ur, pr
    return rho, u, pres


def test_sod_exact_solution_reference_values():
    rho, u, p = sod_exact(np.array([0.6, 0.8]), 0.2)
    # star region of the Sod problem: p* = 0.30313, u* = 0.92745, rho*L = 0.42632, rho*R = 0.26557
    assert abs(p[0] - 0.30313) < 1e-5 and abs(u[0] - 0.92745) < 1e-5
    assert abs(rho[0] - 0.42632) < 1e-5 and abs(rho[1] - 0.26557) < 1e-5


def run_sod(riemann_weno, nx, stop=0.2, cfl=0.3):
    cl = P.Closures.ideal_gas(gamma=1.4, mw=1.0, Ru=1.0, visc_law=0, cond_law=0)
    U, dx = P.sod(nx, 4, 4)
    bc = (2, -1, -1)
    sc = P.Scheme(flux_euler=0, riemann_weno=riemann_weno, rhs_visc=0)
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=bc, bc_hi=bc)
    dt = lev.compute_initial_dt(cfl)
    steps = 0
    while lev.time < stop and steps < 5000:
        lev.advance(lev.time, dt)
        dt = lev.compute_new_dt(cfl, dt, stop)
        steps += 1
    lev.h.sync_check()
    V = lev.valid().cpu().numpy()
    x = (np.arange(nx) + 0.5) / nx
    return x, V[0, 2, 2, :], lev.time


def test_weno_riemann_sod_converges_to_exact_solution():
    """L1 density error against the exact solution at t = 0.2 falls as the
    grid is refined (first order at the discontinuities)."""
    errs = []
    for nx in (64, 128, 256):
        x, rho, t = run_sod(1, nx)
        assert abs(t - 0.2) < 1e-12
        assert np.isfinite(rho).all() and rho.min() > 0.1 and rho.max() < 1.0 + 1e-6
        ex, _, _ = sod_exact(x, t)
        errs.append(float(np.mean(np.abs(rho - ex))))
    assert errs[1] < 0.8 * errs[0] and errs[2] < 0.8 * errs[1], errs
    assert errs[2] < 6e-3, errs


def test_weno_riemann_sod_matches_oracle_run(orc):
    """The whole Sod run (64 cells, dynamic dt, to t = 0.2) against the
    oracle's loop: same step count, same final time, states within 1e-10."""
    nx, stop, cfl = 64, 0.2, 0.3
    x, rho, t = run_sod(1, nx)
    cl = P.Closures.ideal_gas(gamma=1.4, mw=1.0, Ru=1.0, visc_law=0, cond_law=0)
    U, dx = P.sod(nx, 4, 4)
    bc = (2, -1, -1)
    sc = P.Scheme(flux_euler=0, riemann_weno=1, rhs_visc=0)
    S, tt = U, 0.0
    odt = orc.est_timestep(cl, S, dx, cfl)
    while tt < stop:
        S = orc.advance(sc, cl, S, [1.0 / h for h in dx], bc, bc, odt, nthreads=8)
        tt = tt + odt
        Sv = S.copy()
        orc.fill_halo(Sv, bc, bc)
        dt_min = min(orc.est_timestep(cl, Sv, dx, cfl), 1.1 * odt)
        odt = stop - tt if tt + dt_min > stop - 0.001 * dt_min else dt_min
    assert t == tt
    assert G.relmax(rho[None], P.valid(S)[0, 2, 2, :][None]) <= 1e-10


@pytest.mark.parametrize("visc", [0, 1])
def test_weno_riemann_rhs_vjp_dot_product(orc, visc):
    """<v, J w> from the oracle's dual-number JVP against <J^T v, w> from the
    GPU reverse pass (same branches, so equal to rounding)."""
    from tests.test_gpu_adjoint import scaled_direction
    sc = P.Scheme(flux_euler=0, riemann_weno=1, rhs_visc=visc)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    n = (11, 9, 8)
    U = P.random_state(n, seed=61 + visc, amp=0.25)
    dxinv = (1.7, 2.9, 0.8)
    v = np.random.default_rng(62 + visc).standard_normal((5, n[2], n[1], n[0]))
    W = scaled_direction(U, 63 + visc)
    _, JW = orc.rhs_jvp(sc, cl, U, W, dxinv, nthreads=4)
    h = capi.Handle(sc, cl)
    Ud = torch.from_numpy(U).cuda()
    ubar = torch.empty_like(Ud)
    h.rhs_vjp_box(Ud, torch.from_numpy(v).cuda(), ubar, dxinv)
    h.sync_check()
    lhs = float(np.sum(v * JW))
    rhs = float(np.sum(ubar.cpu().numpy() * W))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.linalg.norm(v) * np.linalg.norm(JW)), (lhs, rhs)
