"""Adjoint of RK steps on a domain with code-6 y walls whose ghost cells a
problem bcnormal fills (here an isothermal no-slip wall written with torch
operations, in the manner of the reference's channel problem: velocity
mirrored with a sign flip, pressure copied, wall temperature extrapolated
with the ghost/first-cell distance ratio).  The library's ghosted stage VJP,
the bcnormal's reverse by autograd and the library's ghost fold together
must give the derivative of whole steps: checked against central
differences, one step and a checkpointed multi-step run."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import adjoint, capi, cns
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu
G = P.NGHOST


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def wall_bcnormal(Tw, cl):
    """bcnormal for both y sides: every ghost row j (distance ratio 2g-1 to
    the first interior row) over the whole x/z extent, ghost columns
    included (the library filled those before)."""
    gamma, R, cv = cl.gamma, cl.Rspec, cl.cv

    def fill(t):
        ny = t.shape[2] - 2 * G
        for side in (0, 1):
            jf = G if side == 0 else G + ny - 1
            s = t[:, :, jf, :].clone()
            rho = s[0]
            ux, uy, uz = s[1] / rho, s[2] / rho, s[3] / rho
            ke = 0.5 * (ux * ux + uy * uy + uz * uz)
            p = (gamma - 1.0) * (s[4] - rho * ke)
            T = p / (R * rho)
            for g in range(1, G + 1):
                jg = jf - g if side == 0 else jf + g
                Te = Tw + (2 * g - 1) * (Tw - T)
                re = p / (R * Te)
                t[0, :, jg, :] = re
                t[1, :, jg, :] = -re * ux
                t[2, :, jg, :] = -re * uy
                t[3, :, jg, :] = -re * uz
                t[4, :, jg, :] = re * (cv * Te + ke)

    return fill


def channel_level(sc, cl, n, seed, bcn=True):
    U = P.random_state(n, seed=seed, amp=0.1)
    dx = tuple(1.0 / v for v in n)
    rho, p = 1.0, 1.0 / cl.gamma
    Tw = p / (cl.Rspec * rho)
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=(-1, 6, -1), bc_hi=(-1, 6, -1),
                       bcnormal=wall_bcnormal(Tw, cl) if bcn else None)
    return lev, U


def ghosted(lev, Uv):
    S = torch.zeros(lev.shape, dtype=torch.float64, device="cuda")
    S[:, G:-G, G:-G, G:-G] = Uv
    return S


def step_valid(lev, Uv, dt):
    _, out = adjoint._forward_step(lev, ghosted(lev, Uv), dt)
    return out[:, G:-G, G:-G, G:-G]


def direction(shape, seed, U):
    rng = np.random.default_rng(seed)
    W = rng.standard_normal(shape)
    for c in range(5):
        W[c] *= np.sqrt(np.mean(U[c] ** 2)) + 1e-3
    return dev(W)


SCHEMES = [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=2, rhs_visc=1)]


@pytest.mark.parametrize("skw", SCHEMES, ids=["keep4_visc", "weno_visc"])
def test_step_vjp_with_walls_vs_fd(skw):
    n = (12, 10, 8)
    cl = P.Closures.nondimensional(1.0 / 200.0)
    sc = P.Scheme(**skw)
    lev, U = channel_level(sc, cl, n, seed=3)
    dt = 4e-3
    Uv = dev(P.valid(U).copy())
    g = dev(np.random.default_rng(5).standard_normal(Uv.shape))
    stages, _ = adjoint._forward_step(lev, ghosted(lev, Uv), dt)
    ubar, _ = adjoint._step_vjp(lev, stages, dt, g)
    # the same with the bcnormal's derivative left out (ghosts as constants)
    keep = lev.bcnormal_vjp
    lev.bcnormal_vjp = lambda t, gb: gb
    ubar_const, _ = adjoint._step_vjp(lev, stages, dt, g)
    lev.bcnormal_vjp = keep
    lev.h.sync_check()
    eps = 1e-6
    worst = 0.0
    for k in range(6):
        W = direction(Uv.shape, 40 + k, P.valid(U))
        fp = float(torch.sum(g * step_valid(lev, Uv + eps * W, dt)))
        fm = float(torch.sum(g * step_valid(lev, Uv - eps * W, dt)))
        fd = (fp - fm) / (2 * eps)
        ad = float(torch.sum(ubar * W))
        worst = max(worst, abs(fd - ad) / abs(ad))
        assert abs(float(torch.sum(ubar_const * W)) - ad) > 1e-6 * abs(ad)
    assert worst <= 1e-6, worst


def test_checkpointed_run_with_walls_vs_fd():
    n = (12, 10, 8)
    cl = P.Closures.nondimensional(1.0 / 200.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    lev, U = channel_level(sc, cl, n, seed=11)
    dt, nsteps = 4e-3, 5
    Uv = dev(P.valid(U).copy())
    adj = adjoint.CheckpointedAdjoint(lev, every=2)
    ubar0, _, _ = adj.run(Uv, nsteps, dt, adjoint.kinetic_energy_grad)

    def run(Ui):
        S = Ui
        for _ in range(nsteps):
            S = step_valid(lev, S, dt).contiguous()
        return float(adjoint.kinetic_energy(S))

    eps = 1e-6
    for k in range(3):
        W = direction(Uv.shape, 70 + k, P.valid(U))
        fd = (run(Uv + eps * W) - run(Uv - eps * W)) / (2 * eps)
        ad = float(torch.sum(ubar0 * W))
        assert abs(fd - ad) <= 1e-6 * abs(ad), (k, fd, ad)
    lev.h.sync_check()


def test_ghosted_stage_vjp_matches_folded_on_periodic_box():
    """Without ext_dir sides, ghosted VJP + the library's fold equals the
    folding stage VJP (same kernels, sums in another order)."""
    n = 10
    U, dx = P.tgv(n, mach=0.2)
    U = U * (1.0 + 0.01 * np.random.default_rng(2).standard_normal(U.shape))
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    h = capi.Handle(sc, cl)
    dxinv = [1.0 / v for v in dx]
    Ud = dev(U)
    bc = (-1, -1, -1)
    capi.fill_halo_box(Ud, bc, bc)
    wbar = dev(np.random.default_rng(3).standard_normal((5, n, n, n)))
    for p in capi.rk_program(3, 3, 1e-2):
        s1a = torch.zeros_like(wbar)
        ina = torch.zeros_like(wbar)
        h.rk_stage_vjp_box(p, bc, bc, Ud, wbar, s1a, ina, dxinv)
        s1b = torch.zeros_like(wbar)
        ug = torch.empty_like(Ud)
        h.rk_stage_vjp_box_ghosted(p, Ud, wbar, s1b, ug, dxinv)
        capi.fill_halo_box_adjoint(ug, bc, bc)
        inb = ug[:, G:-G, G:-G, G:-G]
        h.sync_check()
        assert torch.equal(s1a, s1b)
        scale = float(ina.abs().max())
        assert float((ina - inb).abs().max()) <= 1e-14 * scale


def test_folding_stage_vjp_rejects_ext_dir_codes():
    cl = P.Closures.nondimensional(1e-2)
    h = capi.Handle(P.Scheme(), cl)
    U = torch.from_numpy(P.random_state((8, 8, 8), seed=1)).cuda()
    z = torch.zeros((5, 8, 8, 8), dtype=torch.float64, device="cuda")
    prog = capi.rk_program(3, 3, 1e-3)[0]
    for code in (1, 6):
        with pytest.raises(capi.AmrsError):
            h.rk_stage_vjp_box(prog, (-1, code, -1), (-1, 2, -1), U, z, z.clone(), z.clone(), (8.0, 8.0, 8.0))
