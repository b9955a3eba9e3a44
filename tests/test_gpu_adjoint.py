"""Adjoint (VJP) kernels of the RHS and of the RK step.

Checks: dot-product test <v, J w> = <J^T v, w> against the CPU oracle's
dual-number JVP (the reference's own autodiff build does not exist), central
finite differences (eps = 1e-6) along random directions, the
torch.autograd.Function wrappers, and the checkpointed multi-step gradient of
the kinetic energy with respect to the initial amplitude V0 and viscosity mu.
"""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import adjoint, capi, cns
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu
G = 3


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def perturbed_tgv(n, mach=0.3, seed=0):
    U, dx = P.tgv(n, mach=mach)
    rng = np.random.default_rng(seed)
    U = U * (1.0 + 0.01 * rng.standard_normal(U.shape))
    return U, dx


def scaled_direction(U, seed):
    rng = np.random.default_rng(seed)
    W = rng.standard_normal(U.shape)
    for c in range(5):
        W[c] *= np.sqrt(np.mean(U[c] ** 2)) + 1e-3
    return W


@pytest.mark.parametrize("kind", ["const", "suth"])
def test_rhs_vjp_dot_product(orc, kind):
    n = 12
    if kind == "const":
        U, dx = perturbed_tgv(n)
        cl = P.Closures.nondimensional(1.0 / 400.0)
    else:
        cl = P.Closures.air_sutherland()
        U = P.random_state((n, n, n), seed=3)
        rho = U[0]
        T = 300.0 + 5.0 * np.sin(np.arange(rho.size).reshape(rho.shape))
        U = P.prims_to_cons(rho, 20 * U[1] / rho, 20 * U[2] / rho, 20 * U[3] / rho, rho * cl.Rspec * T, cl.gamma)
        dx = (1e-2, 1e-2, 1e-2)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    rng = np.random.default_rng(11)
    v = rng.standard_normal((5, n, n, n))
    W = scaled_direction(U, 12)
    _, JW = orc.rhs_jvp(sc, cl, U, W, dxinv, nthreads=4)
    h = capi.Handle(sc, cl)
    ubar = torch.empty_like(dev(U))
    h.rhs_vjp_box(dev(U), dev(v), ubar, dxinv)
    h.sync_check()
    lhs = float(np.sum(v * JW))
    rhs = float(np.sum(ubar.cpu().numpy() * W))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.sqrt(np.sum(v * v)) * np.sqrt(np.sum(JW * JW)))


def test_rhs_vjp_central_fd_32_directions():
    """TGV 64^3, M=0.1, Re=400: <v, (R(U+eps w) - R(U-eps w))/2eps> vs <J^T v, w>."""
    n = 64
    U, dx = P.tgv(n, mach=0.1)
    cl = P.Closures.nondimensional(1.0 / 400.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    h = capi.Handle(sc, cl)
    Ud = dev(U)
    rng = np.random.default_rng(2024)
    v = dev(rng.standard_normal((5, n, n, n)))
    ubar = torch.empty_like(Ud)
    h.rhs_vjp_box(Ud, v, ubar, dxinv)
    out_p = torch.empty_like(v)
    out_m = torch.empty_like(v)
    eps = 1e-6
    worst = 0.0
    for k in range(32):
        W = dev(scaled_direction(U, 100 + k))
        h.rhs_box(Ud + eps * W, dxinv, out_p)
        h.rhs_box(Ud - eps * W, dxinv, out_m)
        fd = float(torch.sum(v * (out_p - out_m)) / (2 * eps))
        ad = float(torch.sum(ubar * W))
        worst = max(worst, abs(fd - ad) / abs(ad))
    h.sync_check()
    assert worst <= 1e-6, worst


def oracle_step_jvp(orc, sc, cl, U, W, dxinv, dt, bc=(-1, -1, -1)):
    """Tangent of one CNS::advance step (SSPRK3) by composing the oracle's
    RHS JVPs through the stage programs; ghost fills applied to tangents."""
    v = (slice(None), slice(G, -G), slice(G, -G), slice(G, -G))
    S1, T1 = U.copy(), W.copy()
    S2, T2 = U.copy(), W.copy()
    for p in capi.rk_program(3, 3, dt):
        Sb = (S1 if p.src_state == 0 else S2).copy()
        Tb = (T1 if p.src_state == 0 else T2).copy()
        orc.fill_halo(Sb, bc, bc)
        orc.fill_halo(Tb, bc, bc)
        R, JT = orc.rhs_jvp(sc, cl, Sb, Tb, dxinv, nthreads=4)
        reg = [S1[v].copy(), Sb[v].copy(), R]
        tan = [T1[v].copy(), Tb[v].copy(), JT]
        for o in range(p.nops):
            q = p.ops[o]
            for r in (reg, tan):
                if q.kind == 0:
                    r[q.dst] = q.a * r[q.x] + q.b * r[q.y]
                elif q.kind == 1:
                    r[q.dst] = r[q.dst] + q.a * r[q.x]
                elif q.kind == 2:
                    r[q.dst] = r[q.x] + q.a * r[q.dst]
                else:
                    r[q.dst] = r[q.x].copy()
        S2[v], T2[v] = reg[1], tan[1]
    return S2[v], T2[v]


def test_step_vjp_dot_product(orc):
    n = 12
    U, dx = perturbed_tgv(n, mach=0.2, seed=4)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    dt = 2e-2
    W = scaled_direction(U, 5)
    _, JW = oracle_step_jvp(orc, sc, cl, U, W, dxinv, dt)
    lev = cns.CNSLevel(sc, cl, U, dx)
    g = np.random.default_rng(6).standard_normal((5, n, n, n))
    Uv = dev(P.valid(U).copy())
    Uv.requires_grad_(True)
    out = adjoint.StepFunction.apply(Uv, lev, dt)
    (grad,) = torch.autograd.grad(out, Uv, grad_outputs=dev(g))
    lev.h.sync_check()
    lhs = float(np.sum(g * JW))
    rhs = float(np.sum(grad.cpu().numpy() * P.valid(W)))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.linalg.norm(g) * np.linalg.norm(JW))


def test_rhs_autograd_function_matches_capi():
    n = 10
    U, dx = perturbed_tgv(n, seed=8)
    cl = P.Closures.nondimensional(1.0 / 500.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    h = capi.Handle(sc, cl)
    Ud = dev(U).requires_grad_(True)
    v = dev(np.random.default_rng(9).standard_normal((5, n, n, n)))
    R = adjoint.RHSFunction.apply(Ud, h, dxinv, (0, 0, 0))
    (g,) = torch.autograd.grad((R * v).sum(), Ud)
    ubar = torch.empty_like(Ud)
    h.rhs_vjp_box(Ud.detach(), v, ubar, dxinv)
    h.sync_check()
    assert torch.equal(g, ubar)


def test_checkpointed_gradient_vs_fd():
    """d KE(after N steps) / d(V0, mu) with checkpoints every k steps, against
    central differences of the full forward run."""
    n, nsteps, dt, every = 16, 12, 2e-2, 5
    mach, re = 0.1, 400.0
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)

    def run(amp, mu):
        U, dx = P.tgv(n, mach=mach, amp=amp)
        lev = cns.CNSLevel(sc, P.Closures.nondimensional(mu), U, dx)
        for _ in range(nsteps):
            lev.advance(lev.time, dt)
        return float(adjoint.kinetic_energy(lev.valid()))

    mu0 = 1.0 / re
    U, dx = P.tgv(n, mach=mach, amp=1.0)
    cl = P.Closures.nondimensional(mu0)
    lev = cns.CNSLevel(sc, cl, U, dx)
    adj = adjoint.CheckpointedAdjoint(lev, every=every)
    ubar0, pbar, _ = adj.run(dev(P.valid(U).copy()), nsteps, dt, adjoint.kinetic_energy_grad)
    # d U0 / d V0 (the initial field is quadratic in V0: central difference is exact to rounding)
    e = 1e-3
    dU = (P.valid(P.tgv(n, mach=mach, amp=1.0 + e)[0]) - P.valid(P.tgv(n, mach=mach, amp=1.0 - e)[0])) / (2 * e)
    g_v0 = float(np.sum(ubar0.cpu().numpy() * dU))
    pb = pbar.cpu().numpy()
    g_mu = float(pb[0] + cl.cp / 0.71 * pb[1])
    eps = 1e-6
    fd_v0 = (run(1.0 + eps, mu0) - run(1.0 - eps, mu0)) / (2 * eps)
    fd_mu = (run(1.0, mu0 * (1 + eps)) - run(1.0, mu0 * (1 - eps))) / (2 * eps * mu0)
    assert abs(g_v0 - fd_v0) <= 1e-6 * abs(fd_v0), (g_v0, fd_v0)
    assert abs(g_mu - fd_mu) <= 1e-6 * abs(fd_mu), (g_mu, fd_mu)


def test_checkpointed_gradient_vs_fd_tgv64_200_steps():
    """The adjoint configuration at full size: TGV 64^3, M = 0.1, Re = 400,
    d KE(after 200 SSPRK3 steps) / d(V0, mu) with a checkpoint every 20
    steps, against central differences of the whole forward run."""
    n, nsteps, dt, every = 64, 200, 2e-3, 20
    mach, re = 0.1, 400.0
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)

    def run(amp, mu):
        U, dx = P.tgv(n, mach=mach, amp=amp)
        lev = cns.CNSLevel(sc, P.Closures.nondimensional(mu), U, dx)
        for _ in range(nsteps):
            lev.advance(lev.time, dt)
        return float(adjoint.kinetic_energy(lev.valid()))

    mu0 = 1.0 / re
    U, dx = P.tgv(n, mach=mach, amp=1.0)
    cl = P.Closures.nondimensional(mu0)
    lev = cns.CNSLevel(sc, cl, U, dx)
    adj = adjoint.CheckpointedAdjoint(lev, every=every)
    ubar0, pbar, _ = adj.run(dev(P.valid(U).copy()), nsteps, dt, adjoint.kinetic_energy_grad)
    e = 1e-3
    dU = (P.valid(P.tgv(n, mach=mach, amp=1.0 + e)[0]) - P.valid(P.tgv(n, mach=mach, amp=1.0 - e)[0])) / (2 * e)
    g_v0 = float(np.sum(ubar0.cpu().numpy() * dU))
    pb = pbar.cpu().numpy()
    g_mu = float(pb[0] + cl.cp / 0.71 * pb[1])
    eps = 1e-6
    fd_v0 = (run(1.0 + eps, mu0) - run(1.0 - eps, mu0)) / (2 * eps)
    fd_mu = (run(1.0, mu0 * (1 + eps)) - run(1.0, mu0 * (1 - eps))) / (2 * eps * mu0)
    lev.h.sync_check()
    assert abs(g_v0 - fd_v0) <= 1e-6 * abs(fd_v0), (g_v0, fd_v0)
    assert abs(g_mu - fd_mu) <= 1e-6 * abs(fd_mu), (g_mu, fd_mu)


def test_parameter_gradient_bitwise_repeatable():
    """d KE / d(mu, k) is reduced in a fixed order (per-block sums, then the
    blocks in order, no atomics): two runs give the same bits, and the
    state cotangent too."""
    n, nsteps, dt, every = 24, 6, 1e-2, 3
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    U, dx = P.tgv(n, mach=0.1, amp=1.0)
    cl = P.Closures.nondimensional(1.0 / 400.0)
    outs = []
    for _ in range(3):
        lev = cns.CNSLevel(sc, cl, U, dx)
        adj = adjoint.CheckpointedAdjoint(lev, every=every)
        ubar0, pbar, _ = adj.run(dev(P.valid(U).copy()), nsteps, dt, adjoint.kinetic_energy_grad)
        lev.h.sync_check()
        outs.append((ubar0.cpu().numpy(), pbar.cpu().numpy()))
    assert np.all(outs[0][1] != 0.0)
    for u, p in outs[1:]:
        np.testing.assert_array_equal(p, outs[0][1])
        np.testing.assert_array_equal(u, outs[0][0])
