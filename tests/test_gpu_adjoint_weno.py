"""Adjoint (VJP) of the WENO5-JS LLF RHS, with and without viscous fluxes.

Checks: dot-product test <v, J w> = <J^T v, w> against the CPU oracle's
dual-number JVP (same branches of max and |.|, so the identity holds to
rounding), central finite differences on a state whose local wave-speed
maxima are unique with a margin (so no perturbation switches a branch), and
the RK-stage VJP through the autograd wrapper against the oracle's tangent
of a whole SSPRK3 step.
"""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import adjoint, capi, cns
from amrsolver_gb300 import problems as P
from tests.test_gpu_adjoint import dev, oracle_step_jvp, scaled_direction

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def turbulent_state(n, seed):
    U, dx = P.random_turbulence(n, mach_t=0.5, k0=2.0, seed=seed)
    rng = np.random.default_rng(seed + 1)
    return U * (1.0 + 0.01 * rng.standard_normal(U.shape)), dx


def graded_state(n, gamma=1.4, amp=0.05):
    """Velocity increasing along every axis (|u|+c grows along each axis, so
    its maximum over a six-cell stencil is the upper end by a margin) with
    smooth sinusoidal curvature."""
    h = 1.0 / n
    X, Y, Z = P.cell_centres((n, n, n), (h, h, h))
    s = lambda a, b, c: amp * np.sin(2 * np.pi * (a * X + b * Y + c * Z) + 0.3)
    u = 0.3 + 0.5 * X + 0.1 * Y + 0.1 * Z + s(1.0, 0.5, 0.2)
    v = 0.2 + 0.1 * X + 0.5 * Y + 0.1 * Z + s(0.3, 1.0, 0.4)
    w = 0.1 + 0.1 * X + 0.1 * Y + 0.5 * Z + s(0.2, 0.6, 1.0)
    rho = 1.0 + 0.05 * np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y)
    p = 1.0 / gamma + 0.02 * np.cos(2 * np.pi * (X + Y + Z))
    return P.prims_to_cons(rho, u, v, w, p, gamma), (h, h, h)


@pytest.mark.parametrize("visc", [0, 1])
def test_weno_rhs_vjp_dot_product(orc, visc):
    n = 12
    U, dx = turbulent_state(n, seed=31 + visc)
    cl = P.Closures.nondimensional(1e-2)
    sc = P.Scheme(flux_euler=2, rhs_visc=visc)
    dxinv = [1.0 / h for h in dx]
    v = np.random.default_rng(7).standard_normal((5, n, n, n))
    W = scaled_direction(U, 8)
    _, JW = orc.rhs_jvp(sc, cl, U, W, dxinv, nthreads=4)
    h = capi.Handle(sc, cl)
    ubar = torch.empty_like(dev(U))
    h.rhs_vjp_box(dev(U), dev(v), ubar, dxinv)
    h.sync_check()
    lhs = float(np.sum(v * JW))
    rhs = float(np.sum(ubar.cpu().numpy() * W))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.linalg.norm(v) * np.linalg.norm(JW)), (lhs, rhs)


def test_weno_rhs_vjp_central_fd():
    """WENO5-JS weights (eps = 1e-40) vary fast with the smoothness
    indicators of smooth data, so a central difference at eps = 1e-6 carries
    an O(eps^2) error of ~1e-4 here; Richardson extrapolation of the central
    differences at eps and eps/2 removes it (oracle check: 7e-8)."""
    n = 24
    U, dx = graded_state(n)
    cl = P.Closures.nondimensional(1e-3)
    sc = P.Scheme(flux_euler=2, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    h = capi.Handle(sc, cl)
    Ud = dev(U)
    v = dev(np.random.default_rng(5).standard_normal((5, n, n, n)))
    ubar = torch.empty_like(Ud)
    h.rhs_vjp_box(Ud, v, ubar, dxinv)
    out_p, out_m = torch.empty_like(v), torch.empty_like(v)

    def central(W, e):
        h.rhs_box(Ud + e * W, dxinv, out_p)
        h.rhs_box(Ud - e * W, dxinv, out_m)
        return float(torch.sum(v * (out_p - out_m))) / (2 * e)

    eps = 1e-6
    fds, ads = [], []
    for k in range(8):
        W = dev(scaled_direction(U, 300 + k))
        fds.append((4.0 * central(W, 0.5 * eps) - central(W, eps)) / 3.0)
        ads.append(float(torch.sum(ubar * W)))
    h.sync_check()
    # one of the eight inner products nearly cancels (-16 against ~3e4), so
    # errors are measured against the RMS inner product of the set
    scale = float(np.sqrt(np.mean(np.square(ads))))
    worst = max(abs(f - a) for f, a in zip(fds, ads)) / scale
    assert worst <= 1e-6, (worst, fds, ads)


def test_weno_vjp_fast_and_reference_order_forward_agree():
    """Both forward variants share one VJP; they are the same function."""
    n = 16
    U, dx = turbulent_state(n, seed=3)
    cl = P.Closures.nondimensional(1e-3)
    dxinv = [1.0 / h for h in dx]
    outs = []
    for fast in (0, 1):
        h = capi.Handle(P.Scheme(flux_euler=2, rhs_visc=1, weno_fast=fast), cl)
        R = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
        h.rhs_box(dev(U), dxinv, R)
        h.sync_check()
        outs.append(R.cpu().numpy())
    scale = np.abs(outs[0]).reshape(5, -1).max(axis=1)
    assert np.all(np.abs(outs[1] - outs[0]).reshape(5, -1).max(axis=1) <= 1e-11 * scale)


def test_weno_step_vjp_dot_product(orc):
    n = 12
    U, dx = turbulent_state(n, seed=11)
    cl = P.Closures.nondimensional(1e-2)
    sc = P.Scheme(flux_euler=2, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    dt = 1e-2
    W = scaled_direction(U, 13)
    _, JW = oracle_step_jvp(orc, sc, cl, U, W, dxinv, dt)
    lev = cns.CNSLevel(sc, cl, U, dx)
    g = np.random.default_rng(14).standard_normal((5, n, n, n))
    Uv = dev(P.valid(U).copy())
    Uv.requires_grad_(True)
    out = adjoint.StepFunction.apply(Uv, lev, dt)
    (grad,) = torch.autograd.grad(out, Uv, grad_outputs=dev(g))
    lev.h.sync_check()
    lhs = float(np.sum(g * JW))
    rhs = float(np.sum(grad.cpu().numpy() * P.valid(W)))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.linalg.norm(g) * np.linalg.norm(JW)), (lhs, rhs)
