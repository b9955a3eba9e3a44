"""Adjoint (VJP) of the MUSCL + two-shock Riemann RHS, with and without
viscous fluxes.

Checks: dot-product test <v, J w> = <J^T v, w> against the CPU oracle's
dual-number JVP (same branches of the limiters, max, |.| and the solver's
state selection, so the identity holds to rounding) on smooth turbulence,
random and strong-wave states, and the RK-stage VJP through the autograd
wrapper against the oracle's tangent of a whole SSPRK3 step.

No finite-difference check: the solver's pressure iteration ends with
|pstar - pstnm1| within a few ulps of zero on smooth data (the kink of |.|), so
the discrete RHS is differentiable only within a neighbourhood far smaller
than any usable difference step (a central difference at 1e-6 measures a
secant across the kink; the oracle's own dual-number derivative misses it
by tens of percent the same way).  States whose extrapolated density or
pressure reach the 1e-40 floor are avoided too: sensitivities there reach
1e20 and rounding dominates both derivative modes.
"""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import adjoint, capi, cns
from amrsolver_gb300 import problems as P
from tests.test_gpu_adjoint import dev, oracle_step_jvp, scaled_direction
from tests.test_gpu_adjoint_weno import turbulent_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def strong_state(n, seed):
    """Cell-to-cell jumps of tens of percent in density and pressure,
    velocities up to about the sound speed: shocks, rarefactions, supersonic
    sides and transonic fans, with no extrapolated state at the floor."""
    rng = np.random.default_rng(seed)
    shape = (n[2] + 6, n[1] + 6, n[0] + 6)
    rho = np.exp(rng.normal(0.0, 0.3, shape))
    p = np.exp(rng.normal(0.0, 0.3, shape))
    c = np.sqrt(1.4 * p / rho)
    u, v, w = (rng.normal(0.0, 0.8, shape) * c for _ in range(3))
    return P.prims_to_cons(rho, u, v, w, p, 1.4)


def dot_check(orc, sc, cl, U, dxinv, seed, tol=1e-11):
    n = tuple(s - 6 for s in U.shape[1:])
    v = np.random.default_rng(seed).standard_normal((5,) + n)
    W = scaled_direction(U, seed + 1)
    _, JW = orc.rhs_jvp(sc, cl, U, W, dxinv, nthreads=4)
    h = capi.Handle(sc, cl)
    ubar = torch.empty_like(dev(U))
    h.rhs_vjp_box(dev(U), dev(v), ubar, dxinv)
    h.sync_check()
    lhs = float(np.sum(v * JW))
    rhs = float(np.sum(ubar.cpu().numpy() * W))
    assert abs(lhs - rhs) <= tol * (abs(lhs) + np.linalg.norm(v) * np.linalg.norm(JW)), (lhs, rhs)


@pytest.mark.parametrize("visc", [0, 1])
def test_muscl_rhs_vjp_dot_product_turbulence(orc, visc):
    U, dx = turbulent_state(12, seed=41 + visc)
    dot_check(orc, P.Scheme(flux_euler=0, rhs_visc=visc), P.Closures.nondimensional(1e-2), U,
              [1.0 / h for h in dx], 17 + visc)


@pytest.mark.parametrize("visc", [0, 1])
def test_muscl_rhs_vjp_dot_product_random(orc, visc):
    U = P.random_state((11, 9, 7), seed=5 + visc, amp=0.2)
    dot_check(orc, P.Scheme(flux_euler=0, rhs_visc=visc), P.Closures.nondimensional(1.0 / 300.0), U,
              (1.7, 2.9, 0.8), 23 + visc)


def test_muscl_rhs_vjp_dot_product_strong_waves(orc):
    U = strong_state((10, 8, 7), seed=3)
    dot_check(orc, P.Scheme(flux_euler=0, rhs_visc=0), P.Closures.nondimensional(1e-2), U, (1.3, 0.7, 2.1), 29)


def test_muscl_step_vjp_dot_product(orc):
    n = 10
    U, dx = turbulent_state(n, seed=19)
    cl = P.Closures.nondimensional(1e-2)
    sc = P.Scheme(flux_euler=0, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    dt = 1e-2
    W = scaled_direction(U, 21)
    _, JW = oracle_step_jvp(orc, sc, cl, U, W, dxinv, dt)
    lev = cns.CNSLevel(sc, cl, U, dx)
    g = np.random.default_rng(22).standard_normal((5, n, n, n))
    Uv = dev(P.valid(U).copy())
    Uv.requires_grad_(True)
    out = adjoint.StepFunction.apply(Uv, lev, dt)
    (grad,) = torch.autograd.grad(out, Uv, grad_outputs=dev(g))
    lev.h.sync_check()
    lhs = float(np.sum(g * JW))
    rhs = float(np.sum(grad.cpu().numpy() * P.valid(W)))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.linalg.norm(g) * np.linalg.norm(JW)), (lhs, rhs)
