"""Adjoint (VJP) of the RHS with JST artificial dissipation (art_diss = 1)
on top of each Euler flux, with and without viscous fluxes: dot-product test
<v, J w> = <J^T v, w> against the CPU oracle's dual-number JVP (same
branches of max and |.|, so the identity holds to rounding), and one whole
SSPRK3 step through the autograd wrapper."""
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


def closures():
    cl = P.Closures.nondimensional(1e-2)
    cl.Cshock, cl.Cdamp = 1.0, 0.05  # sensor and fourth-difference terms both active
    return cl


@pytest.mark.parametrize("skw", [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=1, order_keep=2, rhs_visc=0),
                                 dict(flux_euler=2, rhs_visc=1), dict(flux_euler=0, rhs_visc=0)],
                         ids=["keep4-visc", "keep2", "weno-visc", "muscl"])
def test_jst_rhs_vjp_dot_product(orc, skw):
    n = 12
    U, dx = turbulent_state(n, seed=71)
    sc = P.Scheme(art_diss=1, **skw)
    cl = closures()
    dxinv = [1.0 / h for h in dx]
    v = np.random.default_rng(72).standard_normal((5, n, n, n))
    W = scaled_direction(U, 73)
    _, JW = orc.rhs_jvp(sc, cl, U, W, dxinv, nthreads=4)
    h = capi.Handle(sc, cl)
    ubar = torch.empty_like(dev(U))
    h.rhs_vjp_box(dev(U), dev(v), ubar, dxinv)
    h.sync_check()
    lhs = float(np.sum(v * JW))
    rhs = float(np.sum(ubar.cpu().numpy() * W))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.linalg.norm(v) * np.linalg.norm(JW)), (lhs, rhs)


def test_jst_step_vjp_dot_product(orc):
    n = 10
    U, dx = turbulent_state(n, seed=75)
    cl = closures()
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, art_diss=1)
    dxinv = [1.0 / h for h in dx]
    dt = 1e-2
    W = scaled_direction(U, 76)
    _, JW = oracle_step_jvp(orc, sc, cl, U, W, dxinv, dt)
    lev = cns.CNSLevel(sc, cl, U, dx)
    g = np.random.default_rng(77).standard_normal((5, n, n, n))
    Uv = dev(P.valid(U).copy())
    Uv.requires_grad_(True)
    out = adjoint.StepFunction.apply(Uv, lev, dt)
    (grad,) = torch.autograd.grad(out, Uv, grad_outputs=dev(g))
    lev.h.sync_check()
    lhs = float(np.sum(g * JW))
    rhs = float(np.sum(grad.cpu().numpy() * P.valid(W)))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.linalg.norm(g) * np.linalg.norm(JW)), (lhs, rhs)
