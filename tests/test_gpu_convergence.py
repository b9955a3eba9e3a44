"""Order of accuracy of the GPU RHS on a smooth periodic field (the
reference's MMS RHS-only convergence check, exm/MMS_euler): the Euler RHS of
a field that varies along x only is -d/dx F_x(U(x)), whose exact value comes
from a spectral derivative of the point flux.  Halving dx divides the error
by 2^order for KEEP of order 2, 4, 6."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu
NG = P.NGHOST
GAMMA = 1.4


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def prims(x):
    rho = 1.0 + 0.2 * np.sin(x) + 0.05 * np.cos(2 * x)
    u = 0.3 + 0.1 * np.cos(x)
    v = 0.05 * np.sin(2 * x)
    w = -0.02 * np.cos(x)
    p = 1.0 / GAMMA + 0.1 * np.sin(x + 0.4)
    return rho, u, v, w, p


def gpu_rhs(order, n):
    h = 2 * np.pi / n
    X, Y, Z = P.cell_centres((n, 4, 4), (h, h, h))
    rho, u, v, w, p = prims(X)
    U = P.prims_to_cons(rho, u, v, w, p, GAMMA)
    cl = P.Closures.nondimensional(1e-3)
    hdl = capi.Handle(P.Scheme(flux_euler=1, order_keep=order, rhs_visc=0), cl)
    R = torch.empty((5, 4, 4, n), dtype=torch.float64, device="cuda")
    hdl.rhs_box(torch.from_numpy(U).cuda(), (1 / h, 1 / h, 1 / h), R)
    hdl.sync_check()
    return R.cpu().numpy()[:, 1, 1, :]


def exact_at_centres(n):
    """Exact RHS at the n cell centres x_i = (i + 1/2) h by spectral interpolation."""
    m = 4096
    xf = np.arange(m) * 2 * np.pi / m
    rho, u, v, w, p = prims(xf)
    E = p / (GAMMA - 1) + 0.5 * rho * (u * u + v * v + w * w)
    F = np.stack([rho * u, rho * u * u + p, rho * u * v, rho * u * w, (E + p) * u])
    k = np.fft.fftfreq(m, d=1.0 / m)
    Fh = np.fft.fft(F, axis=1)
    xc = (np.arange(n) + 0.5) * 2 * np.pi / n
    # evaluate -dF/dx = -sum 1j k Fh e^{ikx} / m at the centres
    phase = np.exp(1j * np.outer(k, xc))
    return -np.real((1j * k * Fh) @ phase) / m


@pytest.mark.parametrize("order", [2, 4, 6])
def test_keep_order_of_accuracy(order):
    errs = []
    for n in (32, 64, 128):
        e = gpu_rhs(order, n) - exact_at_centres(n)
        errs.append(np.abs(e).max())
    rates = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    # oracle on the same fields: 1.99/2.00, 3.92/3.98, 5.66/5.94
    assert rates[-1] > order - 0.2 and min(rates) > order - 0.5, (errs, rates)
