"""Every entry of the RHS VJP, cell by cell, against the oracle.

For a small box, J^T v is assembled on the CPU one state entry at a time
from the oracle's dual-number JVP (<v, J e_i> for every component and cell
of the ghosted state, ghosts included) and compared with the GPU reverse
pass entry by entry, so a cell the reverse pass misses (a ghost layer, a
stencil end, a component) shows up directly rather than averaged into one
inner product."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


SCHEMES = [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=1, order_keep=6, rhs_visc=0),
           dict(flux_euler=2, rhs_visc=1), dict(flux_euler=0, rhs_visc=1),
           dict(flux_euler=0, riemann_weno=1, rhs_visc=1), dict(flux_euler=1, order_keep=4, rhs_visc=1, art_diss=1),
           dict(rhs_euler=0, rhs_visc=1)]


@pytest.mark.parametrize("skw", SCHEMES, ids=lambda d: "-".join("%s%s" % kv for kv in d.items()))
def test_vjp_every_entry(orc, skw):
    sc = P.Scheme(**skw)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    cl.Cshock, cl.Cdamp = 1.0, 0.05
    n = (5, 4, 3)
    U = P.random_state(n, seed=3 + len(str(skw)), amp=0.2)
    dxinv = (1.7, 2.9, 0.8)
    v = np.random.default_rng(4).standard_normal((5, n[2], n[1], n[0]))
    h = capi.Handle(sc, cl)
    Ud = torch.from_numpy(U).cuda()
    ub = torch.empty_like(Ud)
    h.rhs_vjp_box(Ud, torch.from_numpy(v).cuda(), ub, dxinv)
    h.sync_check()
    ub = ub.cpu().numpy()
    G = np.zeros_like(U)
    W = np.zeros_like(U)
    for idx in np.ndindex(U.shape):
        W[idx] = 1.0
        _, JW = orc.rhs_jvp(sc, cl, U, W, dxinv)
        G[idx] = np.sum(v * JW)
        W[idx] = 0.0
    scale = np.abs(G).max()
    assert scale > 0
    bad = np.argwhere(np.abs(G - ub) > 1e-10 * scale)
    assert len(bad) == 0, [(tuple(int(x) for x in b), G[tuple(b)], ub[tuple(b)]) for b in bad[:10]]
