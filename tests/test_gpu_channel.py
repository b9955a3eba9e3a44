"""The reference's channel configuration on the GPU path, end to end: x and
z periodic, code-6 y walls (the reference's wall treatment in compute_rhs),
their ghost cells filled by an isothermal no-slip bcnormal after the
library's fill (velocity mirrored with a sign flip, pressure copied, wall
temperature extrapolated with the ghost/first-cell distance ratio, as
exm/Channel/prob.h:158-186 does), cns.rhs_source with the x body force of
exm/Channel/prob.h:189-193, KEEP4 + viscous, SSPRK3.  Against the oracle
composed stage by stage with the same bcnormal in numpy: bit for bit."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu
G = P.NGHOST


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def make_bcnormal(Tw, cl, xp):
    """bcnormal for both y sides over the whole x/z extent; xp is numpy or
    torch (the same operations in the same order on either)."""
    gamma, R, cv = cl.gamma, cl.Rspec, cl.cv

    def fill(t):
        ny = t.shape[2] - 2 * G
        for side in (0, 1):
            jf = G if side == 0 else G + ny - 1
            s = t[:, :, jf, :].copy() if xp is np else t[:, :, jf, :].clone()
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


def channel_state(n, cl, seed):
    """A laminar profile across y with a small random perturbation."""
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    shape = (nz + 2 * G, ny + 2 * G, nx + 2 * G)
    y = (np.arange(-G, ny + G) + 0.5) / ny
    prof = 4.0 * y * (1.0 - y)
    rho = np.ones(shape) * (1.0 + 0.02 * rng.standard_normal(shape))
    u = 0.3 * prof[None, :, None] * np.ones(shape) + 0.01 * rng.standard_normal(shape)
    v = 0.01 * rng.standard_normal(shape)
    w = 0.01 * rng.standard_normal(shape)
    p = np.ones(shape) / cl.gamma * (1.0 + 0.01 * rng.standard_normal(shape))
    return P.prims_to_cons(rho, u, v, w, p, cl.gamma)


def oracle_step(orc, sc, cl, S1, dxinv, dt, bcn, bl, bh, walls):
    v = (slice(None), slice(G, -G), slice(G, -G), slice(G, -G))
    S2 = S1.copy()
    for p in capi.rk_program(3, 3, dt):
        Sb = (S1 if p.src_state == 0 else S2).copy()
        orc.fill_halo(Sb, bl, bh)
        bcn(Sb)
        reg = [S1[v].copy(), Sb[v].copy(), orc.rhs(sc, cl, Sb, dxinv, walls=walls, nthreads=4)]
        for o in range(p.nops):
            q = p.ops[o]
            if q.kind == 0:
                reg[q.dst] = q.a * reg[q.x] + q.b * reg[q.y]
            elif q.kind == 1:
                reg[q.dst] = reg[q.dst] + q.a * reg[q.x]
            elif q.kind == 2:
                reg[q.dst] = reg[q.x] + q.a * reg[q.dst]
            else:
                reg[q.dst] = reg[q.x].copy()
        S2[v] = reg[1]
    return S2


@pytest.mark.parametrize("order", [4, 6])
def test_channel_steps_bitexact(orc, order):
    n = (24, 16, 12)
    cl = P.Closures.nondimensional(1.0 / 500.0)
    sc = P.Scheme(flux_euler=1, order_keep=order, rhs_visc=1, rhs_source=1, body_force=(0.8, 0.0, 0.0))
    U = channel_state(n, cl, seed=order)
    dx = (2.0 / n[0], 1.0 / n[1], 1.0 / n[2])
    dxinv = [1.0 / h for h in dx]
    Tw = 1.0 / cl.gamma / cl.Rspec
    bl, bh = (-1, 6, -1), (-1, 6, -1)
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=bl, bc_hi=bh, bcnormal=make_bcnormal(Tw, cl, torch))
    bcn = make_bcnormal(Tw, cl, np)
    walls = (1, 1, 0, n[1] - 1)
    dt = 2e-3
    ref = U.copy()
    for _ in range(4):
        lev.advance(lev.time, dt)
        ref = oracle_step(orc, sc, cl, ref, dxinv, dt, bcn, bl, bh, walls)
    lev.h.sync_check()
    got = lev.valid().cpu().numpy()
    np.testing.assert_array_equal(got, P.valid(ref))
    # the x body force pushed the flow: sum of x momentum grew
    assert got[1].sum() > P.valid(U)[1].sum()
