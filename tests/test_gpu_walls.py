"""y walls of boundary code 6 (the reference's wall treatment in
compute_rhs): second-order KEEP y fluxes next to the wall and one-sided
viscous fluxes in the wall's ghost row, for boxes that touch the wall.
Ghost cells beyond code-6 sides are the caller's and stay as stored."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import problems as P
from tests import golden_io as G

pytestmark = pytest.mark.gpu
NG = P.NGHOST

SCHEMES = [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=1, order_keep=6, rhs_visc=0),
           dict(flux_euler=1, order_keep=2, rhs_visc=1), dict(flux_euler=2, rhs_visc=1),
           dict(flux_euler=0, rhs_visc=1)]


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def check(R, ref, skw):
    if skw.get("flux_euler") == 2:
        assert G.relmax(R, ref) <= 1e-13
    else:
        np.testing.assert_array_equal(R, ref)


@pytest.mark.parametrize("walls", [(1, 1), (1, 0), (0, 1)])
@pytest.mark.parametrize("skw", SCHEMES, ids=lambda d: "-".join("%s%s" % kv for kv in d.items()))
def test_rhs_box_on_walls(orc, skw, walls):
    n = (12, 14, 10)
    lo = (2, -3, 1)
    U = P.random_state(n, seed=41 + walls[0] + 2 * walls[1], amp=0.15)
    dxinv = (12.0, 14.0, 10.0)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(**skw)
    h = capi.Handle(sc, cl)
    bl = (-1, 6 if walls[0] else 2, -1)
    bh = (-1, 6 if walls[1] else 2, -1)
    h.set_domain(lo, n, bl, bh)
    R = torch.empty((5, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    h.rhs_box(torch.from_numpy(U).cuda(), dxinv, R, lo=lo)
    h.sync_check()
    ref = orc.rhs(sc, cl, U, dxinv, lo=lo, walls=(walls[0], walls[1], lo[1], lo[1] + n[1] - 1), nthreads=4)
    check(R.cpu().numpy(), ref, skw)
    # the wall treatment changed the result
    assert not np.array_equal(ref, orc.rhs(sc, cl, U, dxinv, lo=lo, nthreads=4))


def test_rhs_sub_boxes_of_a_walled_domain(orc):
    """Boxes of a taller domain: only the ones touching a wall change."""
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    h = capi.Handle(sc, cl)
    dom_lo, dom_n = (0, 0, 0), (10, 30, 8)
    h.set_domain(dom_lo, dom_n, (-1, 6, -1), (-1, 6, -1))
    dxinv = (10.0, 30.0, 8.0)
    for y0, ny in [(0, 9), (9, 12), (21, 9)]:
        n = (10, ny, 8)
        lo = (0, y0, 0)
        U = P.random_state(n, seed=y0, amp=0.15)
        R = torch.empty((5, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
        h.rhs_box(torch.from_numpy(U).cuda(), dxinv, R, lo=lo)
        h.sync_check()
        ref = orc.rhs(sc, cl, U, dxinv, lo=lo, walls=(1, 1, 0, 29), nthreads=4)
        np.testing.assert_array_equal(R.cpu().numpy(), ref)


@pytest.mark.parametrize("skw", [SCHEMES[0], SCHEMES[3]], ids=["keep4", "weno"])
def test_steps_between_walls_match_oracle(orc, skw):
    """Channel-like box: periodic x and z, code-6 walls in y whose ghost
    cells keep the caller's values; three SSPRK3 steps."""
    n = (16, 12, 8)
    U = P.random_state(n, seed=5, amp=0.1)
    dx = (1.0 / 16, 1.0 / 12, 1.0 / 8)
    cl = P.Closures.nondimensional(1.0 / 200.0)
    sc = P.Scheme(**skw)
    bc = (-1, 6, -1)
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=bc, bc_hi=bc)
    dt = 2e-4
    S = U
    for _ in range(3):
        lev.advance(lev.time, dt)
        S = orc.advance(sc, cl, S, [1.0 / v for v in dx], bc, bc, dt, nthreads=4)
    lev.h.sync_check()
    check(lev.valid().cpu().numpy(), P.valid(S), skw)


def test_level_between_walls_matches_one_box():
    """A level of uneven boxes with code-6 y walls stepped as one graph
    equals one box covering the domain (ghosts beyond the walls: the initial
    field's, in every slot)."""
    n = (24, 20, 12)
    U = P.random_state(n, seed=8, amp=0.1)
    dx = (1.0 / 24, 1.0 / 20, 1.0 / 12)
    cl = P.Closures.nondimensional(1.0 / 200.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    bc = (-1, 6, -1)
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=bc, bc_hi=bc)
    for _ in range(2):
        lev.advance(lev.time, 1e-4)
    ref = lev.valid().cpu().numpy()
    h = capi.Handle(sc, cl)
    edges = [(0, 10, 24), (0, 7, 13, 20), (0, 12)]
    los, slots = [], []
    for z0, z1 in zip(edges[2][:-1], edges[2][1:]):
        for y0, y1 in zip(edges[1][:-1], edges[1][1:]):
            for x0, x1 in zip(edges[0][:-1], edges[0][1:]):
                B = np.ascontiguousarray(U[:, z0:z1 + 2 * NG, y0:y1 + 2 * NG, x0:x1 + 2 * NG])
                t = torch.from_numpy(B).cuda()
                slots.append([t, t.clone(), t.clone()])
                los.append((x0, y0, z0))
    bl = capi.BoxList(h, los, slots, [1.0 / v for v in dx])
    bl.set_domain((0, 0, 0), n, bc, bc)
    s1, w1, w2 = 0, 1, 2
    for _ in range(2):
        r = bl.step(3, 3, 1e-4, s1, w1, w2, use_graph=True)
        others = [s for s in (0, 1, 2) if s != r]
        s1, w1, w2 = r, others[0], others[1]
    h.sync_check()
    out = np.empty_like(ref)
    for lo, sl in zip(los, slots):
        V = sl[s1][:, NG:-NG, NG:-NG, NG:-NG].cpu().numpy()
        x0, y0, z0 = lo
        out[:, z0:z0 + V.shape[1], y0:y0 + V.shape[2], x0:x0 + V.shape[3]] = V
    np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("walls", [(1, 1), (1, 0)])
@pytest.mark.parametrize("skw", [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=1, order_keep=6, rhs_visc=0),
                                 dict(flux_euler=2, rhs_visc=1)], ids=["keep4-visc", "keep6", "weno-visc"])
def test_vjp_on_walls_every_entry(orc, skw, walls):
    """The RHS VJP next to code-6 walls (reduced KEEP faces, one-sided
    viscous y derivatives on the wall's ghost row), every entry of J^T v
    against the oracle's dual-number JVP with the same walls."""
    n = (4, 7, 3)
    lo = (1, -2, 0)
    U = P.random_state(n, seed=51 + walls[1], amp=0.15)
    dxinv = (4.0, 7.0, 3.0)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(**skw)
    h = capi.Handle(sc, cl)
    bl = (-1, 6 if walls[0] else 2, -1)
    bh = (-1, 6 if walls[1] else 2, -1)
    h.set_domain(lo, n, bl, bh)
    v = np.random.default_rng(52).standard_normal((5, n[2], n[1], n[0]))
    Ud = torch.from_numpy(U).cuda()
    ub = torch.empty_like(Ud)
    h.rhs_vjp_box(Ud, torch.from_numpy(v).cuda(), ub, dxinv, lo=lo)
    h.sync_check()
    ub = ub.cpu().numpy()
    wl = (walls[0], walls[1], lo[1], lo[1] + n[1] - 1)
    G = np.zeros_like(U)
    W = np.zeros_like(U)
    for idx in np.ndindex(U.shape):
        W[idx] = 1.0
        _, JW = orc.rhs_jvp(sc, cl, U, W, dxinv, lo=lo, walls=wl)
        G[idx] = np.sum(v * JW)
        W[idx] = 0.0
    scale = np.abs(G).max()
    bad = np.argwhere(np.abs(G - ub) > 1e-10 * scale)
    assert len(bad) == 0, [(tuple(int(x) for x in b), G[tuple(b)], ub[tuple(b)]) for b in bad[:10]]


def test_stage_vjp_rejects_walls():
    """The RK-stage VJP folds ghost cotangents back through the ghost fill;
    beyond a code-6 side the ghosts come from the caller's bcnormal, so a
    handle with walls is refused there (the RHS VJP above accepts it, and
    the ghosted stage VJP of test_gpu_adjoint_walls.py covers RK stages)."""
    cl = P.Closures.nondimensional(1e-2)
    h = capi.Handle(P.Scheme(), cl)
    h.set_domain((0, 0, 0), (8, 8, 8), (-1, 6, -1), (-1, 6, -1))
    U = torch.from_numpy(P.random_state((8, 8, 8), seed=1)).cuda()
    z = torch.zeros((5, 8, 8, 8), dtype=torch.float64, device="cuda")
    prog = capi.rk_program(3, 3, 1e-3)[0]
    with pytest.raises(capi.AmrsError):
        h.rk_stage_vjp_box(prog, (-1, 6, -1), (-1, 6, -1), U, z, z.clone(), z.clone(), (8.0, 8.0, 8.0))
