"""A level of several boxes tiling one domain (amrs_boxlist_set_domain):
the ghost fill copies neighbour cells, periodic images and physical BCs in
one launch, so a level of uneven boxes stepped as one graph must give the
same bits as a single box covering the domain."""
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


def split(U, cuts):
    """Boxes of a domain field U (ghosted) at the given cut points per axis
    (x, y, z); each box gets its valid cells and NaN ghosts."""
    n = [U.shape[3] - 2 * G, U.shape[2] - 2 * G, U.shape[1] - 2 * G]
    edges = [[0] + list(c) + [n[d]] for d, c in enumerate(cuts)]
    los, fields = [], []
    for z0, z1 in zip(edges[2][:-1], edges[2][1:]):
        for y0, y1 in zip(edges[1][:-1], edges[1][1:]):
            for x0, x1 in zip(edges[0][:-1], edges[0][1:]):
                B = np.full((5, z1 - z0 + 2 * G, y1 - y0 + 2 * G, x1 - x0 + 2 * G), np.nan)
                B[:, G:-G, G:-G, G:-G] = U[:, G + z0:G + z1, G + y0:G + y1, G + x0:G + x1]
                los.append((x0, y0, z0))
                fields.append(B)
    return los, fields


def run_level(sc, cl, U, dx, cuts, bc, dt, steps):
    los, fields = split(U, cuts)
    h = capi.Handle(sc, cl)
    slots = [[torch.from_numpy(f).cuda() for _ in range(3)] for f in fields]
    bl = capi.BoxList(h, los, slots, [1.0 / v for v in dx])
    n = (U.shape[3] - 2 * G, U.shape[2] - 2 * G, U.shape[1] - 2 * G)
    bl.set_domain((0, 0, 0), n, bc, bc)
    s1, w1, w2 = 0, 1, 2
    for _ in range(steps):
        r = bl.step(3, 3, dt, s1, w1, w2, use_graph=True)
        others = [s for s in (0, 1, 2) if s != r]
        s1, w1, w2 = r, others[0], others[1]
    h.sync_check()
    out = np.empty((5,) + U.shape[1:])[:, G:-G, G:-G, G:-G].copy()
    for lo, sl in zip(los, slots):
        V = sl[s1][:, G:-G, G:-G, G:-G].cpu().numpy()
        x0, y0, z0 = lo
        out[:, z0:z0 + V.shape[1], y0:y0 + V.shape[2], x0:x0 + V.shape[3]] = V
    return out


def run_single(sc, cl, U, dx, bc, dt, steps):
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=bc, bc_hi=bc)
    for _ in range(steps):
        lev.advance(lev.time, dt)
    lev.h.sync_check()
    return lev.valid().cpu().numpy()


def test_periodic_level_of_uneven_boxes_matches_one_box():
    U, dx = P.tgv(48, mach=0.2)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    bc = (-1, -1, -1)
    ref = run_single(sc, cl, U, dx, bc, 2e-3, 3)
    got = run_level(sc, cl, U, dx, [(20,), (16,), (24, 40)], bc, 2e-3, 3)
    np.testing.assert_array_equal(got, ref)


def test_outflow_level_weno_matches_one_box():
    U, dx = P.sod(64, 16, 16)
    cl = P.Closures.air_sutherland()
    sc = P.Scheme(flux_euler=2, rhs_visc=0)
    bc = (2, -1, -1)
    ref = run_single(sc, cl, U, dx, bc, 2e-4, 3)
    got = run_level(sc, cl, U, dx, [(24, 40), (8,), ()], bc, 2e-4, 3)
    np.testing.assert_array_equal(got, ref)


def test_reflecting_level_matches_one_box():
    U = P.random_state((24, 24, 24), seed=9)
    dx = (1.0 / 24,) * 3
    cl = P.Closures.nondimensional(1.0 / 500.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    bc = (3, 5, 4)  # symmetry, no-slip wall, slip wall (reflections with sign flips)
    ref = run_single(sc, cl, U, dx, bc, 1e-3, 2)
    got = run_level(sc, cl, U, dx, [(8, 16), (12,), (10,)], bc, 1e-3, 2)
    np.testing.assert_array_equal(got, ref)


def test_set_domain_rejects_gaps_and_overlaps():
    U, dx = P.tgv(16)
    cl = P.Closures.nondimensional(1e-2)
    h = capi.Handle(P.Scheme(), cl)
    los, fields = split(U, [(8,), (), ()])
    slots = [[torch.from_numpy(f).cuda() for _ in range(3)] for f in fields]
    # a gap: only the first half of the domain is covered
    bl = capi.BoxList(h, los[:1], slots[:1], [1.0 / v for v in dx])
    with pytest.raises(capi.AmrsError):
        bl.set_domain((0, 0, 0), (16, 16, 16), (-1, -1, -1), (-1, -1, -1))
    # an overlap: the same box twice
    bl2 = capi.BoxList(h, [los[0], los[0]], [slots[0], slots[0]], [1.0 / v for v in dx])
    with pytest.raises(capi.AmrsError):
        bl2.set_domain((0, 0, 0), (8, 16, 16), (2, -1, -1), (2, -1, -1))
