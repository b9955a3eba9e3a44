"""The device bcnormal (amrs_bcnormal kind 1: the channel problem's
isothermal no-slip wall, exm/Channel/prob.h:158-186, as cns_bcfill calls it)
against the oracle's restatement: the single-box fill, the level fill of a
box list (and its step graph), and whole channel steps."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import problems as P
from tests.test_gpu_channel import channel_state
from tests.test_gpu_level import split

pytestmark = pytest.mark.gpu
G = P.NGHOST


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


CL = P.Closures.nondimensional(1.0 / 500.0)


@pytest.mark.parametrize("sides", [((-1, 6, -1), (-1, 6, -1)), ((-1, 6, -1), (-1, 2, -1)),
                                   ((2, 2, -1), (2, 6, -1))])
@pytest.mark.parametrize("tmin", [0.0, 0.72])
def test_fill_matches_oracle(orc, sides, tmin):
    """tmin 0.72 sits inside the range of extrapolated ghost temperatures,
    so the max() floor takes both branches."""
    n = (10, 8, 6)
    bl, bh = sides
    U = channel_state(n, CL, seed=4)
    dx = (0.3, 1.0 / n[1], 0.5)
    Tw = 1.0 / CL.gamma / CL.Rspec
    bn = P.BCNormal.channel_wall(Tw, n, dx, prob_lo=(0.0, 0.0, 0.0), Tmin=tmin)
    Ud = dev(U)
    capi.fill_halo_box_bcnormal(Ud, bl, bh, CL, bn)
    torch.cuda.synchronize()
    ref = U.copy()
    orc.fill_halo_bcnormal(ref, bl, bh, CL, bn)
    got = Ud.cpu().numpy()
    np.testing.assert_array_equal(got, ref)
    # the wall ghosts were written (not the caller's values)
    if bl[1] == 6:
        assert not np.array_equal(got[:, :, :G, :], U[:, :, :G, :])


def test_level_fill_and_graph_step_match_one_box(orc):
    """A level of 2 x 2 x 1 boxes with code-6 y walls and the device
    bcnormal: the fill equals the single-box fill of the domain cut into the
    boxes, and two SSPRK3 steps through the step graph equal the single box."""
    n = (16, 12, 8)
    U = channel_state(n, CL, seed=9)
    dx = (2.0 / n[0], 1.0 / n[1], 1.0 / n[2])
    bc_lo, bc_hi = (-1, 6, -1), (-1, 6, -1)
    Tw = 1.0 / CL.gamma / CL.Rspec
    bn = P.BCNormal.channel_wall(Tw, n, dx, Tmin=0.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1, body_force=(0.5, 0.0, 0.0))
    # single box
    ref = U.copy()
    orc.fill_halo_bcnormal(ref, bc_lo, bc_hi, CL, bn)
    # level
    los, fields = split(U, [[7], [5], []])
    h = capi.Handle(sc, CL)
    slots = [[dev(f) for _ in range(3)] for f in fields]
    blist = capi.BoxList(h, los, slots, [1.0 / v for v in dx])
    blist.set_domain((0, 0, 0), n, bc_lo, bc_hi)
    blist.set_bcnormal(bn)
    blist.fill_halo(0)
    h.sync_check()
    for lo, sl in zip(los, slots):
        B = sl[0].cpu().numpy()
        x0, y0, z0 = lo
        R = ref[:, z0:z0 + B.shape[1], y0:y0 + B.shape[2], x0:x0 + B.shape[3]]
        np.testing.assert_array_equal(B, R)
    # steps: the level graph against the single-box level with the same bcnormal
    dt = 2e-3
    s1, w1, w2 = 0, 1, 2
    for _ in range(2):
        r = blist.step(3, 3, dt, s1, w1, w2, use_graph=True)
        others = [s for s in (0, 1, 2) if s != r]
        s1, w1, w2 = r, others[0], others[1]
    h.sync_check()
    lev = cns.CNSLevel(sc, CL, U, dx, bc_lo=bc_lo, bc_hi=bc_hi, bcnormal=bn)
    for _ in range(2):
        lev.advance(lev.time, dt)
    lev.h.sync_check()
    one = lev.valid().cpu().numpy()
    for lo, sl in zip(los, slots):
        V = sl[s1][:, G:-G, G:-G, G:-G].cpu().numpy()
        x0, y0, z0 = lo
        np.testing.assert_array_equal(V, one[:, z0:z0 + V.shape[1], y0:y0 + V.shape[2], x0:x0 + V.shape[3]])


def test_channel_steps_device_bcnormal(orc):
    n = (24, 16, 12)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1, body_force=(0.8, 0.0, 0.0))
    U = channel_state(n, CL, seed=21)
    dx = (2.0 / n[0], 1.0 / n[1], 1.0 / n[2])
    dxinv = [1.0 / h for h in dx]
    Tw = 1.0 / CL.gamma / CL.Rspec
    bn = P.BCNormal.channel_wall(Tw, n, dx, Tmin=0.5)
    bc = (-1, 6, -1)
    lev = cns.CNSLevel(sc, CL, U, dx, bc_lo=bc, bc_hi=bc, bcnormal=bn)
    walls = (1, 1, 0, n[1] - 1)
    v = (slice(None), slice(G, -G), slice(G, -G), slice(G, -G))
    dt = 2e-3
    S1 = U.copy()
    for _ in range(3):
        lev.advance(lev.time, dt)
        S2 = S1.copy()
        for p in capi.rk_program(3, 3, dt):
            Sb = (S1 if p.src_state == 0 else S2).copy()
            orc.fill_halo_bcnormal(Sb, bc, bc, CL, bn)
            reg = [S1[v].copy(), Sb[v].copy(), orc.rhs(sc, CL, Sb, dxinv, walls=walls, nthreads=4)]
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
        S1 = S2
    lev.h.sync_check()
    np.testing.assert_array_equal(lev.valid().cpu().numpy(), P.valid(S1))


def test_bad_bcnormal_is_rejected():
    U = dev(channel_state((8, 8, 8), CL, seed=1))
    bn = P.BCNormal(Tw=-1.0, prob_lo=(0.0, 0.0, 0.0), prob_hi=(1.0, 1.0, 1.0), dx=(0.125, 0.125, 0.125))
    with pytest.raises(capi.AmrsError):
        capi.fill_halo_box_bcnormal(U, (-1, 6, -1), (-1, 6, -1), CL, bn)


def test_device_time_loop_with_walls_bcnormal_and_source():
    """The channel level's whole run as one launch (conditional-node time
    loop, fixed dt; the fill with the device bcnormal is a node of its
    body): equals the same steps taken one by one."""
    n = (16, 12, 8)
    U = channel_state(n, CL, seed=31)
    dx = (2.0 / n[0], 1.0 / n[1], 1.0 / n[2])
    bc = (-1, 6, -1)
    Tw = 1.0 / CL.gamma / CL.Rspec
    bn = P.BCNormal.channel_wall(Tw, n, dx, Tmin=0.5)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1, body_force=(0.8, 0.0, 0.0))
    los, fields = split(U, [[8], [], []])
    h = capi.Handle(sc, CL)
    slots = [[dev(f) for _ in range(3)] for f in fields]
    blist = capi.BoxList(h, los, slots, [1.0 / v for v in dx])
    blist.set_domain((0, 0, 0), n, bc, bc)
    blist.set_bcnormal(bn)
    blist.run(3, 3, stop_time=1e9, max_steps=6, dt=1.5e-3)
    t, dt, steps = blist.run_state()
    h.sync_check()
    assert steps == 6
    lev = cns.CNSLevel(sc, CL, U, dx, bc_lo=bc, bc_hi=bc, bcnormal=bn)
    for _ in range(6):
        lev.advance(lev.time, 1.5e-3)
    lev.h.sync_check()
    one = lev.valid().cpu().numpy()
    for lo, sl in zip(los, slots):
        V = sl[0][:, G:-G, G:-G, G:-G].cpu().numpy()
        x0, y0, z0 = lo
        np.testing.assert_array_equal(V, one[:, z0:z0 + V.shape[1], y0:y0 + V.shape[2], x0:x0 + V.shape[3]])


def test_step_vjp_through_device_bcnormal_vs_fd():
    """The adjoint of a walled step whose ghosts the device bcnormal fills:
    its derivative comes from the same formula in torch (autograd), checked
    against central differences of whole steps."""
    from amrsolver_gb300 import adjoint
    n = (12, 10, 8)
    U = channel_state(n, CL, seed=13)
    dx = (1.0 / n[0], 1.0 / n[1], 1.0 / n[2])
    Tw = 1.0 / CL.gamma / CL.Rspec
    bn = P.BCNormal.channel_wall(Tw, n, dx, Tmin=0.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1, body_force=(0.8, 0.0, 0.0))
    bc = (-1, 6, -1)
    lev = cns.CNSLevel(sc, CL, U, dx, bc_lo=bc, bc_hi=bc, bcnormal=bn)
    dt = 4e-3
    Uv = dev(P.valid(U).copy())
    g = dev(np.random.default_rng(5).standard_normal(Uv.shape))

    def ghosted(x):
        S = torch.zeros(lev.shape, dtype=torch.float64, device="cuda")
        S[:, G:-G, G:-G, G:-G] = x
        return S

    stages, _ = adjoint._forward_step(lev, ghosted(Uv), dt)
    ubar, _ = adjoint._step_vjp(lev, stages, dt, g)

    def f(x):
        _, out = adjoint._forward_step(lev, ghosted(x), dt)
        return float(torch.sum(g * out[:, G:-G, G:-G, G:-G]))

    eps = 1e-6
    for k in range(4):
        W = np.random.default_rng(50 + k).standard_normal(Uv.shape)
        for c in range(5):
            W[c] *= float(Uv[c].abs().mean()) + 1e-3
        W = dev(W)
        fd = (f(Uv + eps * W) - f(Uv - eps * W)) / (2 * eps)
        ad = float(torch.sum(ubar * W))
        assert abs(fd - ad) <= 1e-6 * abs(ad), (k, fd, ad)
    lev.h.sync_check()
