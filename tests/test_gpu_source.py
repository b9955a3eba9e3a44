"""cns.rhs_source with a body-force user_source (the channel problem's form,
exm/Channel/prob.h:189-193): the source step of compute_rhs on every GPU
path (fused KEEP kernel, face-array WENO5 / MUSCL / JST, box lists, RK
stages) against the oracle, which the reference build pins; and its reverse
in the RHS VJP."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import adjoint, capi, cns
from amrsolver_gb300 import problems as P
from tests import golden_io as G

pytestmark = pytest.mark.gpu
NG = P.NGHOST


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


SCHEMES = [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=1, order_keep=6, rhs_visc=0),
           dict(flux_euler=2, rhs_visc=1), dict(flux_euler=0, rhs_visc=1),
           dict(flux_euler=1, order_keep=4, rhs_visc=1, art_diss=1)]
FORCES = [(3.5, 0.0, 0.0), (0.7, -2.0, 0.3)]


def check(got, ref, skw):
    if skw.get("flux_euler") == 2:
        assert G.relmax(got, ref) <= 1e-13
    else:
        np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("force", FORCES)
@pytest.mark.parametrize("skw", SCHEMES, ids=lambda d: "-".join("%s%s" % kv for kv in d.items()))
def test_rhs_with_source(orc, skw, force):
    n = (12, 10, 9)
    lo = (3, -2, 1)
    U = P.random_state(n, seed=5 + len(str(skw)), amp=0.15)
    dxinv = (12.0, 10.0, 9.0)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(rhs_source=1, body_force=force, **skw)
    h = capi.Handle(sc, cl)
    R = torch.empty((5, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    h.rhs_box(dev(U), dxinv, R, lo=lo)
    h.sync_check()
    ref = orc.rhs(sc, cl, U, dxinv, lo=lo, nthreads=4)
    check(R.cpu().numpy(), ref, skw)
    assert not np.array_equal(ref, orc.rhs(P.Scheme(**skw), cl, U, dxinv, lo=lo, nthreads=4))


def test_source_off_is_the_plain_rhs(orc):
    n = (10, 8, 6)
    U = P.random_state(n, seed=3)
    dxinv = (10.0, 8.0, 6.0)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    ref = orc.rhs(sc, cl, U, dxinv, nthreads=4)
    for setting in [(0, (3.0, 0.0, 0.0)), (1, (0.0, 0.0, 0.0))]:
        h = capi.Handle(sc, cl)
        h.set_source(setting[1], on=bool(setting[0]))
        R = torch.empty((5, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
        h.rhs_box(dev(U), dxinv, R)
        h.sync_check()
        np.testing.assert_array_equal(R.cpu().numpy(), ref)


@pytest.mark.parametrize("skw", [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=2, rhs_visc=1)],
                         ids=["keep4_visc", "weno_visc"])
def test_steps_with_source(orc, skw):
    """Five SSPRK3 steps of a TGV 20^3 driven by an x body force."""
    U, dx = P.tgv(20, mach=0.2)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    sc = P.Scheme(rhs_source=1, body_force=(2.0, 0.0, 0.0), **skw)
    lev = cns.CNSLevel(sc, cl, U, dx)
    ref = U.copy()
    dxinv = [1.0 / h for h in dx]
    for _ in range(5):
        lev.advance(lev.time, 1e-2)
        ref = orc.advance(sc, cl, ref, dxinv, (-1, -1, -1), (-1, -1, -1), 1e-2, nthreads=4)
    lev.h.sync_check()
    check(lev.valid().cpu().numpy(), P.valid(ref), skw)
    # the force accelerated the flow in x: total x momentum grew by rho_total f t
    mx0 = float(P.valid(U)[1].sum())
    mx = float(lev.valid()[1].sum())
    rho = float(P.valid(U)[0].sum())
    assert abs((mx - mx0) - rho * 2.0 * 5e-2) <= 1e-9 * rho


def test_boxlist_graph_step_with_source(orc):
    """The box-list path (one launch per kernel kind, CUDA graph) carries the
    handle's source into its closures table."""
    specs, fields, dx = P.batched_boxes(nboxes=6, seed=11, edges=(8, 16))
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1, body_force=(0.0, 1.5, 0.0))
    dxinv = [1.0 / v for v in dx]
    h = capi.Handle(sc, cl)
    slots = []
    for U in fields:
        t = dev(U)
        slots.append([t, t.clone(), t.clone()])
    bl = capi.BoxList(h, [s.lo for s in specs], slots, dxinv)
    dt = 2e-3
    res = bl.step(3, 3, dt, use_graph=True)
    h.sync_check()
    from tests.test_gpu_boxlist import oracle_step_frozen
    for b, (s, U) in enumerate(zip(specs, fields)):
        ref = oracle_step_frozen(orc, sc, cl, U, dxinv, s.lo, dt)
        np.testing.assert_array_equal(slots[b][res][:, NG:-NG, NG:-NG, NG:-NG].cpu().numpy(), ref)


@pytest.mark.parametrize("skw", [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=2, rhs_visc=1)],
                         ids=["keep4_visc", "weno_visc"])
def test_vjp_with_source_dot_product(orc, skw):
    n = 10
    U, dx = P.tgv(n, mach=0.2)
    U = U * (1.0 + 0.01 * np.random.default_rng(2).standard_normal(U.shape))
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(rhs_source=1, body_force=(1.5, -0.5, 0.25), **skw)
    dxinv = [1.0 / h for h in dx]
    rng = np.random.default_rng(8)
    W = rng.standard_normal(U.shape)
    v = rng.standard_normal((5, n, n, n))
    _, JW = orc.rhs_jvp(sc, cl, U, W, dxinv, nthreads=4)
    h = capi.Handle(sc, cl)
    ubar = torch.empty_like(dev(U))
    h.rhs_vjp_box(dev(U), dev(v), ubar, dxinv)
    h.sync_check()
    lhs = float(np.sum(v * JW))
    rhs = float(np.sum(ubar.cpu().numpy() * W))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + np.linalg.norm(v) * np.linalg.norm(JW))


def test_step_vjp_with_source_vs_fd():
    """Whole SSPRK3 step with an x body force: <g, step'(U) w> by central
    differences against the step VJP."""
    n = 12
    U, dx = P.tgv(n, mach=0.2)
    U = U * (1.0 + 0.01 * np.random.default_rng(4).standard_normal(U.shape))
    cl = P.Closures.nondimensional(1.0 / 300.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1, body_force=(4.0, 0.0, 0.0))
    lev = cns.CNSLevel(sc, cl, U, dx)
    dt = 1e-2
    Uv = dev(P.valid(U).copy())
    g = dev(np.random.default_rng(6).standard_normal(Uv.shape))
    S = torch.zeros(lev.shape, dtype=torch.float64, device="cuda")
    S[:, NG:-NG, NG:-NG, NG:-NG] = Uv
    stages, _ = adjoint._forward_step(lev, S, dt)
    ubar, _ = adjoint._step_vjp(lev, stages, dt, g)

    def f(x):
        T = torch.zeros_like(S)
        T[:, NG:-NG, NG:-NG, NG:-NG] = x
        _, out = adjoint._forward_step(lev, T, dt)
        return float(torch.sum(g * out[:, NG:-NG, NG:-NG, NG:-NG]))

    eps = 1e-6
    for k in range(4):
        W = np.random.default_rng(30 + k).standard_normal(Uv.shape)
        for c in range(5):
            W[c] *= float(Uv[c].abs().mean()) + 1e-3
        W = dev(W)
        fd = (f(Uv + eps * W) - f(Uv - eps * W)) / (2 * eps)
        ad = float(torch.sum(ubar * W))
        assert abs(fd - ad) <= 1e-6 * abs(ad), (k, fd, ad)
    lev.h.sync_check()
