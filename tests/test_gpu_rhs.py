"""GPU parity of the RHS and RK stages against the golden vectors and the oracle.

Bar: bit-for-bit equality with the reference's CPU build wherever the
operation order is reproducible (KEEP, MUSCL-Riemann, JST, viscous fluxes,
RK programs, halo, dt); WENO5 within 1e-13 relative max-norm per conserved
variable, because the reference squares its smoothness terms with pow(x,2)
(glibc) where the kernels multiply (1-ulp differences in the weights).
"""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import problems as P
from tests import golden_io as G

pytestmark = pytest.mark.gpu
WENO_TOL = 1e-13


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_rhs(scheme, closures, U, dxinv, lo=(0, 0, 0)):
    h = capi.Handle(scheme, closures)
    n = tuple(s - 6 for s in U.shape[1:])
    out = torch.full((5,) + n, float("nan"), dtype=torch.float64, device="cuda")
    Ud = dev(U)
    h.rhs_box(Ud, dxinv, out, lo=lo)
    h.sync_check()
    return out.cpu().numpy(), h


@pytest.mark.parametrize("case", G.rhs_cases(), ids=lambda c: c["name"])
def test_rhs_golden(case):
    R, _ = gpu_rhs(case["scheme"], case["closures"], case["U"], case["dxinv"], case["lo"])
    if case["scheme"].flux_euler == 2:
        assert G.relmax(R, case["dSdt"]) <= WENO_TOL
    else:
        np.testing.assert_array_equal(R, case["dSdt"])


@pytest.mark.parametrize("case", G.adv_cases(), ids=lambda c: c["name"])
def test_advance_golden(case):
    cl = G.closures("const")
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    lev = cns.CNSLevel(sc, cl, case["U"], [1.0 / v for v in case["dxinv"]], order_rk=case["order_rk"],
                       stages_rk=case["stages_rk"])
    lev.advance(0.0, case["dt"])
    lev.h.sync_check()
    np.testing.assert_array_equal(lev.valid().cpu().numpy(), case["S2"])


def test_halo_golden():
    z = np.load(G.HERE + "/halo.npz")
    for tag in ("outflow", "walls", "periodic"):
        U = dev(z["V"])
        bc = z["bc_" + tag]
        capi.fill_halo_box(U, tuple(bc[0]), tuple(bc[1]))
        torch.cuda.synchronize()
        np.testing.assert_array_equal(U.cpu().numpy(), z["U_" + tag])


def test_sod_step_golden():
    z = np.load(G.HERE + "/sod_step.npz")
    cl = G.closures("suth")
    sc = P.Scheme(flux_euler=2, rhs_visc=0)
    lev = cns.CNSLevel(sc, cl, z["U"], z["dx"], bc_lo=(2, -1, -1), bc_hi=(2, -1, -1))
    dt = lev.est_time_step(0.3)
    assert dt == float(z["dt"])
    lev.advance(0.0, dt)
    assert G.relmax(lev.valid().cpu().numpy(), z["S2"]) <= WENO_TOL


SCHEMES = [dict(flux_euler=1, order_keep=o, rhs_visc=v) for o in (2, 4, 6) for v in (0, 1)] + \
          [dict(flux_euler=1, order_keep=4, rhs_visc=1, art_diss=1), dict(flux_euler=0, rhs_visc=1),
           dict(flux_euler=0, rhs_visc=0), dict(flux_euler=2, rhs_visc=1), dict(rhs_euler=0, rhs_visc=1)]


@pytest.mark.parametrize("skw", SCHEMES, ids=lambda d: "-".join("%s%s" % kv for kv in d.items()))
@pytest.mark.parametrize("n", [(8, 8, 8), (13, 7, 5), (37, 19, 11), (3, 4, 40), (1, 1, 1), (1, 6, 2), (2, 1, 9)])
def test_rhs_vs_oracle_random(orc, skw, n):
    sc = P.Scheme(**skw)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    U = P.random_state(n, seed=sum(n) + len(str(skw)), amp=0.2)
    lo = (n[0] % 5 - 2, -n[1], 7)
    dxinv = (1.7, 2.9, 0.8)
    R, _ = gpu_rhs(sc, cl, U, dxinv, lo)
    ref = orc.rhs(sc, cl, U, dxinv, lo=lo)
    if sc.flux_euler == 2 and sc.rhs_euler:
        assert G.relmax(R, ref) <= WENO_TOL
    else:
        np.testing.assert_array_equal(R, ref)


@pytest.mark.parametrize("visc", [0, 1])
def test_muscl_strong_waves_bitexact(orc, visc):
    """MUSCL-Riemann on cell-to-cell jumps of a few decades in density and
    pressure and supersonic velocities of both signs: every branch of the
    two-shock solver (shock or rarefaction on each side, sign of u*,
    supersonic side state, star state, transonic mix) is taken, and the
    result equals the oracle's to the bit."""
    rng = np.random.default_rng(7 + visc)
    n = (24, 20, 18)
    shape = (n[2] + 6, n[1] + 6, n[0] + 6)
    rho = np.exp(rng.normal(0.0, 1.0, shape))
    p = np.exp(rng.normal(0.0, 1.5, shape))
    c = np.sqrt(1.4 * p / rho)
    u, v, w = (rng.normal(0.0, 1.2, shape) * c for _ in range(3))
    U = P.prims_to_cons(rho, u, v, w, p, 1.4)
    sc = P.Scheme(flux_euler=0, rhs_visc=visc)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    dxinv = (1.3, 0.7, 2.1)
    R, _ = gpu_rhs(sc, cl, U, dxinv)
    ref = orc.rhs(sc, cl, U, dxinv)
    assert np.isfinite(ref).all()
    np.testing.assert_array_equal(R, ref)


def test_other_flux_values_take_the_riemann_path():
    """compute_rhs sends every flux_euler other than 1 and 2 to the Riemann
    path (src/tim/CNS_advance.cpp:221-223); the library does the same."""
    U = P.random_state((10, 9, 8), seed=4, amp=0.2)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    R0, _ = gpu_rhs(P.Scheme(flux_euler=0, rhs_visc=1), cl, U, (1.0, 2.0, 3.0))
    for fe in (-1, 3, 7):
        R, _ = gpu_rhs(P.Scheme(flux_euler=fe, rhs_visc=1), cl, U, (1.0, 2.0, 3.0))
        np.testing.assert_array_equal(R, R0)
    W0, _ = gpu_rhs(P.Scheme(flux_euler=0, riemann_weno=1, rhs_visc=1), cl, U, (1.0, 2.0, 3.0))
    W, _ = gpu_rhs(P.Scheme(flux_euler=5, riemann_weno=1, rhs_visc=1), cl, U, (1.0, 2.0, 3.0))
    np.testing.assert_array_equal(W, W0)
    assert not np.array_equal(W0, R0)


def test_tgv_rhs_bitexact_64(orc):
    """TGV 64^3, KEEP4 + viscous: GPU == oracle to the last bit."""
    U, dx = P.tgv(64)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    R, h = gpu_rhs(sc, cl, U, dxinv)
    np.testing.assert_array_equal(R, orc.rhs(sc, cl, U, dxinv, nthreads=8))


def test_tgv_steps_bitexact(orc):
    """Five SSPRK3 steps of TGV 24^3: GPU == oracle after N steps (bar 1e-10)."""
    U, dx = P.tgv(24)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    lev = cns.CNSLevel(sc, cl, U, dx)
    ref = U.copy()
    dxinv = [1.0 / h for h in dx]
    for _ in range(5):
        lev.advance(lev.time, 1e-2)
        ref = orc.advance(sc, cl, ref, dxinv, (-1, -1, -1), (-1, -1, -1), 1e-2)
    lev.h.sync_check()
    np.testing.assert_array_equal(lev.valid().cpu().numpy(), P.valid(ref))


def test_fused_matches_plain_keep():
    """The fused KEEP kernel (pair terms shared across faces) and the
    face-array path with JST switched off produce identical bits."""
    U, dx = P.tgv(40)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    dxinv = [1.0 / h for h in dx]
    Rf, _ = gpu_rhs(P.Scheme(flux_euler=1, order_keep=4), cl, U, dxinv)
    # JST with Cshock = Cdamp = 0 routes through the face-array path and adds zeros
    cl0 = P.Closures.nondimensional(1.0 / 800.0)
    cl0.Cshock = 0.0
    cl0.Cdamp = 0.0
    Rp, _ = gpu_rhs(P.Scheme(flux_euler=1, order_keep=4, art_diss=1), cl0, U, dxinv)
    np.testing.assert_array_equal(Rf, Rp)


def test_conservation_periodic():
    """Periodic domain: sum of dS/dt over the box is zero to round-off."""
    U, dx = P.tgv(32, mach=0.3)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    R, _ = gpu_rhs(P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1), cl, U, [1.0 / h for h in dx])
    scale = np.abs(R).reshape(5, -1).max(axis=1) + 1.0
    assert np.all(np.abs(R.reshape(5, -1).sum(axis=1)) <= 1e-9 * scale * R[0].size)


def test_oversized_box_is_rejected():
    """A box whose cells with ghosts reach 2^31 is refused before anything
    runs (the arrays passed cover only a 4^3 box, so a missed check would
    still stop at the layout check)."""
    import ctypes
    h = capi.Handle(P.Scheme(), P.Closures.nondimensional(1e-3))
    U = torch.zeros((5, 10, 10, 10), dtype=torch.float64, device="cuda")
    out = torch.zeros((5, 4, 4, 4), dtype=torch.float64, device="cuda")
    L = capi.load()
    big = capi.c_box((0, 0, 0), (1400, 1400, 1400))
    st = L.amrs_rhs_box(h.h, ctypes.byref(big), capi.d3((1.0, 1.0, 1.0)), capi.array4(U, (0, 0, 0), 3),
                        capi.array4(out, (0, 0, 0), 0), None)
    assert st == 2  # AMRS_ERR_BOX
    h.sync_check()


def test_bounded_wait_timeout_reports_and_context_survives():
    """A device wait that runs out (an mbarrier nothing arrives at, bounded
    to a few thousand polls) raises the handle's error flag: sync_check
    reports AMRS_ERR_TIMEOUT once, clears it, and the next RHS is correct."""
    U = P.random_state((6, 5, 4), seed=9, amp=0.2)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    cl = P.Closures.nondimensional(1.0 / 300.0)
    h = capi.Handle(sc, cl)
    h.debug_wait_timeout(4096)
    with pytest.raises(capi.AmrsError, match="(?i)time"):
        h.sync_check()
    h.sync_check()  # cleared
    out = torch.empty((5, 4, 5, 6), dtype=torch.float64, device="cuda")
    h.rhs_box(torch.from_numpy(U).cuda(), (1.0, 1.0, 1.0), out)
    h.sync_check()
    R, _ = gpu_rhs(sc, cl, U, (1.0, 1.0, 1.0))
    np.testing.assert_array_equal(out.cpu().numpy(), R)
    with pytest.raises(capi.AmrsError):
        h.debug_wait_timeout(0)


def test_bad_inputs_fail_loudly():
    h = capi.Handle(P.Scheme(), P.Closures.nondimensional(1e-3))
    U = torch.zeros((5, 10, 10, 10), dtype=torch.float64, device="cuda")
    out = torch.zeros((5, 3, 3, 3), dtype=torch.float64, device="cuda")  # smaller than the 4^3 box
    with pytest.raises(capi.AmrsError):
        h.rhs_box(U, (1.0, 1.0, 1.0), out)
    with pytest.raises(capi.AmrsError):
        capi.fill_halo_box(U, (7, -1, -1), (7, -1, -1))  # no such boundary code
    with pytest.raises(capi.AmrsError):
        capi.fill_halo_box(U, (-1, -1, -1), (2, -1, -1))  # periodic on one side only
    with pytest.raises(capi.AmrsError):
        capi.Handle(P.Scheme(flux_euler=1, order_keep=3), P.Closures.nondimensional(1e-3))
