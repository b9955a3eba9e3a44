"""The CPU restatement against the reference build on fresh random inputs.

Runs only where oracle/_ref exists (the reference sources compiled by
oracle/build_ref.sh); it checks bit-for-bit agreement on inputs the golden
fixtures do not cover.
"""
import numpy as np
import pytest

from amrsolver_gb300 import problems as P
from oracle import pyoracle

CL = P.Closures.nondimensional(1.0 / 800.0)
REF = pyoracle.reference(CL)
pytestmark = pytest.mark.skipif(REF is None, reason="reference build (oracle/_ref) not present")

SCHEMES = [dict(flux_euler=1, order_keep=o, rhs_visc=v, art_diss=a) for o in (2, 4, 6) for v in (0, 1)
           for a in (0, 1)] + [dict(flux_euler=f, rhs_visc=v) for f in (0, 2) for v in (0, 1)]


@pytest.mark.parametrize("skw", SCHEMES, ids=lambda d: "-".join("%s%s" % kv for kv in d.items()))
def test_rhs_bitexact(orc, skw):
    sc = P.Scheme(**skw)
    rng = np.random.default_rng(len(str(skw)))
    n = tuple(int(v) for v in rng.integers(3, 9, 3))
    U = P.random_state(n, seed=int(rng.integers(1 << 30)), amp=0.2)
    lo = tuple(int(v) for v in rng.integers(-5, 5, 3))
    dxinv = tuple(float(v) for v in rng.uniform(1.0, 5.0, 3))
    np.testing.assert_array_equal(orc.rhs(sc, CL, U, dxinv, lo=lo), REF.rhs(sc, CL, U, dxinv, lo=lo))


WALL_SCHEMES = [dict(flux_euler=1, order_keep=o, rhs_visc=v) for o in (2, 4, 6) for v in (0, 1)] + \
    [dict(flux_euler=2, rhs_visc=1), dict(flux_euler=0, rhs_visc=1)]


@pytest.mark.parametrize("walls", [(1, 1), (1, 0), (0, 1)])
@pytest.mark.parametrize("skw", WALL_SCHEMES, ids=lambda d: "-".join("%s%s" % kv for kv in d.items()))
def test_rhs_walls_bitexact(orc, skw, walls):
    """y sides with boundary code 6: the reference's own Flux_2nd_Order_KEEP
    and ViscousWallFluxes branches of compute_rhs against the restatement."""
    sc = P.Scheme(**skw)
    rng = np.random.default_rng(len(str(skw)) + 7 * walls[0] + walls[1])
    n = tuple(int(v) for v in rng.integers(4, 10, 3))
    U = P.random_state(n, seed=int(rng.integers(1 << 30)), amp=0.2)
    lo = tuple(int(v) for v in rng.integers(-5, 5, 3))
    dxinv = tuple(float(v) for v in rng.uniform(1.0, 5.0, 3))
    w = (walls[0], walls[1], lo[1], lo[1] + n[1] - 1)
    np.testing.assert_array_equal(orc.rhs(sc, CL, U, dxinv, lo=lo, walls=w), REF.rhs(sc, CL, U, dxinv, lo=lo, walls=w))


@pytest.mark.parametrize("ork,srk", [(3, 3), (3, 4), (2, 2), (2, 4), (1, 1), (0, 1), (-2, 2)])
def test_advance_bitexact(orc, ork, srk):
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    U, dx = P.tgv(10, mach=0.2)
    dxinv = [1.0 / h for h in dx]
    a = orc.advance(sc, CL, U, dxinv, (-1, -1, -1), (-1, -1, -1), 3e-3, ork, srk)
    b = REF.advance(sc, CL, U, dxinv, (-1, -1, -1), (-1, -1, -1), 3e-3, ork, srk)
    np.testing.assert_array_equal(P.valid(a), P.valid(b))


SOURCE_FORCES = [(3.5, 0.0, 0.0), (0.0, -1.25, 0.0), (0.7, 2.0, -0.3)]


@pytest.mark.parametrize("force", SOURCE_FORCES)
@pytest.mark.parametrize("skw", [dict(flux_euler=1, order_keep=4, rhs_visc=1), dict(flux_euler=2, rhs_visc=1),
                                 dict(flux_euler=0, rhs_visc=0)], ids=["keep4_visc", "weno_visc", "muscl"])
def test_rhs_source_bitexact(orc, skw, force):
    """cns.rhs_source: the source step of the reference's compute_rhs (after
    the divergence, from the stage input) with a body-force user_source; the
    first force is the channel problem's form, (fx, 0, 0)."""
    sc = P.Scheme(rhs_source=1, body_force=force, **skw)
    rng = np.random.default_rng(17 + len(str(skw)))
    n = tuple(int(v) for v in rng.integers(4, 9, 3))
    U = P.random_state(n, seed=int(rng.integers(1 << 30)), amp=0.2)
    lo = tuple(int(v) for v in rng.integers(-5, 5, 3))
    dxinv = tuple(float(v) for v in rng.uniform(1.0, 5.0, 3))
    a = orc.rhs(sc, CL, U, dxinv, lo=lo)
    np.testing.assert_array_equal(a, REF.rhs(sc, CL, U, dxinv, lo=lo))
    # the source changed the momentum and energy RHS, not the mass RHS
    b = orc.rhs(P.Scheme(**skw), CL, U, dxinv, lo=lo)
    np.testing.assert_array_equal(a[0], b[0])
    assert not np.array_equal(a[4], b[4])


def test_advance_with_source_bitexact(orc):
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1, body_force=(2.0, 0.0, 0.0))
    U, dx = P.tgv(10, mach=0.2)
    dxinv = [1.0 / h for h in dx]
    a = orc.advance(sc, CL, U, dxinv, (-1, -1, -1), (-1, -1, -1), 3e-3, 3, 3)
    b = REF.advance(sc, CL, U, dxinv, (-1, -1, -1), (-1, -1, -1), 3e-3, 3, 3)
    np.testing.assert_array_equal(P.valid(a), P.valid(b))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_prim_stats_bitexact(orc, seed):
    """CNS::printTotal's primitive extrema and the reference's own pointCFL
    table (src/cls/CNS_K.h:49-59) against the restatement."""
    rng = np.random.default_rng(seed)
    n = tuple(int(v) for v in rng.integers(3, 9, 3))
    U = P.random_state(n, seed=seed + 50, amp=0.3)
    lo = tuple(int(v) for v in rng.integers(-5, 5, 3))
    dx = tuple(float(v) for v in rng.uniform(0.1, 0.5, 3))
    dt = float(rng.uniform(1e-3, 1e-2))
    a = orc.prim_stats(CL, U, dx, dt, lo=lo)
    b = REF.prim_stats(CL, U, dx, dt, lo=lo)
    np.testing.assert_array_equal(a, b)
    assert np.all(a[:6] <= a[6:12]) and np.all(a[12:] > 0)


@pytest.mark.parametrize("seed", [4, 5])
def test_plot_derive_bitexact(orc, seed):
    """The plotfile's derived variables: the reference's own derpres, dertemp
    and dervel (src/cls/CNS_K.h:76-129) against the restatement."""
    rng = np.random.default_rng(seed)
    n = tuple(int(v) for v in rng.integers(3, 8, 3))
    U = P.random_state(n, seed=seed + 70, amp=0.3)
    lo = tuple(int(v) for v in rng.integers(-4, 4, 3))
    np.testing.assert_array_equal(orc.plot_derive(CL, U, lo=lo), REF.plot_derive(CL, U, lo=lo))
