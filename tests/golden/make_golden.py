"""Generate the golden vectors in tests/golden/ from the reference build.

The outputs come from oracle/_ref (the reference's own src/tim/CNS_advance.cpp
and kernel headers compiled by oracle/build_ref.sh), so the committed
fixtures pin the CPU restatement and the GPU path to the reference even
where the reference sources are not available.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from amrsolver_gb300 import problems as P  # noqa: E402
from oracle import build, pyoracle  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def closures(kind):
    if kind == "const":
        return P.Closures.nondimensional(1.0 / 400.0)
    return P.Closures.air_sutherland()


def dimensional_state(n, seed):
    """Random positive state with air-like temperature for the Sutherland laws."""
    U = P.random_state(n, seed=seed)
    cl = P.Closures.air_sutherland()
    rho = U[0]
    u, v, w = U[1] / rho, U[2] / rho, U[3] / rho
    T = 300.0 * (1.0 + 0.05 * np.sin(np.arange(rho.size).reshape(rho.shape)))
    p = rho * cl.Rspec * T
    return P.prims_to_cons(rho, u * 20.0, v * 20.0, w * 20.0, p, cl.gamma)


RHS_CASES = [
    # name, closures, scheme kwargs, box shape, lo, dxinv
    ("keep4_visc", "const", dict(flux_euler=1, order_keep=4, rhs_visc=1), (7, 6, 5), (2, -1, 5), (3.0, 2.5, 4.0)),
    ("keep2_visc", "const", dict(flux_euler=1, order_keep=2, rhs_visc=1), (6, 5, 4), (0, 0, 0), (2.0, 2.0, 2.0)),
    ("keep6_visc", "const", dict(flux_euler=1, order_keep=6, rhs_visc=1), (6, 5, 4), (1, 2, 3), (2.0, 3.0, 1.5)),
    ("keep4_euler", "const", dict(flux_euler=1, order_keep=4, rhs_visc=0), (6, 5, 4), (0, 0, 0), (2.0, 2.0, 2.0)),
    ("keep4_jst", "const", dict(flux_euler=1, order_keep=4, rhs_visc=1, art_diss=1), (6, 5, 4), (0, 0, 0),
     (2.0, 2.0, 2.0)),
    ("weno_visc", "const", dict(flux_euler=2, rhs_visc=1), (6, 5, 4), (-3, 0, 2), (2.0, 2.5, 3.0)),
    ("weno_euler", "const", dict(flux_euler=2, rhs_visc=0), (6, 5, 4), (0, 0, 0), (2.0, 2.0, 2.0)),
    ("riemann_visc", "const", dict(flux_euler=0, rhs_visc=1), (6, 5, 4), (0, 0, 0), (2.0, 2.0, 2.0)),
    ("riemann_euler", "const", dict(flux_euler=0, rhs_visc=0), (6, 5, 4), (4, 4, 4), (1.0, 2.0, 3.0)),
    ("keep4_suth", "suth", dict(flux_euler=1, order_keep=4, rhs_visc=1), (6, 5, 4), (0, 0, 0), (50.0, 50.0, 50.0)),
    ("weno_suth", "suth", dict(flux_euler=2, rhs_visc=1), (6, 5, 4), (0, 0, 0), (50.0, 50.0, 50.0)),
    ("riemann_suth", "suth", dict(flux_euler=0, rhs_visc=1), (6, 5, 4), (0, 0, 0), (50.0, 50.0, 50.0)),
]

WALL_CASES = [
    # name, scheme kwargs, box shape, lo, dxinv, (wall_lo, wall_hi): y sides with boundary code 6
    ("keep4_visc", dict(flux_euler=1, order_keep=4, rhs_visc=1), (6, 7, 4), (1, -2, 0), (2.0, 3.0, 2.5), (1, 1)),
    ("keep6_euler", dict(flux_euler=1, order_keep=6, rhs_visc=0), (5, 8, 4), (0, 0, 3), (2.0, 2.0, 2.0), (1, 0)),
    ("weno_visc", dict(flux_euler=2, rhs_visc=1), (5, 6, 4), (0, 3, 0), (2.0, 2.5, 3.0), (0, 1)),
]

SOURCE_CASES = [
    # name, scheme kwargs, body force (cns.rhs_source = 1), box shape, lo, dxinv; the first is the channel
    # problem's form (fx, 0, 0)
    ("keep4_visc", dict(flux_euler=1, order_keep=4, rhs_visc=1), (2.5, 0.0, 0.0), (6, 5, 4), (1, 0, -2),
     (2.0, 2.5, 3.0)),
    ("weno_visc", dict(flux_euler=2, rhs_visc=1), (0.5, -1.5, 0.25), (5, 6, 4), (0, 0, 0), (2.0, 2.0, 2.0)),
]

ADV_CASES = [
    # name, order_rk, stages_rk
    ("ssprk3", 3, 3), ("ssprk43", 3, 4), ("ssprkm2_3", 2, 3), ("euler", 1, 1), ("heun", -2, 2), ("rhsonly", 0, 1),
]


def write_wall_cases():
    """RHS of boxes on code-6 y walls (the reference's Flux_2nd_Order_KEEP and
    ViscousWallFluxes branches); the box is the domain."""
    cl = closures("const")
    ref = pyoracle.reference(cl)
    for i, (name, skw, n, lo, dxinv, walls) in enumerate(WALL_CASES):
        sc = P.Scheme(**skw)
        U = P.random_state(n, seed=300 + i)
        w = (walls[0], walls[1], lo[1], lo[1] + n[1] - 1)
        R = ref.rhs(sc, cl, U, dxinv, lo=lo, walls=w)
        np.savez_compressed(os.path.join(HERE, "wall_%s.npz" % name), U=U, dSdt=R, lo=np.array(lo),
                            dxinv=np.array(dxinv), walls=np.array(w),
                            scheme=np.array([sc.rhs_euler, sc.rhs_visc, sc.flux_euler, sc.order_keep, sc.art_diss]),
                            closures="const")


def write_source_cases():
    """RHS with cns.rhs_source on and a body-force user_source: the source
    step of the reference's compute_rhs (rhs_source_*.npz; the `force` entry
    switches it on when loaded)."""
    cl = closures("const")
    ref = pyoracle.reference(cl)
    for i, (name, skw, force, n, lo, dxinv) in enumerate(SOURCE_CASES):
        sc = P.Scheme(rhs_source=1, body_force=force, **skw)
        U = P.random_state(n, seed=400 + i)
        R = ref.rhs(sc, cl, U, dxinv, lo=lo)
        np.savez_compressed(os.path.join(HERE, "rhs_source_%s.npz" % name), U=U, dSdt=R, lo=np.array(lo),
                            dxinv=np.array(dxinv), force=np.array(force),
                            scheme=np.array([sc.rhs_euler, sc.rhs_visc, sc.flux_euler, sc.order_keep, sc.art_diss]),
                            closures="const")


def main():
    build.build_oracle()
    for kind in ("const", "suth"):
        if pyoracle.reference(closures(kind)) is None:
            raise SystemExit("reference build missing: run bash oracle/build_ref.sh REFERENCE_ROOT first")
    out = {}
    for i, (name, kind, skw, n, lo, dxinv) in enumerate(RHS_CASES):
        cl = closures(kind)
        sc = P.Scheme(**skw)
        U = dimensional_state(n, 100 + i) if kind == "suth" else P.random_state(n, seed=100 + i)
        R = pyoracle.reference(cl).rhs(sc, cl, U, dxinv, lo=lo)
        np.savez_compressed(os.path.join(HERE, "rhs_%s.npz" % name), U=U, dSdt=R, lo=np.array(lo),
                            dxinv=np.array(dxinv), scheme=np.array([sc.rhs_euler, sc.rhs_visc, sc.flux_euler,
                                                                   sc.order_keep, sc.art_diss]),
                            closures=kind)
        out[name] = float(np.abs(R).max())
    cl = closures("const")
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    U, dx = P.tgv(8)
    dxinv = [1.0 / h for h in dx]
    for name, ork, srk in ADV_CASES:
        S2 = pyoracle.reference(cl).advance(sc, cl, U, dxinv, (-1, -1, -1), (-1, -1, -1), 5e-3, ork, srk)
        np.savez_compressed(os.path.join(HERE, "adv_%s.npz" % name), U=U, S2=P.valid(S2), dxinv=np.array(dxinv),
                            dt=5e-3, order_rk=ork, stages_rk=srk)
    # Sod: WENO-LLF, outflow in x, periodic y/z, Sutherland air, dt from cns_estdt
    cls = closures("suth")
    Us, dxs = P.sod(24, 4, 4)
    ref = pyoracle.reference(cls)
    dt = ref.est_timestep(cls, Us, dxs, 0.3)
    sc = P.Scheme(flux_euler=2, rhs_visc=0)
    S2 = ref.advance(sc, cls, Us, [1.0 / h for h in dxs], (2, -1, -1), (2, -1, -1), dt, 3, 3)
    np.savez_compressed(os.path.join(HERE, "sod_step.npz"), U=Us, S2=P.valid(S2), dx=np.array(dxs), dt=dt)
    # halo fill
    V = P.random_state((5, 4, 3), seed=9)
    halo = {}
    for tag, bl, bh in [("outflow", (2, -1, -1), (2, -1, -1)), ("walls", (3, 4, 5), (5, 2, 3)),
                        ("periodic", (-1, -1, -1), (-1, -1, -1))]:
        A = V.copy()
        ref.fill_halo(A, bl, bh)
        halo["U_" + tag] = A
        halo["bc_" + tag] = np.array([bl, bh])
    np.savez_compressed(os.path.join(HERE, "halo.npz"), V=V, **halo)
    write_wall_cases()
    write_source_cases()
    print("wrote golden fixtures:", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
