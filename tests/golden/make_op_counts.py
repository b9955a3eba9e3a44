"""Algorithmic operation counts of one RHS evaluation, as exact polynomials
in the edge n of a cubic box, from the oracle's op-counting scalar.

Every phase of compute_rhs (primitives, Euler face fluxes, viscous cell
fluxes, viscous face averages, divergence) does a fixed number of additions,
multiplications, divisions and square roots per cell or face of a region of
edge n + c, so each count is a cubic in n; four box sizes determine it and a
fifth checks it.  The counts follow the reference's source expressions
operation by operation (+, -, * each 1, / and sqrt each 1, no FMA in the
oracle); comparisons are not flops.  `bench.py` reads the JSON this writes,
so the roofline needs no oracle at run time.

MUSCL-Riemann and WENO5-Riemann are the exceptions: the two-shock solver's
branches (weak-wave switch, sign of u*, shock or rarefaction at the face)
make their counts depend on the data, so they are recorded for the one input
the bench times: the first RHS of the TGV 128^3 (M = 0.1, mu = 1/1600)
initial state.

    python tests/golden/make_op_counts.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from amrsolver_gb300 import problems as P  # noqa: E402
from oracle import pyoracle  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "op_counts.json")

SCHEMES = {
    "keep4_visc": dict(flux_euler=1, order_keep=4, rhs_visc=1),
    "keep4": dict(flux_euler=1, order_keep=4, rhs_visc=0),
    "weno_visc": dict(flux_euler=2, rhs_visc=1),
    "weno": dict(flux_euler=2, rhs_visc=0),
}
FIT_N = (6, 8, 10, 12)
CHECK_N = 14
# data-dependent counts: (switches, edge, TGV Mach, mu) of the bench input
DATA_DEPENDENT = {
    "muscl_visc": (dict(flux_euler=0, rhs_visc=1), 128, 0.1, 1.0 / 1600.0),
    "weno_riemann_visc": (dict(flux_euler=0, riemann_weno=1, rhs_visc=1), 128, 0.1, 1.0 / 1600.0),
}


def flops(d):
    return d["add"] + d["mul"] + d["div"] + d["sqrt"]


def counts(orc, scheme, n):
    U, dx = P.tgv(n, mach=0.3)
    cl = P.Closures.nondimensional(1.0 / 400.0)
    per = orc.rhs_counts(P.Scheme(**scheme), cl, U, [1.0 / h for h in dx], per_phase=True)
    return {ph: flops(v) for ph, v in per.items()}


def tgv_counts(orc, scheme, n, mach, mu):
    U, dx = P.tgv(n, mach=mach)
    per = orc.rhs_counts(P.Scheme(**scheme), P.Closures.nondimensional(mu), U, [1.0 / h for h in dx],
                         per_phase=True)
    return {ph: flops(v) for ph, v in per.items()}


def fit(orc, scheme):
    rows = [counts(orc, scheme, n) for n in FIT_N]
    V = np.array([[n ** 3, n ** 2, n, 1] for n in FIT_N], dtype=np.float64)
    out = {}
    for ph in rows[0]:
        y = np.array([r[ph] for r in rows], dtype=np.float64)
        c = np.linalg.solve(V, y)
        out[ph] = [int(round(x)) for x in c]
    chk = counts(orc, scheme, CHECK_N)
    for ph, c in out.items():
        got = c[0] * CHECK_N ** 3 + c[1] * CHECK_N ** 2 + c[2] * CHECK_N + c[3]
        if got != chk[ph]:
            raise RuntimeError("count of %s/%s is not a cubic in n" % (scheme, ph))
    return out


def main():
    orc = pyoracle.oracle()
    data = {"doc": "per-RHS flops (+,-,*,/,sqrt each 1) of each compute_rhs phase as cubic coefficients "
                   "[n^3, n^2, n, 1] for an n^3 box, from the oracle's op-counting scalar",
            "schemes": {name: {"switches": sc, "phases": fit(orc, sc)} for name, sc in SCHEMES.items()},
            "data_dependent": {name: {"switches": sc, "n": n, "tgv_mach": mach, "mu": mu,
                                      "phases": tgv_counts(orc, sc, n, mach, mu)}
                               for name, (sc, n, mach, mu) in DATA_DEPENDENT.items()}}
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
