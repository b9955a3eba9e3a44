"""Loading helpers for the golden vectors in tests/golden/."""
import glob
import os

import numpy as np

from amrsolver_gb300 import problems as P

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def closures(kind):
    kind = str(kind)
    if kind == "const":
        return P.Closures.nondimensional(1.0 / 400.0)
    return P.Closures.air_sutherland()


def rhs_cases():
    out = []
    for f in sorted(glob.glob(os.path.join(HERE, "rhs_*.npz"))):
        z = np.load(f)
        s = z["scheme"]
        sc = P.Scheme(rhs_euler=int(s[0]), rhs_visc=int(s[1]), flux_euler=int(s[2]), order_keep=int(s[3]),
                      art_diss=int(s[4]))
        if "force" in z.files:  # cns.rhs_source with a body force
            sc.rhs_source = 1
            sc.body_force = tuple(float(v) for v in z["force"])
        out.append(dict(name=os.path.basename(f)[4:-4], U=z["U"], dSdt=z["dSdt"], lo=tuple(int(v) for v in z["lo"]),
                        dxinv=tuple(float(v) for v in z["dxinv"]), scheme=sc, closures=closures(z["closures"])))
    return out


def wall_cases():
    """RHS fixtures of boxes on code-6 y walls (walls = wall_lo, wall_hi, dom_lo_y, dom_hi_y)."""
    out = []
    for f in sorted(glob.glob(os.path.join(HERE, "wall_*.npz"))):
        z = np.load(f)
        s = z["scheme"]
        sc = P.Scheme(rhs_euler=int(s[0]), rhs_visc=int(s[1]), flux_euler=int(s[2]), order_keep=int(s[3]),
                      art_diss=int(s[4]))
        out.append(dict(name=os.path.basename(f)[5:-4], U=z["U"], dSdt=z["dSdt"], lo=tuple(int(v) for v in z["lo"]),
                        dxinv=tuple(float(v) for v in z["dxinv"]), walls=tuple(int(v) for v in z["walls"]),
                        scheme=sc, closures=closures(z["closures"])))
    return out


def adv_cases():
    out = []
    for f in sorted(glob.glob(os.path.join(HERE, "adv_*.npz"))):
        z = np.load(f)
        out.append(dict(name=os.path.basename(f)[4:-4], U=z["U"], S2=z["S2"], dxinv=tuple(z["dxinv"]),
                        dt=float(z["dt"]), order_rk=int(z["order_rk"]), stages_rk=int(z["stages_rk"])))
    return out


def relmax(a, b):
    """max |a-b| / max |b| per conserved component (max over components)."""
    a = np.asarray(a).reshape(a.shape[0], -1)
    b = np.asarray(b).reshape(b.shape[0], -1)
    r = 0.0
    for n in range(a.shape[0]):
        den = np.abs(b[n]).max()
        num = np.abs(a[n] - b[n]).max()
        r = max(r, num / den if den > 0 else num)
    return r
