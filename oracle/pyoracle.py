"""ctypes front end of the CPU oracle library (test infrastructure only).

Loads oracle/_build/liboracle.so (built from oracle/cns_oracle.cpp) and,
when present, oracle/_ref/libcnsref.so (the reference's own kernel sources
compiled here).  Both expose the same call shapes for one box:
  rhs(U_ghosted) -> dSdt_valid, advance(...), fill_halo(...), est_timestep(...)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

NG = 3
NCONS = 5


class CClosures(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("cv", ctypes.c_double), ("cp", ctypes.c_double),
                ("Rspec", ctypes.c_double), ("visc_law", ctypes.c_int32), ("cond_law", ctypes.c_int32),
                ("visc_ref", ctypes.c_double), ("Tvisc_ref", ctypes.c_double),
                ("cond_ref", ctypes.c_double), ("Tcond_ref", ctypes.c_double),
                ("Cshock", ctypes.c_double), ("Cdamp", ctypes.c_double)]


class CScheme(ctypes.Structure):
    _fields_ = [("rhs_euler", ctypes.c_int32), ("rhs_visc", ctypes.c_int32),
                ("flux_euler", ctypes.c_int32), ("order_keep", ctypes.c_int32),
                ("art_diss", ctypes.c_int32), ("rhs_source", ctypes.c_int32),
                ("force", ctypes.c_double * 3)]


class CBcNormal(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("Tw", ctypes.c_double), ("Tmin", ctypes.c_double),
                ("prob_lo", ctypes.c_double * 3), ("prob_hi", ctypes.c_double * 3), ("dx", ctypes.c_double * 3)]


def c_closures(cl):
    return CClosures(cl.gamma, cl.cv, cl.cp, cl.Rspec, int(cl.visc_law), int(cl.cond_law),
                     cl.visc_ref, cl.Tvisc_ref, cl.cond_ref, cl.Tcond_ref, cl.Cshock, cl.Cdamp)


def c_scheme(sc):
    # the oracle's flux code: 1 KEEP, 2 WENO5 LLF, 3 WENO5-Riemann (the
    # riemann_weno extension), anything else MUSCL + Riemann
    fe = int(sc.flux_euler)
    if fe not in (1, 2):
        fe = 3 if int(getattr(sc, "riemann_weno", 0)) else 0
    src = int(getattr(sc, "rhs_source", 0))
    f = getattr(sc, "body_force", (0.0, 0.0, 0.0))
    return CScheme(int(sc.rhs_euler), int(sc.rhs_visc), fe, int(sc.order_keep), int(sc.art_diss), src,
                   (ctypes.c_double * 3)(*[float(x) for x in f]))


def _i3(v):
    return (ctypes.c_int * 3)(*[int(x) for x in v])


def _d3(v):
    return (ctypes.c_double * 3)(*[float(x) for x in v])


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One loaded oracle library (the restatement or the reference build)."""

    def __init__(self, path):
        self.path = path
        self.lib = ctypes.CDLL(path)
        L = self.lib
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_compute_rhs.argtypes = [ctypes.POINTER(CScheme), ctypes.POINTER(CClosures), ip, ip, dp,
                                      dp, dp, ctypes.c_int]
        L.orc_compute_rhs.restype = ctypes.c_int
        L.orc_compute_rhs_walls.argtypes = [ctypes.POINTER(CScheme), ctypes.POINTER(CClosures), ip, ip, dp,
                                            dp, dp, ctypes.c_int, ip]
        L.orc_compute_rhs_walls.restype = ctypes.c_int
        L.orc_fill_halo.argtypes = [ip, ip, ip, ip, dp, ctypes.c_int]
        L.orc_fill_halo.restype = ctypes.c_int
        L.orc_est_timestep.argtypes = [ctypes.POINTER(CClosures), ip, ip, dp, dp, ctypes.c_int,
                                       ctypes.c_double]
        L.orc_est_timestep.restype = ctypes.c_double
        L.orc_advance.argtypes = [ctypes.POINTER(CScheme), ctypes.POINTER(CClosures), ip, ip, dp, ip, ip,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, dp, ctypes.c_int]
        L.orc_advance.restype = ctypes.c_int
        self.has_jvp = hasattr(L, "orc_compute_rhs_jvp")
        if self.has_jvp:
            L.orc_compute_rhs_jvp.argtypes = [ctypes.POINTER(CScheme), ctypes.POINTER(CClosures), ip, ip,
                                              dp, dp, dp, dp, dp, ctypes.c_int]
            L.orc_compute_rhs_jvp.restype = ctypes.c_int
            L.orc_compute_rhs_jvp_walls.argtypes = [ctypes.POINTER(CScheme), ctypes.POINTER(CClosures), ip, ip,
                                                    dp, dp, dp, dp, dp, ctypes.c_int, ip]
            L.orc_compute_rhs_jvp_walls.restype = ctypes.c_int
            L.orc_compute_rhs_count.argtypes = [ctypes.POINTER(CScheme), ctypes.POINTER(CClosures), ip,
                                                ip, dp, dp, ctypes.POINTER(ctypes.c_longlong)]
            L.orc_compute_rhs_count.restype = ctypes.c_int
        if hasattr(L, "orc_plot_derive"):
            L.orc_plot_derive.argtypes = [ctypes.POINTER(CClosures), ip, ip, dp, dp]
            L.orc_plot_derive.restype = ctypes.c_int
        if hasattr(L, "orc_prim_stats"):
            L.orc_prim_stats.argtypes = [ctypes.POINTER(CClosures), ip, ip, dp, dp, ctypes.c_double, dp]
            L.orc_prim_stats.restype = ctypes.c_int
        if hasattr(L, "orc_fill_halo_bcnormal"):
            L.orc_fill_halo_bcnormal.argtypes = [ip, ip, ip, ip, dp, ctypes.POINTER(CClosures),
                                                 ctypes.POINTER(CBcNormal)]
            L.orc_fill_halo_bcnormal.restype = ctypes.c_int

    # -------------------------------------------------------------- calls --
    def rhs(self, scheme, closures, U, dxinv, lo=(0, 0, 0), nthreads=1, walls=None):
        """dS/dt of one ghost-filled box.  walls = (wall_lo, wall_hi, dom_lo_y,
        dom_hi_y): y sides of the domain with boundary code 6."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        nz, ny, nx = (s - 2 * NG for s in U.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        out = np.empty((NCONS, nz, ny, nx))
        sc, cl = c_scheme(scheme), c_closures(closures)
        if walls is not None:
            w4 = (ctypes.c_int * 4)(*[int(v) for v in walls])
            rc = self.lib.orc_compute_rhs_walls(ctypes.byref(sc), ctypes.byref(cl), _i3(lo), _i3(hi), _d3(dxinv),
                                                _ptr(U), _ptr(out), int(nthreads), w4)
            if rc:
                raise RuntimeError("orc_compute_rhs_walls failed: %d" % rc)
            return out
        rc = self.lib.orc_compute_rhs(ctypes.byref(sc), ctypes.byref(cl), _i3(lo), _i3(hi), _d3(dxinv),
                                      _ptr(U), _ptr(out), int(nthreads))
        if rc:
            raise RuntimeError("orc_compute_rhs failed: %d" % rc)
        return out

    def rhs_jvp(self, scheme, closures, U, W, dxinv, lo=(0, 0, 0), nthreads=1, walls=None):
        U = np.ascontiguousarray(U, dtype=np.float64)
        W = np.ascontiguousarray(W, dtype=np.float64)
        nz, ny, nx = (s - 2 * NG for s in U.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        R = np.empty((NCONS, nz, ny, nx))
        JW = np.empty((NCONS, nz, ny, nx))
        sc, cl = c_scheme(scheme), c_closures(closures)
        if walls is not None:
            w4 = (ctypes.c_int * 4)(*[int(v) for v in walls])
            rc = self.lib.orc_compute_rhs_jvp_walls(ctypes.byref(sc), ctypes.byref(cl), _i3(lo), _i3(hi),
                                                    _d3(dxinv), _ptr(U), _ptr(W), _ptr(R), _ptr(JW), int(nthreads), w4)
            if rc:
                raise RuntimeError("orc_compute_rhs_jvp_walls failed: %d" % rc)
            return R, JW
        rc = self.lib.orc_compute_rhs_jvp(ctypes.byref(sc), ctypes.byref(cl), _i3(lo), _i3(hi), _d3(dxinv),
                                          _ptr(U), _ptr(W), _ptr(R), _ptr(JW), int(nthreads))
        if rc:
            raise RuntimeError("orc_compute_rhs_jvp failed: %d" % rc)
        return R, JW

    PHASES = ("prims", "euler_faces", "jst", "visc_cells", "visc_faces", "divergence")

    def rhs_counts(self, scheme, closures, U, dxinv, lo=(0, 0, 0), per_phase=False):
        """{add, mul, div, sqrt, cmp} operation counts of one RHS of this box
        (summed, or per phase of compute_rhs when per_phase)."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        nz, ny, nx = (s - 2 * NG for s in U.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        cnt = (ctypes.c_longlong * 30)()
        sc, cl = c_scheme(scheme), c_closures(closures)
        rc = self.lib.orc_compute_rhs_count(ctypes.byref(sc), ctypes.byref(cl), _i3(lo), _i3(hi),
                                            _d3(dxinv), _ptr(U), cnt)
        if rc:
            raise RuntimeError("orc_compute_rhs_count failed: %d" % rc)
        keys = ("add", "mul", "div", "sqrt", "cmp")
        per = {ph: dict(zip(keys, list(cnt)[5 * p:5 * p + 5])) for p, ph in enumerate(self.PHASES)}
        if per_phase:
            return per
        return {k: sum(per[ph][k] for ph in self.PHASES) for k in keys}

    def fill_halo_bcnormal(self, U, bc_lo, bc_hi, closures, bn, lo=(0, 0, 0)):
        """fill_halo, then the channel problem's isothermal bcnormal beyond
        code-6 y sides; bn: an object with kind, Tw, Tmin, prob_lo, prob_hi, dx."""
        assert U.flags.c_contiguous
        nz, ny, nx = (s - 2 * NG for s in U.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        cb = CBcNormal(int(bn.kind), float(bn.Tw), float(bn.Tmin), _d3(bn.prob_lo), _d3(bn.prob_hi), _d3(bn.dx))
        rc = self.lib.orc_fill_halo_bcnormal(_i3(lo), _i3(hi), _i3(bc_lo), _i3(bc_hi), _ptr(U),
                                             ctypes.byref(c_closures(closures)), ctypes.byref(cb))
        if rc:
            raise RuntimeError("orc_fill_halo_bcnormal failed: %d" % rc)

    def prim_stats(self, closures, U, dx, dt, lo=(0, 0, 0)):
        """CNS::printTotal's primitive min/max and pointCFL table of one
        ghosted box: 21 values, min[6], max[6] of (rho, u, v, w, T, p), then per
        direction max|u+c|, max|u-c|, CFL."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        nz, ny, nx = (s - 2 * NG for s in U.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        out = np.empty(21)
        rc = self.lib.orc_prim_stats(ctypes.byref(c_closures(closures)), _i3(lo), _i3(hi), _d3(dx), _ptr(U),
                                     float(dt), _ptr(out))
        if rc:
            raise RuntimeError("orc_prim_stats failed: %d" % rc)
        return out

    def plot_derive(self, closures, U, lo=(0, 0, 0)):
        """Derived plot variables (pressure, temperature, x/y/z velocity) of
        one ghosted box's valid cells: (5, nz, ny, nx)."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        nz, ny, nx = (s - 2 * NG for s in U.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        out = np.empty((5, nz, ny, nx))
        rc = self.lib.orc_plot_derive(ctypes.byref(c_closures(closures)), _i3(lo), _i3(hi), _ptr(U), _ptr(out))
        if rc:
            raise RuntimeError("orc_plot_derive failed: %d" % rc)
        return out

    def fill_halo(self, U, bc_lo, bc_hi, lo=(0, 0, 0)):
        """In-place ghost fill of a single-box domain."""
        assert U.flags.c_contiguous
        nz, ny, nx = (s - 2 * NG for s in U.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        rc = self.lib.orc_fill_halo(_i3(lo), _i3(hi), _i3(bc_lo), _i3(bc_hi), _ptr(U), int(U.shape[0]))
        if rc:
            raise RuntimeError("orc_fill_halo failed: %d" % rc)
        return U

    def est_timestep(self, closures, U, dx, cfl, nghost=NG, lo=(0, 0, 0)):
        U = np.ascontiguousarray(U, dtype=np.float64)
        nz, ny, nx = (s - 2 * nghost for s in U.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        cl = c_closures(closures)
        return float(self.lib.orc_est_timestep(ctypes.byref(cl), _i3(lo), _i3(hi), _d3(dx), _ptr(U),
                                               int(nghost), float(cfl)))

    def advance(self, scheme, closures, S1, dxinv, bc_lo, bc_hi, dt, order_rk=3, stages_rk=3,
                lo=(0, 0, 0), nthreads=1):
        """One CNS::advance step; returns S2 (ghosted; valid cells meaningful)."""
        S1 = np.ascontiguousarray(S1, dtype=np.float64).copy()
        # S2 starts as S1: its ghost cells beyond ext_dir sides (codes 1, 6)
        # are the caller's values, as in every state buffer of a level
        S2 = S1.copy()
        nz, ny, nx = (s - 2 * NG for s in S1.shape[1:])
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        sc, cl = c_scheme(scheme), c_closures(closures)
        rc = self.lib.orc_advance(ctypes.byref(sc), ctypes.byref(cl), _i3(lo), _i3(hi), _d3(dxinv),
                                  _i3(bc_lo), _i3(bc_hi), int(order_rk), int(stages_rk), float(dt),
                                  _ptr(S1), _ptr(S2), int(nthreads))
        if rc:
            raise RuntimeError("orc_advance failed: %d" % rc)
        return S2


_cache = {}


def oracle():
    """The restatement (always available; built on first use)."""
    if "orc" not in _cache:
        _cache["orc"] = Oracle(_build.build_oracle())
    return _cache["orc"]


def reference(closures):
    """The reference's own sources compiled here for this closure family
    (constant or Sutherland transport), or None when not built."""
    key = "ref_const" if int(closures.visc_law) == 0 else "ref_suth"
    if key not in _cache:
        p = os.path.join(os.path.dirname(_build.REF_LIB), "libcnsref_%s.so" % key[4:])
        _cache[key] = Oracle(p) if os.path.exists(p) else None
    return _cache[key]
