"""ctypes binding of the C ABI in include/amrs_gb300.h.

Device memory comes from torch (cuda float64 tensors in the Array4 layout
(ncomp, nz+2g, ny+2g, nx+2g)); only raw pointers, strides and sizes cross
the boundary.  Every call raises AmrsError on a non-zero status.  There is
no CPU fallback: without the compiled library or a GPU, calls fail.
"""
from __future__ import annotations

import ctypes
import weakref
import os

from . import build as _build
from .problems import NCONS, NGHOST

_lib = None


class AmrsError(RuntimeError):
    pass


# Order of the 21 values of amrs_boxlist_prim_stats / amrs_prim_stats_box.
PRIM_STATS_KEYS = (["min_" + q for q in ("rho", "u", "v", "w", "T", "p")]
                   + ["max_" + q for q in ("rho", "u", "v", "w", "T", "p")]
                   + ["%s_%s" % (a, d) for d in "xyz" for a in ("max_u_plus_c", "max_u_minus_c", "cfl")])


class Array4(ctypes.Structure):
    _fields_ = [("p", ctypes.c_void_p), ("jstride", ctypes.c_int64), ("kstride", ctypes.c_int64),
                ("nstride", ctypes.c_int64), ("begin", ctypes.c_int32 * 3), ("end", ctypes.c_int32 * 3),
                ("ncomp", ctypes.c_int32)]


class CClosures(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("cv", ctypes.c_double), ("cp", ctypes.c_double),
                ("Rspec", ctypes.c_double), ("visc_law", ctypes.c_int32), ("cond_law", ctypes.c_int32),
                ("visc_ref", ctypes.c_double), ("Tvisc_ref", ctypes.c_double), ("cond_ref", ctypes.c_double),
                ("Tcond_ref", ctypes.c_double), ("Cshock", ctypes.c_double), ("Cdamp", ctypes.c_double)]


class CScheme(ctypes.Structure):
    _fields_ = [("rhs_euler", ctypes.c_int32), ("rhs_visc", ctypes.c_int32), ("flux_euler", ctypes.c_int32),
                ("order_keep", ctypes.c_int32), ("art_diss", ctypes.c_int32), ("weno_fast", ctypes.c_int32),
                ("riemann_weno", ctypes.c_int32)]


class CBcNormal(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("Tw", ctypes.c_double), ("Tmin", ctypes.c_double),
                ("prob_lo", ctypes.c_double * 3), ("prob_hi", ctypes.c_double * 3), ("dx", ctypes.c_double * 3)]


def c_bcnormal(bn):
    return CBcNormal(int(bn.kind), float(bn.Tw), float(bn.Tmin), d3(bn.prob_lo), d3(bn.prob_hi), d3(bn.dx))


class CBox(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_int32 * 3), ("hi", ctypes.c_int32 * 3)]


class RkOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("dst", ctypes.c_int32), ("x", ctypes.c_int32), ("y", ctypes.c_int32),
                ("a", ctypes.c_double), ("b", ctypes.c_double)]


class StageProg(ctypes.Structure):
    _fields_ = [("src_state", ctypes.c_int32), ("nops", ctypes.c_int32), ("ops", RkOp * 3)]


# name -> (restype, argtypes); every symbol declared in include/amrs_gb300.h
_P = ctypes.c_void_p
_S = ctypes.c_int
SIGNATURES = {
    "amrs_create": (_S, [ctypes.POINTER(_P), ctypes.POINTER(CScheme), ctypes.POINTER(CClosures), ctypes.c_int]),
    "amrs_destroy": (_S, [_P]),
    "amrs_set_closures": (_S, [_P, ctypes.POINTER(CClosures)]),
    "amrs_set_domain": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "amrs_status_string": (ctypes.c_char_p, [_S]),
    "amrs_last_cuda_error": (ctypes.c_char_p, []),
    "amrs_version": (ctypes.c_int32, []),
    "amrs_cuda_arch": (ctypes.c_int32, []),
    "amrs_rk_program": (_S, [ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.POINTER(StageProg),
                             ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    "amrs_rhs_box": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double), Array4, Array4, _P]),
    "amrs_rhs_box_noalloc": (_S, [ctypes.POINTER(CScheme), ctypes.POINTER(CClosures), ctypes.POINTER(CBox),
                                  ctypes.POINTER(ctypes.c_double), Array4, Array4, _P]),
    "amrs_rk_stage_box": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(StageProg),
                               ctypes.c_double, Array4, Array4, Array4, _P]),
    "amrs_fill_halo_box": (_S, [ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                Array4, _P]),
    "amrs_est_timestep_box": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double), ctypes.c_double, Array4,
                                   _P, _P]),
    "amrs_boxlist_create": (_S, [_P, ctypes.c_int32, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double),
                                 ctypes.c_int32, ctypes.POINTER(Array4), ctypes.POINTER(ctypes.c_int32),
                                 ctypes.c_int32, ctypes.POINTER(CClosures), ctypes.POINTER(_P)]),
    "amrs_boxlist_destroy": (_S, [_P]),
    "amrs_boxlist_set_tile": (_S, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                   ctypes.c_int32, ctypes.c_int32]),
    "amrs_boxlist_set_tiles": (_S, [_P, ctypes.POINTER(ctypes.c_int32)]),
    "amrs_boxlist_set_bc": (_S, [_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "amrs_boxlist_set_domain": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_int32),
                                     ctypes.POINTER(ctypes.c_int32)]),
    "amrs_boxlist_fill_halo": (_S, [_P, ctypes.c_int32, _P]),
    "amrs_rk_stage_boxlist": (_S, [_P, ctypes.POINTER(StageProg), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                   _P]),
    "amrs_rk_step_boxlist": (_S, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P,
                                  ctypes.POINTER(ctypes.c_int32)]),
    "amrs_rk_run_boxlist": (_S, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                 ctypes.c_int32, _P]),
    "amrs_boxlist_run_state": (_S, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_int32), _P]),
    "amrs_boxlist_totals": (_S, [_P, ctypes.c_int32, ctypes.c_double, _P, _P]),
    "amrs_boxlist_set_schedule": (_S, [_P, ctypes.c_int32]),
    "amrs_boxlist_face_grid": (ctypes.c_int32, [_P]),
    "amrs_boxlist_get_tiles": (_S, [_P, _P]),
    "amrs_plot_derive_box": (_S, [ctypes.POINTER(CClosures), ctypes.POINTER(CBox), Array4, Array4, _P]),
    "amrs_boxlist_prim_stats": (_S, [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.c_double, _P, _P]),
    "amrs_prim_stats_box": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double), Array4, ctypes.c_double,
                                 _P, _P]),
    "amrs_rhs_vjp_box": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double), Array4, Array4, Array4,
                              _P, _P]),
    "amrs_fill_halo_box_adjoint": (_S, [ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int32), Array4, _P]),
    "amrs_rk_stage_vjp_box": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(StageProg), ctypes.POINTER(ctypes.c_int32),
                                   ctypes.POINTER(ctypes.c_int32), Array4, Array4, Array4, Array4, _P, _P]),
    "amrs_rk_stage_vjp_box_ghosted": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(StageProg), Array4, Array4, Array4, Array4, _P, _P]),
    "amrs_set_source": (_S, [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]),
    "amrs_fill_halo_box_bcnormal": (_S, [ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(CClosures),
                                         ctypes.POINTER(CBcNormal), Array4, _P]),
    "amrs_boxlist_set_bcnormal": (_S, [_P, ctypes.POINTER(CBcNormal)]),
    "amrs_sync_check": (_S, [_P, _P]),
    "amrs_probe_fp64_tflops": (_S, [_P, ctypes.POINTER(ctypes.c_double)]),
    "amrs_set_check_nonfinite": (_S, [_P, ctypes.c_int32]),
    "amrs_debug_ddiv_check": (_S, [_P, ctypes.c_uint64, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64),
                                   ctypes.POINTER(ctypes.c_double)]),
    "amrs_debug_dsqrt_check": (_S, [_P, ctypes.c_uint64, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64),
                                    ctypes.POINTER(ctypes.c_double)]),
    "amrs_debug_dmul_check": (_S, [_P, ctypes.c_uint64, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64),
                                   ctypes.POINTER(ctypes.c_double)]),
    "amrs_probe_intpipe": (_S, [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]),
    "amrs_probe_fp64_tflops_timed": (_S, [_P, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
    "amrs_debug_wait_timeout": (_S, [_P, ctypes.c_int32, _P]),
    "amrs_average_down": (_S, [ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_int32), Array4, Array4, ctypes.c_int32,
                               ctypes.c_int32, _P]),
    "amrs_profile_stage_box": (_S, [_P, ctypes.POINTER(CBox), ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(StageProg), Array4, Array4, Array4, ctypes.c_int32, _P,
                                    ctypes.POINTER(ctypes.c_double)]),
    "amrs_debug_tma_enabled": (ctypes.c_int32, [_P]),
    "amrs_boxlist_tma_enabled": (ctypes.c_int32, [_P]),
}


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load the compiled library (never a fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not os.path.exists(p):
        if not build_if_missing:
            raise AmrsError("libamrs_gb300.so not built: run amrsolver_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(p)
    for name, (rt, at) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = rt
        f.argtypes = at
    _lib = L
    return L


def check(status, what=""):
    if status != 0:
        L = load()
        msg = L.amrs_status_string(status).decode()
        cuda = L.amrs_last_cuda_error().decode()
        raise AmrsError("%s failed: %s (%d)%s" % (what, msg, status, (" [" + cuda + "]") if cuda else ""))


def c_closures(cl):
    return CClosures(cl.gamma, cl.cv, cl.cp, cl.Rspec, int(cl.visc_law), int(cl.cond_law), cl.visc_ref,
                     cl.Tvisc_ref, cl.cond_ref, cl.Tcond_ref, cl.Cshock, cl.Cdamp)


def c_scheme(sc):
    return CScheme(int(sc.rhs_euler), int(sc.rhs_visc), int(sc.flux_euler), int(sc.order_keep), int(sc.art_diss),
                   int(getattr(sc, "weno_fast", 0)), int(getattr(sc, "riemann_weno", 0)))


def c_box(lo, n):
    return CBox((ctypes.c_int32 * 3)(*lo), (ctypes.c_int32 * 3)(*[lo[d] + n[d] - 1 for d in range(3)]))


def d3(v):
    return (ctypes.c_double * 3)(*[float(x) for x in v])


def i3(v):
    return (ctypes.c_int32 * 3)(*[int(x) for x in v])


def array4(t, lo, g):
    """Array4 of a contiguous cuda float64 tensor (ncomp, nz+2g, ny+2g, nx+2g)
    whose valid box starts at `lo`."""
    if not t.is_cuda or t.dtype.itemsize != 8 or not t.is_contiguous():
        raise AmrsError("expected a contiguous cuda float64 tensor")
    nc, nz, ny, nx = t.shape
    b = [lo[0] - g, lo[1] - g, lo[2] - g]
    return Array4(t.data_ptr(), nx, nx * ny, nx * ny * nz, (ctypes.c_int32 * 3)(*b),
                  (ctypes.c_int32 * 3)(b[0] + nx, b[1] + ny, b[2] + nz), nc)


def rk_program(order_rk, stages_rk, dt):
    L = load()
    progs = (StageProg * 16)()
    n = ctypes.c_int32()
    check(L.amrs_rk_program(order_rk, stages_rk, dt, progs, 16, ctypes.byref(n)), "amrs_rk_program")
    return [progs[i] for i in range(n.value)]


def _stream_ptr(stream):
    return ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)


class Handle:
    """amrs_handle: scheme + closures bound to one CUDA device."""

    def __init__(self, scheme, closures, device=0):
        L = load()
        self._L = L
        self.scheme = scheme
        self.closures = closures
        h = ctypes.c_void_p()
        sc, cl = c_scheme(scheme), c_closures(closures)
        check(L.amrs_create(ctypes.byref(h), ctypes.byref(sc), ctypes.byref(cl), int(device)), "amrs_create")
        self.h = h
        # box lists created on this handle: closed before it (a list must not
        # outlive its handle, whatever order a garbage collection finds them in)
        self._lists = weakref.WeakSet()
        if int(getattr(scheme, "rhs_source", 0)):
            self.set_source(getattr(scheme, "body_force", (0.0, 0.0, 0.0)))

    def set_source(self, force, on=True):
        """amrs_set_source: cns.rhs_source with a body force per unit mass."""
        check(self._L.amrs_set_source(self.h, 1 if on else 0, d3(force)), "amrs_set_source")

    def close(self):
        if self.h:
            for bl in list(self._lists):
                bl.close()
            self._L.amrs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_domain(self, dom_lo, dom_n, bc_lo, bc_hi):
        """amrs_set_domain: domain box (lo, extents x,y,z) and boundary codes of
        the per-box calls; code 6 on a y side is a wall.  None clears."""
        if dom_lo is None:
            check(self._L.amrs_set_domain(self.h, None, None, None), "amrs_set_domain")
            return
        dom = c_box(dom_lo, dom_n)
        check(self._L.amrs_set_domain(self.h, ctypes.byref(dom), i3(bc_lo), i3(bc_hi)), "amrs_set_domain")

    def rhs_box(self, U, dxinv, out, lo=(0, 0, 0), stream=None):
        """dSdt of one ghost-filled box into `out` (ncomp, nz, ny, nx)."""
        nz, ny, nx = (s - 2 * NGHOST for s in U.shape[1:])
        bx = c_box(lo, (nx, ny, nz))
        check(self._L.amrs_rhs_box(self.h, ctypes.byref(bx), d3(dxinv), array4(U, lo, NGHOST), array4(out, lo, 0),
                                   _stream_ptr(stream)), "amrs_rhs_box")
        return out

    def rk_stage_box(self, prog, Uin, U1, Uout, dxinv, lo=(0, 0, 0), stream=None):
        nz, ny, nx = (s - 2 * NGHOST for s in Uin.shape[1:])
        g1 = (U1.shape[1] - nz) // 2
        go = (Uout.shape[1] - nz) // 2
        bx = c_box(lo, (nx, ny, nz))
        check(self._L.amrs_rk_stage_box(self.h, ctypes.byref(bx), d3(dxinv), ctypes.byref(prog), 0.0,
                                        array4(Uin, lo, NGHOST), array4(U1, lo, g1), array4(Uout, lo, go),
                                        _stream_ptr(stream)), "amrs_rk_stage_box")

    def est_timestep(self, U, dx, cfl, dt_dev, lo=(0, 0, 0), stream=None):
        nz, ny, nx = (s - 2 * NGHOST for s in U.shape[1:])
        bx = c_box(lo, (nx, ny, nz))
        check(self._L.amrs_est_timestep_box(self.h, ctypes.byref(bx), d3(dx), float(cfl), array4(U, lo, NGHOST),
                                            ctypes.c_void_p(dt_dev.data_ptr()), _stream_ptr(stream)),
              "amrs_est_timestep_box")

    def prim_stats(self, U, dx, dt, out, lo=(0, 0, 0), ng=NGHOST, stream=None):
        """CNS::printTotal's primitive extrema and CFL table of one box into
        the cuda tensor `out` (21 doubles; see PRIM_STATS_KEYS)."""
        nz, ny, nx = (s - 2 * ng for s in U.shape[1:])
        bx = c_box(lo, (nx, ny, nz))
        check(self._L.amrs_prim_stats_box(self.h, ctypes.byref(bx), d3(dx), array4(U, lo, ng), float(dt),
                                          ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream)),
              "amrs_prim_stats_box")
        return out

    def sync_check(self, stream=None):
        check(self._L.amrs_sync_check(self.h, _stream_ptr(stream)), "amrs_sync_check")

    def tma_enabled(self):
        return int(self._L.amrs_debug_tma_enabled(self.h))

    def rhs_vjp_box(self, U, vbar, ubar, dxinv, lo=(0, 0, 0), param_bar=None, stream=None):
        """ubar (ghosted) = (d dSdt/dU)^T vbar; param_bar (cuda, 2 doubles) += d/d(visc_ref, cond_ref)."""
        nz, ny, nx = (s - 2 * NGHOST for s in U.shape[1:])
        bx = c_box(lo, (nx, ny, nz))
        pb = ctypes.c_void_p(param_bar.data_ptr()) if param_bar is not None else None
        check(self._L.amrs_rhs_vjp_box(self.h, ctypes.byref(bx), d3(dxinv), array4(U, lo, NGHOST),
                                       array4(vbar, lo, 0), array4(ubar, lo, NGHOST), pb, _stream_ptr(stream)),
              "amrs_rhs_vjp_box")

    def rk_stage_vjp_box(self, prog, bc_lo, bc_hi, Uin, wbar, s1bar, inbar, dxinv, lo=(0, 0, 0), param_bar=None,
                         stream=None):
        """Adds the S1 and stage-input cotangents of one RK stage (valid cells)."""
        nz, ny, nx = (s - 2 * NGHOST for s in Uin.shape[1:])
        bx = c_box(lo, (nx, ny, nz))
        g = lambda t: (t.shape[1] - nz) // 2
        pb = ctypes.c_void_p(param_bar.data_ptr()) if param_bar is not None else None
        check(self._L.amrs_rk_stage_vjp_box(self.h, ctypes.byref(bx), d3(dxinv), ctypes.byref(prog), i3(bc_lo),
                                            i3(bc_hi), array4(Uin, lo, NGHOST), array4(wbar, lo, g(wbar)),
                                            array4(s1bar, lo, g(s1bar)), array4(inbar, lo, g(inbar)), pb,
                                            _stream_ptr(stream)), "amrs_rk_stage_vjp_box")

    def rk_stage_vjp_box_ghosted(self, prog, Uin, wbar, s1bar, ubar, dxinv, lo=(0, 0, 0), param_bar=None,
                                 stream=None):
        """Stage VJP without the ghost fold: ubar (ghosted) is overwritten with
        the cotangent of the ghost-filled stage input, s1bar gets the S1
        cotangent added (domains with ext_dir sides; the caller folds)."""
        nz, ny, nx = (s - 2 * NGHOST for s in Uin.shape[1:])
        bx = c_box(lo, (nx, ny, nz))
        g = lambda t: (t.shape[1] - nz) // 2
        pb = ctypes.c_void_p(param_bar.data_ptr()) if param_bar is not None else None
        check(self._L.amrs_rk_stage_vjp_box_ghosted(self.h, ctypes.byref(bx), d3(dxinv), ctypes.byref(prog),
                                                    array4(Uin, lo, NGHOST), array4(wbar, lo, g(wbar)),
                                                    array4(s1bar, lo, g(s1bar)), array4(ubar, lo, NGHOST), pb,
                                                    _stream_ptr(stream)), "amrs_rk_stage_vjp_box_ghosted")

    def profile_stage_box(self, prog, Uin, U1, Uout, dxinv, lo=(0, 0, 0), reps=5, stream=None):
        """Per-kernel ms of one stage: (prims [+ WENO point fluxes], viscous
        cells, Euler face kernel [fused: + divergence + program; MUSCL:
        slopes + Riemann faces], total)."""
        nz, ny, nx = (s - 2 * NGHOST for s in Uin.shape[1:])
        g1 = (U1.shape[1] - nz) // 2
        go = (Uout.shape[1] - nz) // 2
        bx = c_box(lo, (nx, ny, nz))
        ms = (ctypes.c_double * 4)()
        check(self._L.amrs_profile_stage_box(self.h, ctypes.byref(bx), d3(dxinv), ctypes.byref(prog),
                                             array4(Uin, lo, NGHOST), array4(U1, lo, g1), array4(Uout, lo, go),
                                             int(reps), _stream_ptr(stream), ms), "amrs_profile_stage_box")
        return tuple(ms)

    def ddiv_check(self, seed, count, sqrt=False, mul=False):
        """(mismatches, first mismatch (a, b, hardware, library)) of the
        integer-pipe division (or square root, or product) against the
        hardware one on the device."""
        nb = ctypes.c_int64()
        first = (ctypes.c_double * 4)()
        fn = (self._L.amrs_debug_dmul_check if mul else
              self._L.amrs_debug_dsqrt_check if sqrt else self._L.amrs_debug_ddiv_check)
        check(fn(self.h, int(seed), int(count), ctypes.byref(nb), first), "amrs_debug_ddiv_check")
        return nb.value, tuple(first)

    def probe_intpipe(self, mode):
        """ms of the overlap probe (amrs_probe_intpipe): 16 FMA chains per
        thread plus four chains of no (0), hardware (1) or integer-pipe (2)
        products."""
        ms = ctypes.c_double()
        check(self._L.amrs_probe_intpipe(self.h, int(mode), ctypes.byref(ms)), "amrs_probe_intpipe")
        return ms.value

    def set_check_nonfinite(self, on=True):
        """Opt in (or out) of the non-finite check after every stage and RHS;
        sync_check then raises AmrsError with AMRS_ERR_NONFINITE."""
        check(self._L.amrs_set_check_nonfinite(self.h, int(bool(on))), "amrs_set_check_nonfinite")

    def probe_fp64_tflops(self, seconds=None):
        """Measured FP64 FMA rate (TFLOP/s).  With `seconds`, the timed launch
        runs about that long and (tflops, launch ms) is returned."""
        v = ctypes.c_double()
        if seconds is None:
            check(self._L.amrs_probe_fp64_tflops(self.h, ctypes.byref(v)), "amrs_probe_fp64_tflops")
            return v.value
        ms = ctypes.c_double()
        check(self._L.amrs_probe_fp64_tflops_timed(self.h, float(seconds), ctypes.byref(v), ctypes.byref(ms)),
              "amrs_probe_fp64_tflops_timed")
        return v.value, ms.value

    def debug_wait_timeout(self, polls=4096, stream=None):
        """Run the bounded-wait failure path once (amrs_debug_wait_timeout);
        the next sync_check raises AmrsError (AMRS_ERR_TIMEOUT)."""
        check(self._L.amrs_debug_wait_timeout(self.h, int(polls), _stream_ptr(stream)), "amrs_debug_wait_timeout")


def fill_halo_box(U, bc_lo, bc_hi, lo=(0, 0, 0), stream=None):
    L = load()
    nz, ny, nx = (s - 2 * NGHOST for s in U.shape[1:])
    bx = c_box(lo, (nx, ny, nz))
    check(L.amrs_fill_halo_box(ctypes.byref(bx), i3(bc_lo), i3(bc_hi), array4(U, lo, NGHOST), _stream_ptr(stream)),
          "amrs_fill_halo_box")


def fill_halo_box_bcnormal(U, bc_lo, bc_hi, closures, bn, lo=(0, 0, 0), stream=None):
    """fill_halo_box, then the device bcnormal `bn` (problems.BCNormal)
    beyond code-6 y sides (amrs_fill_halo_box_bcnormal)."""
    L = load()
    nz, ny, nx = (s - 2 * NGHOST for s in U.shape[1:])
    bx = c_box(lo, (nx, ny, nz))
    check(L.amrs_fill_halo_box_bcnormal(ctypes.byref(bx), i3(bc_lo), i3(bc_hi), ctypes.byref(c_closures(closures)),
                                        ctypes.byref(c_bcnormal(bn)), array4(U, lo, NGHOST), _stream_ptr(stream)),
          "amrs_fill_halo_box_bcnormal")


def fill_halo_box_adjoint(ubar, bc_lo, bc_hi, lo=(0, 0, 0), stream=None):
    """Adjoint of fill_halo_box, in place on the ghosted cotangent `ubar`:
    valid cells receive the cotangents of the ghosts filled from them
    (ghosts beyond ext_dir sides, codes 1 and 6, are left in place)."""
    L = load()
    nz, ny, nx = (s - 2 * NGHOST for s in ubar.shape[1:])
    bx = c_box(lo, (nx, ny, nz))
    check(L.amrs_fill_halo_box_adjoint(ctypes.byref(bx), i3(bc_lo), i3(bc_hi), array4(ubar, lo, NGHOST),
                                       _stream_ptr(stream)), "amrs_fill_halo_box_adjoint")


def average_down(fine, crse, crse_lo, ratio, fine_g=0, crse_g=0, scomp=0, ncomp=None, stream=None):
    """amrs_average_down: the valid cells of `crse` (box at `crse_lo`, `crse_g`
    ghost layers in the tensor) become the means of their fine cells in
    `fine` (valid box at crse_lo * ratio, `fine_g` ghost layers)."""
    L = load()
    nz, ny, nx = (s - 2 * crse_g for s in crse.shape[1:])
    bx = c_box(crse_lo, (nx, ny, nz))
    flo = tuple(int(a) * int(r) for a, r in zip(crse_lo, ratio))
    nc = crse.shape[0] - scomp if ncomp is None else ncomp
    check(L.amrs_average_down(ctypes.byref(bx), i3(ratio), array4(fine, flo, fine_g), array4(crse, crse_lo, crse_g),
                              int(scomp), int(nc), _stream_ptr(stream)), "amrs_average_down")


class BoxList:
    """amrs_boxlist: many boxes, `nslots` caller-owned ghosted states each."""

    def __init__(self, handle, los, slots, dxinv, closure_index=None, closures=None):
        L = load()
        self._L = L
        self.handle = handle
        self.bl = None
        n = len(los)
        self.n = n
        self.nslots = len(slots[0])
        self.slots = slots  # keep tensors alive
        boxes = (CBox * n)()
        arr = (Array4 * (n * self.nslots))()
        dx = (ctypes.c_double * (3 * n))()
        for b in range(n):
            U = slots[b][0]
            nz, ny, nx = (s - 2 * NGHOST for s in U.shape[1:])
            boxes[b] = c_box(los[b], (nx, ny, nz))
            for s in range(self.nslots):
                arr[b * self.nslots + s] = array4(slots[b][s], los[b], NGHOST)
            dv = dxinv[b] if hasattr(dxinv[0], "__len__") else dxinv
            for d in range(3):
                dx[3 * b + d] = float(dv[d])
        ci = None
        cls = None
        ncl = 0
        if closure_index is not None:
            ci = (ctypes.c_int32 * n)(*closure_index)
            ncl = len(closures)
            cls = (CClosures * ncl)(*[c_closures(c) for c in closures])
        bl = ctypes.c_void_p()
        check(L.amrs_boxlist_create(handle.h, n, boxes, dx, self.nslots, arr, ci, ncl, cls, ctypes.byref(bl)),
              "amrs_boxlist_create")
        self.bl = bl
        handle._lists.add(self)

    def close(self):
        if self.bl:
            self._L.amrs_boxlist_destroy(self.bl)
            self.bl = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tile(self, n, tx, ty, kc):
        check(self._L.amrs_boxlist_set_tile(self.bl, n[0], n[1], n[2], tx, ty, kc), "amrs_boxlist_set_tile")

    def set_tiles(self, tiles):
        """tiles: per box (tx, ty, kchunk)."""
        flat = (ctypes.c_int32 * (3 * self.n))(*[int(v) for t in tiles for v in t])
        check(self._L.amrs_boxlist_set_tiles(self.bl, flat), "amrs_boxlist_set_tiles")

    def set_schedule(self, waves):
        """Shares of the face-kernel schedule per resident CTA (1..8)."""
        check(self._L.amrs_boxlist_set_schedule(self.bl, int(waves)), "amrs_boxlist_set_schedule")

    def face_grid(self):
        return int(self._L.amrs_boxlist_face_grid(self.bl))

    def get_tiles(self):
        """Current per-box (tx, ty, kchunk)."""
        flat = (ctypes.c_int32 * (3 * self.n))()
        check(self._L.amrs_boxlist_get_tiles(self.bl, flat), "amrs_boxlist_get_tiles")
        return [tuple(flat[3 * b:3 * b + 3]) for b in range(self.n)]

    def set_bc(self, bc_lo, bc_hi):
        if bc_lo is None:
            check(self._L.amrs_boxlist_set_bc(self.bl, None, None), "amrs_boxlist_set_bc")
        else:
            check(self._L.amrs_boxlist_set_bc(self.bl, i3(bc_lo), i3(bc_hi)), "amrs_boxlist_set_bc")

    def set_domain(self, dom_lo, dom_n, bc_lo, bc_hi):
        """The boxes tile the domain box starting at `dom_lo` with extents
        `dom_n` (x, y, z): single-level ghost fill across the level."""
        dom = c_box(dom_lo, dom_n)
        check(self._L.amrs_boxlist_set_domain(self.bl, ctypes.byref(dom), i3(bc_lo), i3(bc_hi)),
              "amrs_boxlist_set_domain")

    def set_bcnormal(self, bn):
        """Device bcnormal (problems.BCNormal, None: none) beyond the domain's
        code-6 y sides in every later fill (amrs_boxlist_set_bcnormal)."""
        check(self._L.amrs_boxlist_set_bcnormal(self.bl, ctypes.byref(c_bcnormal(bn)) if bn is not None else None),
              "amrs_boxlist_set_bcnormal")

    def fill_halo(self, slot, stream=None):
        check(self._L.amrs_boxlist_fill_halo(self.bl, slot, _stream_ptr(stream)), "amrs_boxlist_fill_halo")

    def stage(self, prog, s_in, s1, s_out, stream=None):
        check(self._L.amrs_rk_stage_boxlist(self.bl, ctypes.byref(prog), s_in, s1, s_out, _stream_ptr(stream)),
              "amrs_rk_stage_boxlist")

    def step(self, order_rk, stages_rk, dt, s1=0, w1=1, w2=2, use_graph=True, stream=None):
        res = ctypes.c_int32()
        check(self._L.amrs_rk_step_boxlist(self.bl, order_rk, stages_rk, float(dt), s1, w1, w2, int(use_graph),
                                           _stream_ptr(stream), ctypes.byref(res)), "amrs_rk_step_boxlist")
        return res.value

    def tma_enabled(self):
        return int(self._L.amrs_boxlist_tma_enabled(self.bl))

    def run(self, order_rk, stages_rk, stop_time, max_steps, cfl=0.0, dt=0.0, time=0.0, s1=0, w1=1, w2=2,
            stream=None):
        """amrs_rk_run_boxlist: the whole time loop as one device launch
        (CFL-controlled dt when cfl > 0, else fixed dt); state in slot s1."""
        check(self._L.amrs_rk_run_boxlist(self.bl, order_rk, stages_rk, float(cfl), float(dt), float(time),
                                          float(stop_time), int(max_steps), s1, w1, w2, _stream_ptr(stream)),
              "amrs_rk_run_boxlist")

    def run_state(self, stream=None):
        """(time, dt, steps) of the last run (host-synchronising)."""
        t, d, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
        check(self._L.amrs_boxlist_run_state(self.bl, ctypes.byref(t), ctypes.byref(d), ctypes.byref(n),
                                             _stream_ptr(stream)), "amrs_boxlist_run_state")
        return t.value, d.value, n.value

    def prim_stats(self, slot, dx, dt, out, stream=None):
        """Primitive extrema and CFL table over every box (slot -1: the
        primitives of the last RHS's stage input) into `out` (21 doubles)."""
        check(self._L.amrs_boxlist_prim_stats(self.bl, int(slot), d3(dx), float(dt), ctypes.c_void_p(out.data_ptr()),
                                              _stream_ptr(stream)), "amrs_boxlist_prim_stats")
        return out

    def totals(self, slot, scale, out, stream=None):
        """Conserved totals of `slot` times `scale` into the cuda tensor `out` (5 doubles)."""
        check(self._L.amrs_boxlist_totals(self.bl, slot, float(scale), ctypes.c_void_p(out.data_ptr()),
                                          _stream_ptr(stream)), "amrs_boxlist_totals")
        return out


def plot_derive(closures, U, lo, out, ng=NGHOST, stream=None):
    """Derived plot variables (pressure, temperature, x/y/z velocity) of the
    valid cells of one box's state `U` (ghost depth `ng`) into the cuda tensor
    `out` (5, nz, ny, nx): amrs_plot_derive_box."""
    nz, ny, nx = (s - 2 * ng for s in U.shape[1:])
    bx = c_box(lo, (nx, ny, nz))
    cl = c_closures(closures)
    check(load().amrs_plot_derive_box(ctypes.byref(cl), ctypes.byref(bx), array4(U, lo, ng), array4(out, lo, 0),
                                      _stream_ptr(stream)), "amrs_plot_derive_box")
    return out
