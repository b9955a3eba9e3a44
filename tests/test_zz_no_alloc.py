"""amrs_rhs_box_noalloc: the fused RHS for callers that cannot call cudaMalloc.

Hosts whose arena or memory pool owns all device memory, or that run on a
fixed device-memory budget, cannot let a library allocate behind their back.
This entry point keeps its scratch in one static device array instead of a
handle.  Each case calls it through the C ABI twice in a row on different box
shapes (the second call runs over what the first left in the shared array)
and checks every result against amrs_rhs_box on the same input, to the last
bit (the same kernels run either way).  Cases cover KEEP orders 2, 4 and 6
with and without viscous terms, and boxes that take each tile branch (edges
of 8, 16 and up to 32 cells in x).  Boxes beyond the 32-cell limit and
unsupported switches are refused before anything is launched.  The file name
puts it last in collection.
"""
import ctypes

import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _noalloc(L, sc, cl, lo, U, out, dxinv, csc=None, ccl=None):
    nz, ny, nx = (s - 6 for s in U.shape[1:])
    bx = capi.c_box(lo, (nx, ny, nz))
    csc = csc if csc is not None else capi.c_scheme(sc)
    ccl = ccl if ccl is not None else capi.c_closures(cl)
    return L.amrs_rhs_box_noalloc(ctypes.byref(csc), ctypes.byref(ccl), ctypes.byref(bx), capi.d3(dxinv),
                                  capi.array4(U, lo, 3), capi.array4(out, lo, 0), None)


def _cases():
    return [(P.random_state((24, 20, 16), seed=41, amp=0.2), (3, -2, 5), (2.1, 1.7, 3.3)),
            (P.tgv(32, mach=0.2)[0], (0, 0, 0), (32 / (2 * np.pi),) * 3),
            (P.random_state((8, 8, 8), seed=7, amp=0.3), (-4, 0, 2), (1.3, 0.9, 2.2)),
            (P.random_state((16, 12, 10), seed=8, amp=0.25), (1, 2, 3), (0.7, 1.1, 1.9))]


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("visc", [0, 1])
def test_noalloc_matches_handle_path_twice(order, visc):
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    L = capi.load(build_if_missing=True)
    sc = P.Scheme(flux_euler=1, order_keep=order, rhs_visc=visc)
    cl = P.Closures.nondimensional(1.0 / 700.0)
    h = capi.Handle(sc, cl)
    cases = _cases()
    # two calls in a row on every pair of neighbouring shapes
    for U_host, lo, dxinv in cases + cases[:1]:
        U = torch.from_numpy(U_host).cuda()
        n = tuple(s - 6 for s in U.shape[1:])
        ref = torch.full((5,) + n, float("nan"), dtype=torch.float64, device="cuda")
        got = torch.full((5,) + n, float("nan"), dtype=torch.float64, device="cuda")
        h.rhs_box(U, dxinv, ref, lo)
        capi.check(_noalloc(L, sc, cl, lo, U, got, dxinv), "amrs_rhs_box_noalloc")
        torch.cuda.synchronize()
        h.sync_check()
        assert torch.equal(got, ref), (order, visc, n)
    h.close()


def test_noalloc_refusals():
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    L = capi.load(build_if_missing=True)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    cl = P.Closures.nondimensional(1.0 / 700.0)
    # beyond the size limit: refused with a clear status, nothing launched
    U = torch.zeros((5, 39, 38, 38), dtype=torch.float64, device="cuda")
    out = torch.zeros((5, 33, 32, 32), dtype=torch.float64, device="cuda")
    st = _noalloc(L, sc, cl, (0, 0, 0), U, out, (1.0, 1.0, 1.0))
    assert st == 9  # AMRS_ERR_SIZE
    assert L.amrs_status_string(st).decode() == "size beyond limit"
    # switches this path does not run, and an unknown transport law
    U = torch.zeros((5, 14, 14, 14), dtype=torch.float64, device="cuda")
    out = torch.zeros((5, 8, 8, 8), dtype=torch.float64, device="cuda")
    for bad in (dict(flux_euler=2), dict(art_diss=1), dict(order_keep=3), dict(rhs_visc=2)):
        kw = dict(flux_euler=1, order_keep=4, rhs_visc=1)
        kw.update(bad)
        assert _noalloc(L, None, cl, (0, 0, 0), U, out, (1.0, 1.0, 1.0),
                        csc=capi.c_scheme(P.Scheme(**kw))) == 4, bad  # AMRS_ERR_SCHEME
    ccl = capi.c_closures(cl)
    ccl.visc_law = 7
    assert _noalloc(L, sc, None, (0, 0, 0), U, out, (1.0, 1.0, 1.0), ccl=ccl) == 4
    torch.cuda.synchronize()
    assert bool((out == 0).all())
