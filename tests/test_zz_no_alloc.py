"""amrs_rhs_box_noalloc: the fused RHS for callers that cannot call cudaMalloc.

Hosts whose arena or memory pool owns all device memory, or that run on a
fixed device-memory budget, cannot let a library allocate behind their back.
This entry point keeps its scratch in one static device array instead of a
handle.  The test calls it through the C ABI twice in a row (different box
shapes, so the second call runs over what the first left in the shared
array) and checks each result against amrs_rhs_box on the same input, to the
last bit (the same kernels run either way).  It also checks that a box
beyond the 32-cell limit is refused.  The file name puts it last in
collection.
"""
import ctypes

import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _noalloc(L, sc, cl, lo, U, out, dxinv):
    nz, ny, nx = (s - 6 for s in U.shape[1:])
    bx = capi.c_box(lo, (nx, ny, nz))
    csc, ccl = capi.c_scheme(sc), capi.c_closures(cl)
    return L.amrs_rhs_box_noalloc(ctypes.byref(csc), ctypes.byref(ccl), ctypes.byref(bx), capi.d3(dxinv),
                                  capi.array4(U, lo, 3), capi.array4(out, lo, 0), None)


def test_noalloc_matches_handle_path_twice():
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    L = capi.load(build_if_missing=True)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    cl = P.Closures.nondimensional(1.0 / 700.0)
    cases = [(P.random_state((24, 20, 16), seed=41, amp=0.2), (3, -2, 5), (2.1, 1.7, 3.3)),
             (P.tgv(32, mach=0.2)[0], (0, 0, 0), (32 / (2 * np.pi),) * 3)]
    h = capi.Handle(sc, cl)
    for U_host, lo, dxinv in cases:
        U = torch.from_numpy(U_host).cuda()
        n = tuple(s - 6 for s in U.shape[1:])
        ref = torch.full((5,) + n, float("nan"), dtype=torch.float64, device="cuda")
        got = torch.full((5,) + n, float("nan"), dtype=torch.float64, device="cuda")
        h.rhs_box(U, dxinv, ref, lo)
        capi.check(_noalloc(L, sc, cl, lo, U, got, dxinv), "amrs_rhs_box_noalloc")
        torch.cuda.synchronize()
        h.sync_check()
        assert torch.equal(got, ref)
    # beyond the size limit: refused with a clear status, nothing launched
    U = torch.zeros((5, 39, 38, 38), dtype=torch.float64, device="cuda")
    out = torch.zeros((5, 33, 32, 32), dtype=torch.float64, device="cuda")
    st = _noalloc(L, sc, cl, (0, 0, 0), U, out, (1.0, 1.0, 1.0))
    assert st == 9  # AMRS_ERR_SIZE
    assert L.amrs_status_string(st).decode() == "size beyond limit"
