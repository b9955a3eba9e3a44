"""Plotfiles from the device: the derived quantities of
amrs_plot_derive_box equal the oracle's restatement of the reference's
derive functions bit for bit, and a level written and read back holds its
state exactly."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import plotfile as PF
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu
G = P.NGHOST


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


@pytest.mark.parametrize("closures", ["nondim", "air"])
def test_plot_derive_bitexact(orc, closures):
    cl = P.Closures.nondimensional(1.0 / 500.0) if closures == "nondim" else P.Closures.air_sutherland()
    U = P.random_state((13, 9, 7), seed=3, amp=0.3)
    if closures == "air":
        U = U.copy()
        U[4] *= 2.5e5  # a dimensional energy scale
    lo = (-3, 2, 5)
    out = torch.empty((5, 7, 9, 13), dtype=torch.float64, device="cuda")
    capi.plot_derive(cl, torch.from_numpy(U).cuda(), lo, out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), orc.plot_derive(cl, U, lo=lo))


def test_level_plotfile_round_trip(orc, tmp_path):
    U, dx = P.tgv(20, mach=0.2)
    cl = P.Closures.nondimensional(1.0 / 800.0)
    lev = cns.CNSLevel(P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1), cl, U, dx)
    for _ in range(2):
        lev.advance(lev.time, 2e-3)
    path = lev.write_plotfile(str(tmp_path / "plt00002"), step=2, derive=("temperature", "pressure", "x_velocity"))
    lev.h.sync_check()
    rd = PF.read_plotfile(path)
    # derived names in the order the reference registers them, not as asked
    assert rd["names"] == list(PF.STATE_NAMES) + ["pressure", "temperature", "x_velocity"]
    assert rd["time"] == lev.time and rd["step"] == 2
    S = lev.state_host()
    np.testing.assert_array_equal(rd["data"][0][:5], S[:, G:-G, G:-G, G:-G])
    np.testing.assert_array_equal(rd["data"][0][5:], orc.plot_derive(cl, S)[[0, 1, 2]])


def test_multibox_plotfile(orc, tmp_path):
    specs, fields, dx = P.batched_boxes(nboxes=5, seed=8, edges=(8, 16))
    cl = P.Closures.nondimensional(1.0 / 800.0)
    states = [torch.from_numpy(F).cuda() for F in fields]
    boxes = [(s.lo, s.shape) for s in specs]
    hi = [max(lo[d] + n[d] for lo, n in boxes) for d in range(3)]
    path = PF.write_plotfile(str(tmp_path / "plt_boxes"), boxes, states, cl, dx, (0.0, 0.0, 0.0),
                             ((0, 0, 0), tuple(hi)), time=0.5, step=7)
    rd = PF.read_plotfile(path)
    assert len(rd["data"]) == 5
    for (lo, n), F, a in zip(boxes, fields, rd["data"]):
        np.testing.assert_array_equal(a[:5], F[:, G:-G, G:-G, G:-G])
        np.testing.assert_array_equal(a[5:], orc.plot_derive(cl, F, lo=lo))
