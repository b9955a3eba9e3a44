"""The plotfile writer's layout on the host: the Header in the order
CNS::writePlotFile writes it (src/CNS.cpp:689-796), the VisMF header and the
FAB data file of Level_0, and a round trip through read_plotfile.  The plot
data here is the oracle's restatement of the reference's derive functions
(pinned to them in tests/test_oracle_vs_reference.py); the device path is
tests/test_gpu_plotfile.py."""
import os

import numpy as np

from amrsolver_gb300 import plotfile as PF
from amrsolver_gb300 import problems as P

G = P.NGHOST


def _level(orc):
    cl = P.Closures.nondimensional(1.0 / 500.0)
    boxes = [((0, 0, 0), (6, 5, 4)), ((6, 0, 0), (4, 5, 4)), ((0, 5, 0), (10, 3, 4))]
    data = []
    for b, (lo, n) in enumerate(boxes):
        U = P.random_state(n, seed=30 + b, amp=0.2)
        der = orc.plot_derive(cl, U, lo=lo)
        data.append(np.concatenate([U[:, G:-G, G:-G, G:-G], der]))
    return boxes, data


def test_header_and_round_trip(orc, tmp_path):
    boxes, data = _level(orc)
    dx = (0.1, 0.125, 0.25)
    names = list(PF.STATE_NAMES) + list(PF.DERIVED_NAMES)
    path = PF.write_plotfile_data(str(tmp_path / "plt00010"), names, boxes, data, dx, (-1.0, 0.0, 2.0),
                                  ((0, 0, 0), (10, 8, 4)), time=0.25, step=10)
    hdr = open(os.path.join(path, "Header")).read().split("\n")
    assert hdr[0] == "HyperCLaw-V1.1" and hdr[1] == "10" and hdr[2:12] == names
    assert hdr[12:16] == ["3", "0.25", "0", "-1 0 2 "]
    assert hdr[16] == "0 1 3 " and hdr[17] == ""                       # prob_hi, no refinement ratios
    assert hdr[18] == "((0,0,0) (9,7,3) (0,0,0)) " and hdr[19] == "10 "  # domain, level steps
    assert hdr[20] == "0.10000000000000001 0.125 0.25 "                 # cell sizes, 17 digits
    assert hdr[21:25] == ["0", "0", "0 3 0.25", "10"]
    # box 0 in physical coordinates: prob_lo + lo dx, prob_lo + (hi + 1) dx (RealBox)
    assert hdr[25:28] == ["-1 %.17g" % (-1.0 + 6 * 0.1), "0 0.625", "2 3"]
    assert hdr[34] == "Level_0/Cell"
    ch = open(os.path.join(path, "Level_0", "Cell_H")).read().split("\n")
    assert ch[:5] == ["1", "1", "10", "0", "(3 0"] and ch[5] == "((0,0,0) (5,4,3) (0,0,0))"
    assert [ln.split()[1] for ln in ch if ln.startswith("FabOnDisk:")] == ["Cell_D_00000"] * 3
    raw = open(os.path.join(path, "Level_0", "Cell_D_00000"), "rb").read()
    assert raw.startswith(b"FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))((0,0,0) (5,4,3) (0,0,0)) 10\n")
    rd = PF.read_plotfile(path)
    assert rd["names"] == names and rd["time"] == 0.25 and rd["step"] == 10 and rd["dx"] == list(dx)
    assert [tuple(b[0]) for b in rd["boxes"]] == [b[0] for b in boxes]
    for a, b in zip(rd["data"], data):
        np.testing.assert_array_equal(a, b)
    # per-FAB minima and maxima in the VisMF header
    mins = [float(v) for v in ch[ch.index("3,10") + 1].split(",")[:-1]]
    np.testing.assert_array_equal(mins, data[0].reshape(10, -1).min(axis=1))
