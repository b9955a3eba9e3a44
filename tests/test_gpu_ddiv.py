"""The integer-pipe FP64 division (amrsolver_gb300/csrc/ddiv.cuh) on the
device against CUDA's own division: 4e9 generated operand pairs (the WENO
weight and normalisation ranges, arbitrary bit patterns, random significands
and signs), every result bit for bit.  The kernels that divide use it, so
this equality is what keeps them equal to the reference's CPU build."""
import pytest
import torch

from amrsolver_gb300 import capi
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu


def test_ddiv_equals_hardware_division():
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    capi.load(build_if_missing=True)
    h = capi.Handle(P.Scheme(), P.Closures.nondimensional(1e-3))
    total = 0
    for seed in (1, 2, 3, 4):
        bad, first = h.ddiv_check(seed, 1_000_000_000)
        assert bad == 0, ("division differs", seed, first)
        total += 1_000_000_000
    assert total >= 4_000_000_000
    h.close()
