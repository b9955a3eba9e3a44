"""The integer-pipe FP64 division, square root and product
(amrsolver_gb300/csrc/ddiv.cuh) on the device against CUDA's own: 4e9
generated operand pairs for the division (the WENO weight and normalisation
ranges, arbitrary bit patterns, random significands and signs, zero
numerators), 2e9 arguments for the square root (arbitrary bits, the whole
exponent range, squares and their neighbours) and 3e9 operand pairs for the
product (arbitrary bits, rounding ties, the edges of underflow and overflow,
zeros, subnormals and specials, the kernels' constant factors), every result
bit for bit.  The kernels use them in place of the hardware operations, so
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


def test_dsqrt_equals_hardware_sqrt():
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    capi.load(build_if_missing=True)
    h = capi.Handle(P.Scheme(), P.Closures.nondimensional(1e-3))
    for seed in (5, 6):
        bad, first = h.ddiv_check(seed, 1_000_000_000, sqrt=True)
        assert bad == 0, ("square root differs", seed, first)
    h.close()


def test_dmul_equals_hardware_product():
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    capi.load(build_if_missing=True)
    h = capi.Handle(P.Scheme(), P.Closures.nondimensional(1e-3))
    for seed in (7, 8, 9):
        bad, first = h.ddiv_check(seed, 1_000_000_000, mul=True)
        assert bad == 0, ("product differs", seed, first)
    h.close()


def test_intpipe_product_overlaps_fp64_stream():
    """The overlap probe: four integer-pipe products per sixteen FMAs cost a
    saturated FP64 stream less than four hardware products (measured 16.6
    against 20.6 ms, FMAs alone 15.9 ms); an unknown mode is refused."""
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    capi.load(build_if_missing=True)
    h = capi.Handle(P.Scheme(), P.Closures.nondimensional(1e-3))
    fma_only, hw, ip = (h.probe_intpipe(m) for m in (0, 1, 2))
    assert 0.0 < fma_only <= ip < hw, (fma_only, ip, hw)
    with pytest.raises(capi.AmrsError):
        h.probe_intpipe(3)
    h.close()
