"""The sharded level on one GPU (world size 1): the halo plan's device
gather/scatter and the library box-list backend must give the same bits as
the library's own level (amrs_boxlist_set_domain) and as the CPU oracle on
one box covering the domain.  The two-rank exchange itself is covered by
tests/test_distributed_cpu.py (gloo)."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi
from amrsolver_gb300 import distributed as D
from amrsolver_gb300 import problems as P
from tests.test_distributed_cpu import _boxes, _cut, _domain_field, CASES

pytestmark = pytest.mark.gpu
G = P.NGHOST


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


@pytest.mark.parametrize("case", sorted(CASES))
def test_sharded_level_one_rank_matches_oracle(orc, case):
    c = CASES[case]
    U, dx = _domain_field(case)
    boxes = _boxes(case)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    cl = P.Closures.nondimensional(1.0 / 500.0)
    lev = D.DistributedLevel(sc, cl, boxes, [_cut(U, lo, n) for lo, n in boxes], dx, ((0, 0, 0), c["n"]),
                             c["bc_lo"], c["bc_hi"], device="cuda")
    Uf = U.copy()
    orc.fill_halo(Uf, c["bc_lo"], c["bc_hi"])
    dt = lev.est_time_step(0.3)
    assert dt == orc.est_timestep(cl, Uf, dx, 0.3)
    S = Uf
    dxinv = [1.0 / v for v in dx]
    for _ in range(3):
        lev.advance(dt)
        S = orc.advance(sc, cl, S, dxinv, c["bc_lo"], c["bc_hi"], dt)
    lev.backend.h.sync_check()
    for b, (lo, n) in enumerate(boxes):
        ref = S[:, G + lo[2]:G + lo[2] + n[2], G + lo[1]:G + lo[1] + n[1], G + lo[0]:G + lo[0] + n[0]]
        np.testing.assert_array_equal(lev.valid(b).cpu().numpy(), ref)
    lev.close()
