"""amrs_average_down against a numpy restatement of AMReX's cell-centred
average_down (Cartesian: the mean of the fine cells of each coarse cell,
summed k-offset outermost, i innermost, from zero, times 1/(rx*ry*rz)).
AMReX is not vendored with the reference, so this follows its published
semantics (parity unpinned against AMReX itself); bit-exact against the
restatement, and conservative to round-off."""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def avgdown_ref(F, ratio, fg=0):
    """F: fine valid+ghost array (ncomp, nzf+2fg, nyf+2fg, nxf+2fg)."""
    rx, ry, rz = ratio
    V = F[:, fg:F.shape[1] - fg, fg:F.shape[2] - fg, fg:F.shape[3] - fg]
    nc, nzf, nyf, nxf = V.shape
    c = np.zeros((nc, nzf // rz, nyf // ry, nxf // rx))
    for kr in range(rz):
        for jr in range(ry):
            for ir in range(rx):
                c = c + V[:, kr::rz, jr::ry, ir::rx]
    return (1.0 / (rx * ry * rz)) * c


@pytest.mark.parametrize("ratio", [(2, 2, 2), (4, 4, 4), (2, 3, 1)])
@pytest.mark.parametrize("crse_lo", [(0, 0, 0), (-3, 5, 2)])
def test_average_down_matches_restatement(ratio, crse_lo):
    rng = np.random.default_rng(sum(ratio) + crse_lo[0])
    nc = (7, 5, 6)
    fg, cg = 2, 1
    F = rng.normal(size=(5, nc[2] * ratio[2] + 2 * fg, nc[1] * ratio[1] + 2 * fg, nc[0] * ratio[0] + 2 * fg))
    C = np.full((5, nc[2] + 2 * cg, nc[1] + 2 * cg, nc[0] + 2 * cg), 7.0)
    Fd, Cd = torch.from_numpy(F).cuda(), torch.from_numpy(C).cuda()
    capi.average_down(Fd, Cd, crse_lo, ratio, fine_g=fg, crse_g=cg)
    torch.cuda.synchronize()
    out = Cd.cpu().numpy()
    np.testing.assert_array_equal(out[:, cg:-cg, cg:-cg, cg:-cg], avgdown_ref(F, ratio, fg))
    # ghosts untouched
    mask = np.ones(out.shape[1:], bool)
    mask[cg:-cg, cg:-cg, cg:-cg] = False
    assert np.all(out[:, mask] == 7.0)
    # conservation: coarse sum times the refinement volume equals the fine sum
    fv = F[:, fg:-fg, fg:-fg, fg:-fg].reshape(5, -1).sum(axis=1)
    cv = out[:, cg:-cg, cg:-cg, cg:-cg].reshape(5, -1).sum(axis=1) * (ratio[0] * ratio[1] * ratio[2])
    np.testing.assert_allclose(cv, fv, rtol=1e-12, atol=1e-12 * np.abs(F).sum())


def test_average_down_component_range_and_bad_inputs():
    F = torch.arange(5 * 4 * 4 * 4, dtype=torch.float64, device="cuda").reshape(5, 4, 4, 4)
    C = torch.zeros((5, 2, 2, 2), dtype=torch.float64, device="cuda")
    capi.average_down(F, C, (0, 0, 0), (2, 2, 2), scomp=2, ncomp=2)
    torch.cuda.synchronize()
    ref = avgdown_ref(F.cpu().numpy(), (2, 2, 2))
    np.testing.assert_array_equal(C.cpu().numpy()[2:4], ref[2:4])
    assert float(C[0].abs().sum()) == 0.0 and float(C[4].abs().sum()) == 0.0
    with pytest.raises(capi.AmrsError):  # the fine array does not cover the refined box
        capi.average_down(F, C, (0, 0, 0), (4, 4, 4))
    with pytest.raises(capi.AmrsError):
        capi.average_down(F, C, (0, 0, 0), (0, 2, 2))
