"""Box-list path (one launch per kernel kind over many boxes, CUDA graph):
bit-for-bit against the oracle applied box by box.

Batched level: isolated boxes whose ghost cells keep their analytic initial
values for the whole step.  Ensemble: periodic TGV members, each with its own
closures (Mach and Reynolds number), advanced in one launch.
"""
import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)


def oracle_step_frozen(orc, sc, cl, U, dxinv, lo, dt, order_rk=3, stages_rk=3):
    """CNS::advance on one isolated box whose ghosts stay at U's ghost values."""
    g = 3
    v = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    S1 = U.copy()
    S2 = U.copy()
    for p in capi.rk_program(order_rk, stages_rk, dt):
        Sb = U.copy()
        Sb[v] = (S1 if p.src_state == 0 else S2)[v]
        reg = [S1[v].copy(), S2[v].copy(), orc.rhs(sc, cl, Sb, dxinv, lo=lo)]
        for o in range(p.nops):
            q = p.ops[o]
            if q.kind == 0:
                reg[q.dst] = q.a * reg[q.x] + q.b * reg[q.y]
            elif q.kind == 1:
                reg[q.dst] = reg[q.dst] + q.a * reg[q.x]
            elif q.kind == 2:
                reg[q.dst] = reg[q.x] + q.a * reg[q.dst]
            else:
                reg[q.dst] = reg[q.x].copy()
        S2[v] = reg[1]
    return S2[v]


@pytest.mark.parametrize("use_graph", [True, False])
def test_batched_boxes_bitexact(orc, use_graph):
    specs, fields, dx = P.batched_boxes(nboxes=20, seed=77, edges=(8, 16, 24))
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / v for v in dx]
    h = capi.Handle(sc, cl)
    slots = []
    for U in fields:
        t = torch.from_numpy(U).cuda()
        slots.append([t, t.clone(), t.clone()])
    bl = capi.BoxList(h, [s.lo for s in specs], slots, dxinv)
    dt = 2e-3
    res = bl.step(3, 3, dt, use_graph=use_graph)
    h.sync_check()
    for b, (s, U) in enumerate(zip(specs, fields)):
        ref = oracle_step_frozen(orc, sc, cl, U, dxinv, s.lo, dt)
        got = slots[b][res][:, 3:-3, 3:-3, 3:-3].cpu().numpy()
        np.testing.assert_array_equal(got, ref)


def test_ensemble_per_member_closures(orc):
    members = P.ensemble_members(4, seed=5)
    n = 16
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    fields, cls = [], []
    for m, re in members:
        U, dx = P.tgv(n, mach=m)
        fields.append(U)
        cls.append(P.Closures.nondimensional(1.0 / re))
    dxinv = [1.0 / h for h in dx]
    h = capi.Handle(sc, cls[0])
    slots = []
    los = []
    for b, U in enumerate(fields):
        t = torch.from_numpy(U).cuda()
        slots.append([t, t.clone(), t.clone()])
        los.append((b * 100, 0, 0))
    bl = capi.BoxList(h, los, slots, dxinv, closure_index=list(range(4)), closures=cls)
    bl.set_bc((-1, -1, -1), (-1, -1, -1))
    dt = 1e-2
    res = bl.step(3, 3, dt, use_graph=True)
    res = bl.step(3, 3, dt, s1=res, w1=(res + 1) % 3, w2=(res + 2) % 3, use_graph=False)
    h.sync_check()
    for b in range(4):
        ref = fields[b]
        for _ in range(2):
            ref = orc.advance(sc, cls[b], ref, dxinv, (-1, -1, -1), (-1, -1, -1), dt, lo=los[b])
        got = slots[b][res][:, 3:-3, 3:-3, 3:-3].cpu().numpy()
        np.testing.assert_array_equal(got, P.valid(ref))


def test_tile_shapes_do_not_change_bits(orc):
    """Every tile shape the autotuner may pick gives the same bits."""
    specs, fields, dx = P.batched_boxes(nboxes=3, seed=3, edges=(24, 32))
    cl = P.Closures.nondimensional(1.0 / 1000.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / v for v in dx]
    h = capi.Handle(sc, cl)
    outs = []
    for tx, ty, kc in [(32, 8, 8), (16, 16, 5), (8, 30, 32), (24, 10, 3), (8, 8, 1)]:
        slots = [[torch.from_numpy(U).cuda() for _ in range(3)] for U in fields]
        bl = capi.BoxList(h, [s.lo for s in specs], slots, dxinv)
        bl.set_tile((0, 0, 0), tx, ty, kc)
        res = bl.step(3, 3, 1e-3, use_graph=False)
        h.sync_check()
        outs.append([slots[b][res].cpu().numpy() for b in range(3)])
        bl.close()
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a[:, 3:-3, 3:-3, 3:-3], b[:, 3:-3, 3:-3, 3:-3])


def test_schedule_waves_do_not_change_bits():
    """The schedule's z coarsening (amrs_boxlist_set_schedule) only moves
    work between CTAs: every setting gives the same bits."""
    specs, fields, dx = P.batched_boxes(nboxes=5, seed=4, edges=(16, 24, 40))
    cl = P.Closures.nondimensional(1.0 / 1000.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / v for v in dx]
    h = capi.Handle(sc, cl)
    outs, grids = [], []
    for waves in (1, 2, 3, 8):
        slots = [[torch.from_numpy(U).cuda() for _ in range(3)] for U in fields]
        bl = capi.BoxList(h, [s.lo for s in specs], slots, dxinv)
        bl.set_schedule(waves)
        grids.append(bl.face_grid())
        res = bl.step(3, 3, 1e-3, use_graph=True)
        h.sync_check()
        outs.append([slots[b][res].cpu().numpy() for b in range(len(specs))])
        bl.close()
    assert grids[0] < grids[1] < grids[2] <= grids[3]
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a[:, 3:-3, 3:-3, 3:-3], b[:, 3:-3, 3:-3, 3:-3])
