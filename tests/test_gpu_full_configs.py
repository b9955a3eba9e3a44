"""The measured configurations at their full sizes, against the CPU oracle.

Each test runs the GPU path the benchmark times, at the size it times, and
the oracle (the restatement that is bit-identical to the reference build) on
the same seeded input, on every host core:

* Taylor-Green vortex 128^3 (M=0.1, Re=1600, Pr=0.71), KEEP4 + viscous,
  100 SSPRK3 steps (src/tim/CNS_advance.cpp:118-139): the kinetic-energy and
  enstrophy series every 10 steps and the final state, bit for bit.
* Batched level: 512 uneven boxes with edges drawn from {8,...,64} (seed
  1234), KEEP4 + viscous, one SSPRK3 step through the box-list CUDA graph:
  every box bit for bit.
* Ensemble: 64 periodic TGV members of 48^3 with their own Mach and
  Reynolds numbers, one SSPRK3 step in one graph: every member bit for bit.
* Large: periodic 256^3 random-phase turbulence (Mt=0.6), mu=1e-4, WENO5-JS
  LLF + viscous in the reference's operation order: one RHS
  (src/tim/CNS_advance.cpp:186-391) within 1e-12 per conserved variable
  (relative max-norm) and three SSPRK3 steps within 1e-10.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest
import torch

from amrsolver_gb300 import capi, cns
from amrsolver_gb300 import problems as P
from tests import golden_io as G
from tests.test_gpu_boxlist import oracle_step_frozen
from tests.test_gpu_configs import ke_enstrophy

pytestmark = pytest.mark.gpu

NT = max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1))


@pytest.fixture(scope="module", autouse=True)
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.load(build_if_missing=True)
    yield
    torch.cuda.empty_cache()


def test_tgv128_100_steps_bitexact(orc):
    n, steps, dt = 128, 100, 1e-3
    U, dx = P.tgv(n, mach=0.1)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    lev = cns.CNSLevel(sc, cl, U, dx)
    dxinv = [1.0 / h for h in dx]
    S = U
    series_gpu, series_orc = [], []
    for s in range(steps):
        lev.advance(lev.time, dt)
        S = orc.advance(sc, cl, S, dxinv, (-1, -1, -1), (-1, -1, -1), dt, nthreads=NT)
        if s % 10 == 9:
            series_gpu.append(ke_enstrophy(lev.valid().cpu().numpy(), dx))
            series_orc.append(ke_enstrophy(P.valid(S), dx))
    lev.h.sync_check()
    assert series_gpu == series_orc
    np.testing.assert_array_equal(lev.valid().cpu().numpy(), P.valid(S))
    assert series_gpu[-1][0] < series_gpu[0][0] and series_gpu[-1][1] > series_gpu[0][1]


def test_batched_512_boxes_graph_bitexact(orc):
    specs, fields, dx = P.batched_boxes(512)
    assert len(specs) == 512 and max(max(s.shape) for s in specs) == 64
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / v for v in dx]
    h = capi.Handle(sc, cl)
    slots = []
    for U in fields:
        t = torch.from_numpy(U).cuda()
        slots.append([t, t.clone(), t.clone()])
    bl = capi.BoxList(h, [s.lo for s in specs], slots, dxinv)
    dt = 1e-4
    res = bl.step(3, 3, dt, use_graph=True)
    h.sync_check()
    got = [slots[b][res][:, 3:-3, 3:-3, 3:-3].cpu().numpy() for b in range(len(specs))]
    bl.close()
    del slots
    # the oracle box by box on every host core (ctypes releases the GIL)
    with cf.ThreadPoolExecutor(NT) as ex:
        refs = list(ex.map(lambda b: oracle_step_frozen(orc, sc, cl, fields[b], dxinv, specs[b].lo, dt),
                           range(len(specs))))
    bad = [b for b in range(len(specs)) if not np.array_equal(got[b], refs[b])]
    assert not bad, "boxes differing from the oracle: %s" % bad[:10]


def test_ensemble_64x48_bitexact(orc):
    nmem, n = 64, 48
    members = P.ensemble_members(nmem, n)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    fields, cls, los, slots = [], [], [], []
    for b, (m, re) in enumerate(members):
        U, dx = P.tgv(n, mach=m)
        fields.append(U)
        cls.append(P.Closures.nondimensional(1.0 / re))
        los.append((b * (n + 16), 0, 0))
        t = torch.from_numpy(U).cuda()
        slots.append([t, t.clone(), t.clone()])
    dxinv = [1.0 / h for h in dx]
    h = capi.Handle(sc, cls[0])
    bl = capi.BoxList(h, los, slots, dxinv, closure_index=list(range(nmem)), closures=cls)
    bl.set_bc((-1, -1, -1), (-1, -1, -1))
    dt = 1e-3
    res = bl.step(3, 3, dt, s1=0, w1=1, w2=2, use_graph=True)
    h.sync_check()
    got = [slots[b][res][:, 3:-3, 3:-3, 3:-3].cpu().numpy() for b in range(nmem)]
    bl.close()
    del slots
    with cf.ThreadPoolExecutor(NT) as ex:
        refs = list(ex.map(lambda b: P.valid(orc.advance(sc, cls[b], fields[b], dxinv, (-1, -1, -1),
                                                         (-1, -1, -1), dt, lo=los[b])), range(nmem)))
    bad = [b for b in range(nmem) if not np.array_equal(got[b], refs[b])]
    assert not bad, "members differing from the oracle: %s" % bad


def test_large_256_weno_visc_rhs_and_steps(orc):
    n = 256
    U, dx = P.random_turbulence(n, mach_t=0.6)
    cl = P.Closures.nondimensional(1e-4)
    sc = P.Scheme(flux_euler=2, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    lev = cns.CNSLevel(sc, cl, U, dx)
    # one RHS of the initial state
    S0 = lev.S.clone()
    lev.fill_patch(S0)
    R = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
    lev.compute_rhs(S0, R)
    lev.h.sync_check()
    got = R.cpu().numpy()
    del S0, R
    ref = orc.rhs(sc, cl, U, dxinv, nthreads=NT)
    dev = G.relmax(got, ref)
    assert dev <= 1e-12, dev
    del got, ref
    # three SSPRK3 steps at CFL 0.3 of the initial state
    dt = lev.est_time_step(0.3)
    S = U
    for _ in range(3):
        lev.advance(lev.time, dt)
        S = orc.advance(sc, cl, S, dxinv, (-1, -1, -1), (-1, -1, -1), dt, nthreads=NT)
    lev.h.sync_check()
    got = lev.valid().cpu().numpy()
    Sv = P.valid(S)
    dev = G.relmax(got, Sv)
    assert dev <= 1e-10, dev
