"""Benchmark of the compressible RHS + SSP-RK path on GB300.

Headline workload: Taylor-Green vortex 128^3 (single periodic box, M=0.1,
Re=1600, Pr=0.71), 4th-order KEEP + viscous fluxes, SSPRK3; one step = one
SSPRK3 step (3 x [ghost fill + primitives + viscous cell fluxes + fused
faces/divergence/stage update]).  Metric: cell-updates/s per RK3 step.

Also reported on the same JSON line:
  e2e       the same step through the public API with host buffers: H2D of
            U^n from pinned memory, the step, D2H of U^{n+1}, every step;
  roofline  the fused face kernel against the measured FP64 FMA peak (this
            path is FP64-pipe bound on GB300), with its algorithmic flops from
            the oracle's operation counts;
  batched   512 uneven boxes, one SSPRK3 step: one persistent launch per
            kernel kind captured in a CUDA graph vs per-box launches;
  ensemble  64 periodic TGV members of 48^3 with per-member closures;
  adjoint   TGV 64^3: VJP of one SSPRK3 step against the forward step
            (adjoint_muscl, adjoint_weno_riemann: the same for those
            schemes; --vjp-only prints every scheme's line alone);
  large     256^3 random-phase turbulence, WENO5-LLF + viscous: 20 SSPRK3
            steps and the adjoint of the final step, with the roofline
            fraction of the whole step; KEEP4 + viscous and the WENO5 ->
            Riemann extension + viscous timed on the same state;
  channel   the reference's channel configuration (walls, device bcnormal,
            body force, Sutherland air) as its own 2 x 2 x 1 decomposition;
  cpu_baseline  the CPU oracle on all host cores and on one thread (bounded
                samples).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s per RK3 step"
UNIT = "cell-updates/s"

# --scheme: (switches, op-count key, dominant kernel, its ncu summary, kernels of ours per stage, label)
SCHEMES = {
    "keep4": (dict(flux_euler=1, order_keep=4, rhs_visc=1), "keep4_visc", "keep_face_kernel<4,true,false>",
              "keep_face_kernel_tgv128.md", 4, "KEEP4 + viscous"),
    "weno": (dict(flux_euler=2, rhs_visc=1), "weno_visc", "weno_face_kernel<true> (reference operation order)",
             "weno_face_kernel_tgv96.md", 7, "WENO5-LLF + viscous, reference operation order"),
    "weno_fast": (dict(flux_euler=2, rhs_visc=1, weno_fast=1), "weno_visc",
                  "weno_face_kernel<false> (common-denominator weights)", "weno_fast_face_kernel_tgv96.md", 7,
                  "WENO5-LLF + viscous, common-denominator weights"),
    "muscl": (dict(flux_euler=0, rhs_visc=1), "muscl_visc", "slope_kernel + riemann_face_kernel",
              "riemann_face_kernel_tgv128.md", 7, "MUSCL-Riemann + viscous"),
    "weno_riemann": (dict(flux_euler=0, riemann_weno=1, rhs_visc=1), "weno_riemann_visc", "weno_riemann_face_kernel",
                     "weno_riemann_face_kernel_tgv128.md", 6,
                     "WENO5-Riemann (extension) + viscous"),
}


def workload_name(scheme, n):
    return "Taylor-Green vortex %d^3 periodic, M=0.1 Re=1600 Pr=0.71, %s, SSPRK3" % (n, SCHEMES[scheme][5])


# --------------------------------------------------------------- helpers --
def headline_config(n, scheme, world, state_bytes):
    """The `config` of the headline line, identical in both arms."""
    return {"workload": workload_name(scheme, n), "cells": n ** 3,
            "l2": "inputs larger than L2 (3 ghosted states + scratch, %.2f GB of states alone)"
            % (3 * state_bytes / 1e9),
            "parallelism": "replicas" if world > 1 else "single GPU"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device):
    """The largest per-rank value over all ranks (the slowest replica's step
    time); `device` is where the process group's backend reduces ("cuda" for
    NCCL, "cpu" for gloo)."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(cells_per_rank, world, ms_max):
    """Whole-job cell-updates/s of `world` replicas that each advanced
    `cells_per_rank` cells in a step of `ms_max` ms (the slowest rank)."""
    return world * cells_per_rank / (ms_max * 1e-3)


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


OP_COUNTS = os.path.join(ROOT, "tests", "golden", "op_counts.json")


def rhs_phase_flops(scheme_name, n):
    """Algorithmic flops per phase of one RHS over an n^3 box: the oracle's
    operation counts (+,-,*,/,sqrt each 1; no FMA in the oracle) as exact
    cubics in n, committed in tests/golden/op_counts.json by
    tests/golden/make_op_counts.py."""
    phases = json.load(open(OP_COUNTS))["schemes"][scheme_name]["phases"]
    return {ph: c[0] * n ** 3 + c[1] * n ** 2 + c[2] * n + c[3] for ph, c in phases.items()}


def face_kernel_flops(scheme_name, n, prog_flops_per_comp):
    """Algorithmic FP64 flops of one fused face-kernel launch over an n^3 box:
    Euler face fluxes, viscous face averages and divergence, plus the stage
    program."""
    per = rhs_phase_flops(scheme_name, n)
    total = per["euler_faces"] + per["visc_faces"] + per["divergence"] + 5 * prog_flops_per_comp * n ** 3
    return total, per


def weno_face_flops(scheme_name, n):
    """Flops of the WENO5 face kernel alone: the Euler phase minus its
    per-cell point fluxes (cons2eulerflux_lambda over grow(box,3), whose
    count is the constant term of the phase's cubic divided by 6^3)."""
    c = json.load(open(OP_COUNTS))["schemes"][scheme_name]["phases"]["euler_faces"]
    per_point = c[3] // 216
    return c[0] * n ** 3 + c[1] * n ** 2 + c[2] * n + c[3] - per_point * (n + 6) ** 3


def riemann_face_flops(key, n):
    """Flops of the Euler faces of one RHS of a Riemann-solver scheme (MUSCL:
    slopes + faces; WENO5-Riemann: faces): the Euler phase as the oracle
    counts it on the first RHS of the TGV 128^3 input (the solver's branches
    make the count data-dependent); other edges scale it by n^3
    (approximate)."""
    ent = json.load(open(OP_COUNTS))["data_dependent"][key]
    return ent["phases"]["euler_faces"] * (n / ent["n"]) ** 3


def prog_flops(progs):
    """FP64 flops per component of the stage programs (LinComb 3, Saxpy 2,
    Xpay 2, Copy 0)."""
    return sum({0: 3, 1: 2, 2: 2, 3: 0}[p.ops[o].kind] for p in progs for o in range(p.nops))


# ----------------------------------------------------------- reference arm --
def run_reference(args, rank, world):
    """The reference's CPU algorithm (the oracle restatement, which is
    bit-identical to the reference build) on the host cores."""
    if rank != 0:
        return 0
    from oracle import pyoracle
    from amrsolver_gb300 import problems as P
    orc = pyoracle.oracle()
    cores = len(os.sched_getaffinity(0))
    n = 128
    U, dx = P.tgv(n)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    dt = 1e-3
    S = U
    for _ in range(args.warmup):
        S = orc.advance(sc, cl, S, dxinv, (-1, -1, -1), (-1, -1, -1), dt, nthreads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        S = orc.advance(sc, cl, S, dxinv, (-1, -1, -1), (-1, -1, -1), dt, nthreads=cores)
    el = time.perf_counter() - t0
    value = n ** 3 * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(n, "keep4", world, U.nbytes),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "full 128^3 SSPRK3 steps, OpenMP over k-planes on %d threads" % cores},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- GPU arm --
def cpu_baseline_sample():
    """Bounded CPU samples: TGV 64^3 SSPRK3 steps with the oracle on all
    cores (OpenMP over k-planes), and on one thread (the reference's CPU
    path has no OpenMP in compute_rhs)."""
    from oracle import pyoracle
    from amrsolver_gb300 import problems as P
    orc = pyoracle.oracle()
    cores = len(os.sched_getaffinity(0))
    n = 64
    U, dx = P.tgv(n)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]

    def sample(threads, seconds, max_steps):
        S = orc.advance(sc, cl, U, dxinv, (-1, -1, -1), (-1, -1, -1), 1e-3, nthreads=threads)
        steps = 0
        t0 = time.perf_counter()
        while True:
            S = orc.advance(sc, cl, S, dxinv, (-1, -1, -1), (-1, -1, -1), 1e-3, nthreads=threads)
            steps += 1
            if time.perf_counter() - t0 > seconds or steps >= max_steps:
                break
        return steps, time.perf_counter() - t0

    steps, el = sample(cores, 8.0, 40)
    steps1, el1 = sample(1, 6.0, 20)
    return {"value": n ** 3 * steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "TGV 64^3 KEEP4+viscous, %d SSPRK3 steps, %d OpenMP threads" % (steps, cores),
            "single_thread": {"value": n ** 3 * steps1 / el1, "unit": UNIT, "cores": 1,
                              "sample": "TGV 64^3 KEEP4+viscous, %d SSPRK3 steps, one thread" % steps1}}


def bench_batched(torch, capi, P, nboxes=512, steps=3, warmup=2):
    """Config: 512 uneven boxes (edges {8..64}), one SSPRK3 step; persistent
    box-list launches in a CUDA graph vs per-box launches (one box list of
    one box each); then the autotuner on the batched list."""
    from amrsolver_gb300 import autotune
    specs, fields, dx = P.batched_boxes(nboxes)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    h = capi.Handle(sc, cl)
    dxinv = [1.0 / v for v in dx]
    slots = []
    for U in fields:
        t = torch.from_numpy(U).cuda()
        slots.append([t, t.clone(), t.clone()])
    cells = sum(s.cells for s in specs)
    los = [s.lo for s in specs]
    bl = capi.BoxList(h, los, slots, dxinv)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    for _ in range(warmup):
        bl.step(3, 3, 1e-4, use_graph=True)
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record()
    for _ in range(steps):
        bl.step(3, 3, 1e-4, use_graph=True)
    e1.record()
    torch.cuda.synchronize()
    ms_b = e0.elapsed_time(e1) / steps
    # per-box launches: one single-box list per box (tables built once)
    singles = [capi.BoxList(h, [los[b]], [slots[b]], dxinv) for b in range(nboxes)]
    for _ in range(warmup):
        for s in singles:
            s.step(3, 3, 1e-4, use_graph=False)
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record()
    for _ in range(steps):
        for s in singles:
            s.step(3, 3, 1e-4, use_graph=False)
    e1.record()
    torch.cuda.synchronize()
    ms_p = e0.elapsed_time(e1) / steps
    for s in singles:
        s.close()
    res = {"workload": "512 uneven boxes, edges from {8,16,24,32,48,64}, KEEP4 + viscous, one SSPRK3 step",
           "cells": cells, "batched_graph_cell_updates_per_s": cells / (ms_b * 1e-3),
           "per_box_cell_updates_per_s": cells / (ms_p * 1e-3), "ms_batched": ms_b, "ms_per_box": ms_p,
           "speedup": ms_p / ms_b}
    # autotuner sweep over tile shapes per box class and the schedule's
    # z coarsening, timed on this list's own graph step
    rep = autotune.tune_level(bl, [tuple(s.shape) for s in specs], dt=1e-4, use_cache=False)
    res["tuned"] = tuned_section(rep, cells)
    res["tuned_speedup_over_per_box"] = ms_p / rep["tuned_ms"]
    bl.close()
    return res


def bench_ensemble(torch, capi, P, nmembers=64, n=48, steps=3, warmup=2):
    """64 independent periodic TGV members of 48^3, M ~ U(0.05,0.3) and
    Re ~ U(200,3200) per member, advanced together: one launch per kernel
    kind per stage, one CUDA graph per SSPRK3 step."""
    members = P.ensemble_members(nmembers, n)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    slots, cls, los = [], [], []
    for b, (m, re) in enumerate(members):
        U, dx = P.tgv(n, mach=m)
        t = torch.from_numpy(U).cuda()
        slots.append([t, t.clone(), t.clone()])
        cls.append(P.Closures.nondimensional(1.0 / re))
        los.append((b * (n + 16), 0, 0))
    h = capi.Handle(sc, cls[0])
    bl = capi.BoxList(h, los, slots, [1.0 / v for v in dx], closure_index=list(range(nmembers)), closures=cls)
    bl.set_bc((-1, -1, -1), (-1, -1, -1))
    s1 = 0
    for _ in range(warmup):
        r = bl.step(3, 3, 1e-3, s1=s1, w1=(s1 + 1) % 3, w2=(s1 + 2) % 3, use_graph=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        bl.step(3, 3, 1e-3, s1=s1, w1=(s1 + 1) % 3, w2=(s1 + 2) % 3, use_graph=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    h.sync_check()
    bl.close()
    cells = nmembers * n ** 3
    return {"workload": "%d periodic TGV members of %d^3, per-member M and Re, one graph per SSPRK3 step"
            % (nmembers, n), "cells": cells, "ms_per_step": ms, "cell_updates_per_s": cells / (ms * 1e-3)}


def bench_adjoint(torch, P, steps=3, scheme=None, label="KEEP4 + viscous"):
    """TGV 64^3, M=0.1, Re=400: one SSPRK3 step forward (keeping the stage
    inputs the adjoint needs) vs the step's VJP (three stage VJPs)."""
    from amrsolver_gb300 import adjoint, cns
    n = 64
    U, dx = P.tgv(n, mach=0.1)
    sc = P.Scheme(**(scheme or dict(flux_euler=1, order_keep=4, rhs_visc=1)))
    lev = cns.CNSLevel(sc, P.Closures.nondimensional(1.0 / 400.0), U, dx)
    dt = 1e-3
    S1 = lev.S.clone()
    wbar = torch.randn((5, n, n, n), dtype=torch.float64, device="cuda")
    for _ in range(2):
        stages, _ = adjoint._forward_step(lev, S1, dt)
        adjoint._step_vjp(lev, stages, dt, wbar)
    torch.cuda.synchronize()
    ev = lambda: torch.cuda.Event(enable_timing=True)
    e0, e1 = ev(), ev()
    e0.record()
    for _ in range(steps):
        lev.advance(lev.time, dt)
    e1.record()
    torch.cuda.synchronize()
    fwd = e0.elapsed_time(e1) / steps
    e0.record()
    for _ in range(steps):
        stages, _ = adjoint._forward_step(lev, S1, dt)
    e1.record()
    torch.cuda.synchronize()
    fwd_save = e0.elapsed_time(e1) / steps
    e0.record()
    for _ in range(steps):
        adjoint._step_vjp(lev, stages, dt, wbar)
    e1.record()
    torch.cuda.synchronize()
    adj = e0.elapsed_time(e1) / steps
    lev.h.sync_check()
    return {"workload": "TGV 64^3 M=0.1 Re=400, %s, one SSPRK3 step" % label, "forward_ms": fwd,
            "forward_keeping_stages_ms": fwd_save, "adjoint_ms": adj, "adjoint_over_forward": adj / fwd}


def bench_checkpointed(torch, P, n=64, nsteps=200, every=20, dt=2e-3):
    """The adjoint configuration at full size: TGV 64^3, M = 0.1, Re = 400,
    d KE(after 200 SSPRK3 steps)/d(V0, mu) with a checkpoint every 20 steps:
    the forward run's time, the checkpointed adjoint run's time (forward with
    checkpoints + recomputed segments + step VJPs) and the gradient against
    central differences of two more forward runs each."""
    from amrsolver_gb300 import adjoint, cns
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    mu0 = 1.0 / 400.0
    U, dx = P.tgv(n, mach=0.1, amp=1.0)
    cl = P.Closures.nondimensional(mu0)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def run(amp, mu):
        Ua, _ = P.tgv(n, mach=0.1, amp=amp)
        lv = cns.CNSLevel(sc, P.Closures.nondimensional(mu), Ua, dx)
        for _ in range(nsteps):
            lv.advance(lv.time, dt)
        return float(adjoint.kinetic_energy(lv.valid()))

    run(1.0, mu0)
    lev = cns.CNSLevel(sc, cl, U, dx)
    e0, e1 = ev(), ev()
    e0.record()
    for _ in range(nsteps):
        lev.advance(lev.time, dt)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1)
    lev = cns.CNSLevel(sc, cl, U, dx)
    adj = adjoint.CheckpointedAdjoint(lev, every=every)
    e0.record()
    ubar0, pbar, _ = adj.run(torch.from_numpy(P.valid(U).copy()).cuda(), nsteps, dt, adjoint.kinetic_energy_grad)
    e1.record()
    torch.cuda.synchronize()
    adj_ms = e0.elapsed_time(e1)
    # the same with every stage input kept (no recompute; 3 ghosted states a step)
    lev2 = cns.CNSLevel(sc, cl, U, dx)
    e0.record()
    adjoint.CheckpointedAdjoint(lev2, every=nsteps).run(torch.from_numpy(P.valid(U).copy()).cuda(), nsteps, dt,
                                                       adjoint.kinetic_energy_grad)
    e1.record()
    torch.cuda.synchronize()
    keep_ms = e0.elapsed_time(e1)
    del lev2
    h = 1e-3
    dU = (P.valid(P.tgv(n, mach=0.1, amp=1.0 + h)[0]) - P.valid(P.tgv(n, mach=0.1, amp=1.0 - h)[0])) / (2 * h)
    g_v0 = float(np.sum(ubar0.cpu().numpy() * dU))
    pb = pbar.cpu().numpy()
    g_mu = float(pb[0] + cl.cp / 0.71 * pb[1])
    eps = 1e-6
    fd_v0 = (run(1.0 + eps, mu0) - run(1.0 - eps, mu0)) / (2 * eps)
    fd_mu = (run(1.0, mu0 * (1 + eps)) - run(1.0, mu0 * (1 - eps))) / (2 * eps * mu0)
    lev.h.sync_check()
    return {"workload": "TGV %d^3 M=0.1 Re=400, KEEP4 + viscous, d KE(after %d SSPRK3 steps)/d(V0, mu), "
                        "checkpoint every %d steps" % (n, nsteps, every),
            "forward_run_ms": fwd_ms, "checkpointed_adjoint_run_ms": adj_ms, "adjoint_over_forward": adj_ms / fwd_ms,
            "all_stages_kept_adjoint_run_ms": keep_ms, "all_stages_kept_over_forward": keep_ms / fwd_ms,
            "dKE_dV0": g_v0, "dKE_dV0_rel_err_vs_fd": abs(g_v0 - fd_v0) / abs(fd_v0),
            "dKE_dmu": g_mu, "dKE_dmu_rel_err_vs_fd": abs(g_mu - fd_mu) / abs(fd_mu)}


VJP_SCHEMES = (("KEEP4 + viscous", dict(flux_euler=1, order_keep=4, rhs_visc=1)),
               ("WENO5-LLF + viscous", dict(flux_euler=2, rhs_visc=1)),
               ("MUSCL-Riemann + viscous", dict(flux_euler=0, rhs_visc=1)),
               ("WENO5-Riemann + viscous", dict(flux_euler=0, riemann_weno=1, rhs_visc=1)),
               ("KEEP4 + JST + viscous", dict(flux_euler=1, order_keep=4, rhs_visc=1, art_diss=1)))


def run_vjp_only():
    """Adjoint-step vs forward-step time of every scheme with a reverse pass
    (bench_adjoint's TGV 64^3 case), one JSON line on rank 0."""
    import torch
    from amrsolver_gb300 import capi
    from amrsolver_gb300 import problems as P
    capi.load(build_if_missing=True)
    res = {"metric": "adjoint/forward time per SSPRK3 step", "schemes": {}}
    for label, skw in VJP_SCHEMES:
        res["schemes"][label] = bench_adjoint(torch, P, steps=2, scheme=skw, label=label)
    print(json.dumps(res), flush=True)
    return 0


def bench_level(torch, capi, P, n=128, box=32, steps=10, warmup=3):
    """TGV n^3 as the reference runs it: a level of (n/box)^3 boxes of box^3
    cells whose ghosts come from their neighbours (single-level FillPatch
    across the level, periodic images included), one CUDA graph per SSPRK3
    step; the same number of cell updates as the single-box headline.  Then
    the autotuner on this level."""
    from amrsolver_gb300 import autotune
    U, dx = P.tgv(n)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    h = capi.Handle(P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1), cl)
    g = P.NGHOST
    los, slots = [], []
    m = n // box
    for kz in range(m):
        for ky in range(m):
            for kx in range(m):
                B = U[:, kz * box:kz * box + box + 2 * g, ky * box:ky * box + box + 2 * g,
                      kx * box:kx * box + box + 2 * g]
                t = torch.from_numpy(np.ascontiguousarray(B)).cuda()
                slots.append([t, torch.empty_like(t), torch.empty_like(t)])
                los.append((kx * box, ky * box, kz * box))
    bl = capi.BoxList(h, los, slots, [1.0 / v for v in dx])
    bl.set_domain((0, 0, 0), (n, n, n), (-1, -1, -1), (-1, -1, -1))
    dt = 1e-3
    for _ in range(warmup):
        r = bl.step(3, 3, dt, 0, 1, 2, use_graph=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        # the same graph every step: result slot copied back is not needed for timing
        r = bl.step(3, 3, dt, 0, 1, 2, use_graph=True)
    e1.record()
    torch.cuda.synchronize()
    h.sync_check()
    ms = e0.elapsed_time(e1) / steps
    res = {"workload": "TGV %d^3 as %d boxes of %d^3, ghosts from neighbours (level FillPatch in the graph), "
                       "KEEP4 + viscous, one SSPRK3 step" % (n, m ** 3, box),
           "ms_per_step": ms, "cell_updates_per_s": n ** 3 / (ms * 1e-3), "result_slot": r}
    res["tuned"] = tuned_section(autotune.tune_level(bl, [(box, box, box)] * m ** 3, dt=dt, use_cache=False),
                                 n ** 3)
    bl.close()
    return res


def tuned_section(rep, cells):
    """The autotuner's report in the JSON line: default vs tuned step time
    (each best of three graph launches, timed back to back at the end of the
    sweep), the choice and the sweep size."""
    return {"default_ms_per_step": rep["default_ms"], "tuned_ms_per_step": rep["tuned_ms"],
            "tuned_over_default": rep["tuned_over_default"],
            "tuned_cell_updates_per_s": cells / (rep["tuned_ms"] * 1e-3), "waves": rep["waves"],
            "class_tiles": rep["class_tiles"], "candidates_timed": rep["candidates_timed"],
            "sweep": [[e["candidate"], e["waves"], round(e["ms"], 4)] for e in rep["sweep"]]}


def bench_sod(torch, capi, P):
    """Sod tube 256x8x8 (WENO5-LLF, outflow x, periodic y/z) to t = 0.2 at
    CFL 0.3 with the reference's dt control: the whole run as one device
    launch (amrs_rk_run_boxlist) against the host-driven loop (one step and
    one dt reduction read back per step)."""
    import time as _time
    from amrsolver_gb300 import cns
    U, dx = P.sod(256, 8, 8)
    cl = P.Closures.air_sutherland()
    sc = P.Scheme(flux_euler=2, rhs_visc=0)
    bc = (2, -1, -1)
    stop, cfl = 0.2, 0.3
    h = capi.Handle(sc, cl)
    t0 = torch.from_numpy(U).cuda()
    slots = [[t0.clone(), t0.clone(), t0.clone()]]
    bl = capi.BoxList(h, [(0, 0, 0)], slots, [1.0 / v for v in dx])
    bl.set_domain((0, 0, 0), (256, 8, 8), bc, bc)
    res = {}
    for rep in range(2):  # the first run captures the graph
        slots[0][0].copy_(t0)
        torch.cuda.synchronize()
        w0 = _time.perf_counter()
        bl.run(3, 3, stop_time=stop, max_steps=100000, cfl=cfl)
        t, dt, steps = bl.run_state()
        res["device_loop_ms"] = (_time.perf_counter() - w0) * 1e3
    res["steps"] = steps
    res["final_time"] = t
    lev = cns.CNSLevel(sc, cl, U, dx, bc_lo=bc, bc_hi=bc)
    torch.cuda.synchronize()
    w0 = _time.perf_counter()
    lev.run(stop, 100000, cfl=cfl)
    torch.cuda.synchronize()
    res["host_loop_ms"] = (_time.perf_counter() - w0) * 1e3
    res["same_state"] = bool(torch.equal(lev.valid(), slots[0][0][:, 3:-3, 3:-3, 3:-3]))
    res["speedup"] = res["host_loop_ms"] / res["device_loop_ms"]
    h.sync_check()
    res["workload"] = "Sod 256x8x8 WENO5-LLF to t=0.2, CFL 0.3 dynamic dt: one graph launch vs host loop (wall clock)"
    return res


def bench_large(torch, capi, P, peak, n=256, steps=20):
    """Periodic 256^3 random-phase turbulence (E(k) ~ k^4 exp(-2 (k/4)^2),
    turbulent Mach 0.6, rho = 1, p = 1/gamma), mu = 1e-4, Pr = 0.71, WENO5-LLF +
    viscous, SSPRK3 at a fixed dt (CFL 0.3 of the initial state): 20 steps,
    then the adjoint of the final step (cotangent: gradient of the mean
    kinetic energy).  Both WENO5 weight evaluations: the reference's
    operation order (bit-identical) and the common-denominator form.  On the
    same state: KEEP4 + viscous (the headline scheme, whole-step FP64
    fraction) and the WENO5 -> Riemann extension + viscous."""
    import gc
    from amrsolver_gb300 import adjoint, cns
    U, dx = P.random_turbulence(n, mach_t=0.6)
    cl = P.Closures.nondimensional(1e-4)
    per = rhs_phase_flops("weno_visc", n)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    res = {"workload": "periodic %d^3 random-phase turbulence (Mt=0.6, E(k)~k^4 exp(-2(k/4)^2)), mu=1e-4, "
                       "Pr=0.71, WENO5-LLF + viscous, SSPRK3: %d steps then the adjoint of the final step"
                       % (n, steps),
           "cells": n ** 3, "algorithmic_flops_per_rhs": sum(per.values()), "dt": None}
    dt = None
    rhs_of, final_of = {}, {}
    for fast in (0, 1):
        lev = cns.CNSLevel(P.Scheme(flux_euler=2, rhs_visc=1, weno_fast=fast), cl, U, dx)
        if dt is None:
            dt = lev.est_time_step(0.3)
            res["dt"] = dt
        progs = capi.rk_program(3, 3, dt)
        flops_step = 3 * sum(per.values()) + 5 * prog_flops(progs) * n ** 3
        # one RHS of the initial state (to compare the two weight forms)
        S0 = lev.S.clone()
        lev.fill_patch(S0)
        R0 = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
        lev.compute_rhs(S0, R0)
        rhs_of[fast] = R0
        del S0
        # one untimed warm-up step, then restart from the initial state
        lev.advance(lev.time, dt)
        lev.bufs[lev.cur].copy_(torch.from_numpy(U))
        lev.time = 0.0
        tot0 = lev.totals()
        torch.cuda.synchronize()
        e0, e1, e2, e3 = ev(), ev(), ev(), ev()
        e0.record()
        for _ in range(steps - 1):
            lev.advance(lev.time, dt)
        e1.record()
        S_last = lev.S.clone()
        e2.record()
        lev.advance(lev.time, dt)
        e3.record()
        torch.cuda.synchronize()
        ms_fwd = (e0.elapsed_time(e1) + e2.elapsed_time(e3)) / steps
        tot1 = lev.totals()
        final = lev.valid().clone()
        wbar = adjoint.kinetic_energy_grad(final)
        f0, f1, f2 = ev(), ev(), ev()
        f0.record()
        stages, out = adjoint._forward_step(lev, S_last, dt)
        f1.record()
        ubar, _ = adjoint._step_vjp(lev, stages, dt, wbar)
        f2.record()
        torch.cuda.synchronize()
        lev.h.sync_check()
        same = bool(torch.equal(out[:, 3:-3, 3:-3, 3:-3], final))
        # periodic box: totals change by round-off only (relative to sum |U_n|)
        scale = (lev.valid().abs().reshape(5, -1).sum(dim=1) * (2 * math.pi) ** 3).cpu().numpy()
        cons = max(abs(float(a) - float(b)) / float(c) for a, b, c in zip(tot0, tot1, scale))
        achieved = flops_step / (ms_fwd * 1e-3) / 1e12
        res["weno_fast" if fast else "weno_reference_order"] = {
            "ms_per_step": ms_fwd, "cell_updates_per_s": n ** 3 / (ms_fwd * 1e-3),
            "achieved_tflops_algorithmic": achieved, "frac_of_fp64_peak": achieved / peak,
            "forward_step_keeping_stages_ms": f0.elapsed_time(f1), "adjoint_step_ms": f1.elapsed_time(f2),
            "adjoint_over_forward": f1.elapsed_time(f2) / ms_fwd,
            "recomputed_final_step_bit_identical": same,
            "conserved_totals_max_rel_change": cons,
            "ubar_norm": float(torch.linalg.vector_norm(ubar))}
        final_of[fast] = final
        del lev, stages, out, S_last, wbar, ubar
        gc.collect()
        torch.cuda.empty_cache()

    def relmax(a, b):
        # max |a-b| / max |b| per conserved component
        return [float((a[c] - b[c]).abs().max() / b[c].abs().max()) for c in range(5)]

    # the common-denominator weights against the reference order (which is
    # bit-identical to the reference build): one RHS and after all the steps
    res["weno_fast"]["relmax_vs_reference_order_one_rhs"] = relmax(rhs_of[1], rhs_of[0])
    res["weno_fast"]["relmax_vs_reference_order_after_steps"] = relmax(final_of[1], final_of[0])
    # the headline scheme on the same 256^3 state: KEEP4 + viscous, whole-step
    # algorithmic FP64 fraction (bit-identical to the reference build)
    lev = cns.CNSLevel(P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1), cl, U, dx)
    progs = capi.rk_program(3, 3, res["dt"])
    kper = rhs_phase_flops("keep4_visc", n)
    kflops = 3 * sum(kper.values()) + 5 * prog_flops(progs) * n ** 3
    for _ in range(2):
        lev.advance(lev.time, res["dt"])
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    ksteps = 10
    e0.record()
    for _ in range(ksteps):
        lev.advance(lev.time, res["dt"])
    e1.record()
    torch.cuda.synchronize()
    lev.h.sync_check()
    kms = e0.elapsed_time(e1) / ksteps
    kach = kflops / (kms * 1e-3) / 1e12
    res["keep4_visc"] = {"ms_per_step": kms, "cell_updates_per_s": n ** 3 / (kms * 1e-3), "steps": ksteps,
                         "achieved_tflops_algorithmic": kach, "frac_of_fp64_peak": kach / peak}
    del lev
    gc.collect()
    torch.cuda.empty_cache()
    # the WENO5 -> two-shock Riemann extension (riemann_weno = 1) + viscous
    # on the same state; its operation count depends on the data (the
    # solver's branches), so only time and rates are reported
    lev = cns.CNSLevel(P.Scheme(flux_euler=0, riemann_weno=1, rhs_visc=1), cl, U, dx)
    tot0 = lev.totals()
    lev.advance(lev.time, res["dt"])
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    wsteps = 5
    e0.record()
    for _ in range(wsteps):
        lev.advance(lev.time, res["dt"])
    e1.record()
    torch.cuda.synchronize()
    lev.h.sync_check()
    wms = e0.elapsed_time(e1) / wsteps
    tot1 = lev.totals()
    scale = (lev.valid().abs().reshape(5, -1).sum(dim=1) * (2 * math.pi) ** 3).cpu().numpy()
    res["weno_riemann_visc"] = {
        "ms_per_step": wms, "cell_updates_per_s": n ** 3 / (wms * 1e-3), "steps": wsteps,
        "conserved_totals_max_rel_change": max(abs(float(a) - float(b)) / float(c)
                                               for a, b, c in zip(tot0, tot1, scale)),
        "finite": bool(torch.isfinite(lev.valid()).all())}
    del lev
    gc.collect()
    torch.cuda.empty_cache()
    return res


def bench_channel(torch, capi, P, steps=10):
    """The reference's channel configuration: 96 x 128 x 64 cells over
    0.08214 x 0.0136871 x 0.02738 m, x and z periodic, code-6 y walls
    (exm/Channel/inputs), air with Sutherland laws, wall temperature 500 K,
    bulk Mach 1.5, the x body force of the example's parameters
    (exm/Channel/prob.h ProbParm), KEEP4 + viscous + source, the isothermal
    no-slip bcnormal on the device; the example's decomposition
    (max_grid_size 64, blocking factor 16: 2 x 2 x 1 boxes of 48 x 64 x 64),
    one CUDA graph per SSPRK3 step.  A laminar profile with a seeded
    perturbation stands in for the example's initial field."""
    n = (96, 128, 64)
    ext = (0.08214, 0.0136871, 0.02738)
    dx = tuple(ext[d] / n[d] for d in range(3))
    cl = P.Closures.air_sutherland()
    g = P.NGHOST
    h_half, Tw, u_tau, re_tau, re_b, mach_b, muw = 0.006845, 500.0, 35.0, 220.0, 3.0e3, 1.5, 2.670533348e-5
    rho_w = re_tau * muw / (u_tau * h_half)
    pw = rho_w * cl.Rspec * Tw
    ub = mach_b * math.sqrt(cl.gamma * cl.Rspec * Tw)
    rho_b = re_b * muw / (ub * h_half)
    fx = rho_w * u_tau * u_tau / (h_half * rho_b)
    rng = np.random.default_rng(2026)
    shape = (n[2] + 2 * g, n[1] + 2 * g, n[0] + 2 * g)
    y = (np.arange(-g, n[1] + g) + 0.5) * dx[1]
    prof = 1.5 * ub * (1.0 - ((y - h_half) / h_half) ** 2)
    u = prof[None, :, None] * (1.0 + 0.02 * rng.standard_normal(shape))
    v = 0.01 * ub * rng.standard_normal(shape)
    w = 0.01 * ub * rng.standard_normal(shape)
    rho = np.full(shape, pw / (cl.Rspec * Tw))
    U = P.prims_to_cons(rho, u, v, w, np.full(shape, pw), cl.gamma)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1, body_force=(fx, 0.0, 0.0))
    h = capi.Handle(sc, cl)
    los, slots = [], []
    for y0 in (0, 64):
        for x0 in (0, 48):
            B = np.ascontiguousarray(U[:, :, y0:y0 + 64 + 2 * g, x0:x0 + 48 + 2 * g])
            t = torch.from_numpy(B).cuda()
            los.append((x0, y0, 0))
            slots.append([t, t.clone(), t.clone()])
    bl = capi.BoxList(h, los, slots, [1.0 / v_ for v_ in dx])
    bl.set_domain((0, 0, 0), n, (-1, 6, -1), (-1, 6, -1))
    bl.set_bcnormal(P.BCNormal.channel_wall(Tw, n, dx, Tmin=50.0))
    cmax = math.sqrt(cl.gamma * cl.Rspec * Tw) + 1.5 * ub * 1.1
    dt = 0.3 * min(dx) / cmax
    s = [0, 1, 2]

    def step():
        r = bl.step(3, 3, dt, s[0], s[1], s[2], use_graph=True)
        others = [q for q in (0, 1, 2) if q != r]
        s[0], s[1], s[2] = r, others[0], others[1]

    for _ in range(2):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    h.sync_check()
    ms = e0.elapsed_time(e1) / steps
    finite = all(bool(torch.isfinite(sl[s[0]]).all()) for sl in slots)
    cells = n[0] * n[1] * n[2]
    return {"workload": "channel 96x128x64 (x/z periodic, code-6 y walls with the device isothermal bcnormal), "
                        "air Sutherland, KEEP4 + viscous + x body force, 2x2x1 boxes of 48x64x64, graph per step",
            "cells": cells, "dt": dt, "steps": steps, "ms_per_step": ms,
            "cell_updates_per_s": cells / (ms * 1e-3), "finite": finite}


def run_gpu(args, rank, world, local):
    import torch
    from amrsolver_gb300 import capi, cns
    from amrsolver_gb300 import problems as P
    torch.cuda.set_device(local)
    capi.load(build_if_missing=True)
    n = args.n
    U, dx = P.tgv(n)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(**SCHEMES[args.scheme][0])
    dt = 1e-3
    lev = cns.CNSLevel(sc, cl, U, dx, device=local)
    stream = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 3)):
        lev.advance(lev.time, dt)
    lev.h.sync_check()
    # clock samples: nvidia-smi starts while further untimed steps keep the
    # GPU loaded, and keeps sampling through the timed region
    clocks = ClockSampler(local)
    clocks.start()
    t_load = time.perf_counter()
    while time.perf_counter() - t_load < 0.8:
        for _ in range(10):
            lev.advance(lev.time, dt)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        lev.advance(lev.time, dt)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    lev.h.sync_check()
    ms_all = max_over_ranks(ms, world, "cuda")
    value = replica_throughput(n ** 3, world, ms_all)

    # ---- end to end through the public API with host buffers: every step
    # copies its input state from pinned host memory and reads its result
    # back.  Two levels alternate, and the input and result copies have
    # their own streams, so one step's copies run on the copy engines while
    # the other step computes.
    pin_in = torch.from_numpy(lev.state_host()).pin_memory()
    pin_out = [torch.empty_like(pin_in).pin_memory() for _ in range(2)]
    lev2 = cns.CNSLevel(sc, cl, U, dx, device=local)
    levs = [lev, lev2]
    s_comp, s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    free = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_steps(count):
        for s in range(count):
            L, b = levs[s % 2], s % 2
            with torch.cuda.stream(s_in):
                s_in.wait_event(free[b])
                L.S.copy_(pin_in, non_blocking=True)
                ev_in = torch.cuda.Event()
                ev_in.record(s_in)
            s_comp.wait_event(ev_in)
            L.advance(L.time, dt, stream=s_comp)
            ev_done = torch.cuda.Event()
            ev_done.record(s_comp)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_done)
                pin_out[b].copy_(L.S, non_blocking=True)
                free[b].record(s_out)

    e2e_steps(4)
    torch.cuda.synchronize()
    e0.record(s_in)
    e2e_steps(args.steps)
    s_in.wait_stream(s_out)
    e1.record(s_in)
    torch.cuda.synchronize()
    lev2.h.sync_check()
    ms_e2e = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, "cuda")
    nbytes = pin_in.numel() * 8
    del lev2, levs

    result = None
    if rank == 0:
        # ---- dominant kernel: fused face kernel, timed alone on the stream
        progs = capi.rk_program(3, 3, dt)
        # stage 2 program: Xpay (2 flops) + LinComb (3 flops) per component
        spec = SCHEMES[args.scheme]
        if args.scheme == "keep4":
            face_flops, per = face_kernel_flops(spec[1], n, prog_flops(progs[1:2]))
            algo_bytes_face = n ** 3 * (3 * 40)  # reads U_s, U^n, writes U_{s+1}: 120 B/cell
        elif args.scheme == "muscl":
            face_flops = riemann_face_flops(spec[1], n)
            # reads Q (6 comps) per cell, writes and re-reads 3 x 5 slopes, writes 3 x 5 face values
            algo_bytes_face = n ** 3 * (48 + 2 * 120) + 3 * (n + 1) * n * n * 40
        elif args.scheme == "weno_riemann":
            face_flops = riemann_face_flops(spec[1], n)
            # reads Q (5 comps) per cell, writes 3 x 5 face values
            algo_bytes_face = n ** 3 * 40 + 3 * (n + 1) * n * n * 40
        else:
            face_flops = weno_face_flops(spec[1], n)
            # reads U (40), point fluxes (120) and lambda (24) per cell, writes 3 x 5 face values
            algo_bytes_face = n ** 3 * (40 + 120 + 24) + 3 * (n + 1) * n * n * 40
        peak, peak_info = fp64_peak(torch, lev.h, local)
        S0 = lev.S
        out = torch.empty_like(S0)
        s1 = lev.bufs[(lev.cur + 1) % 3]
        lev.fill_patch(S0)
        # the face kernel alone, CUDA events on the launching stream
        lev.h.profile_stage_box(progs[1], S0, s1, out, lev.dxinv, lev.lo, reps=2, stream=stream)
        kms = lev.h.profile_stage_box(progs[1], S0, s1, out, lev.dxinv, lev.lo, reps=max(args.steps, 5),
                                      stream=stream)
        tf = kms[2]
        achieved = face_flops / (tf * 1e-3) / 1e12
        roofline = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                    "traffic": None, "kernel": spec[2], "peak_source": peak_info,
                    "algorithmic_flops_per_launch": face_flops, "ms_per_launch": tf,
                    "staging": "tma" if lev.h.tma_enabled() else "plain loads",
                    "stage_kernel_ms": {"prims": kms[0], "visc_cells": kms[1], "faces": kms[2]},
                    "hbm_peak_gbs_measured": None}
        try:
            mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
            roofline["hbm_peak_gbs_measured"] = mp.get("hbm_gbs")
        except Exception:
            pass
        roofline["hbm_achieved_gbs_algorithmic"] = algo_bytes_face / (tf * 1e-3) / 1e9
        prof = os.path.join(ROOT, "profiles", spec[3])
        tr, tcells = read_traffic(prof)
        # DRAM bytes per launch from the committed ncu capture; a capture of a
        # smaller box is scaled by the cells processed (traffic grows with them)
        roofline["traffic"] = None if tr is None else tr * (n ** 3) / tcells
        roofline["traffic_source"] = spec[3]
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_all, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(n, args.scheme, world, U.nbytes),
            "e2e": {"value": replica_throughput(n ** 3, world, ms_e2e), "unit": UNIT, "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "roofline": roofline,
            "gpu_launches": args.steps * 3 * spec[4],
            "clocks": clk,
        }
        if not args.skip_batched:
            result["batched"] = bench_batched(torch, capi, P)
            result["ensemble"] = bench_ensemble(torch, capi, P)
            result["adjoint"] = bench_adjoint(torch, P)
            result["adjoint_muscl"] = bench_adjoint(torch, P, scheme=dict(flux_euler=0, rhs_visc=1),
                                                    label="MUSCL-Riemann + viscous")
            result["adjoint_checkpointed"] = bench_checkpointed(torch, P)
            result["adjoint_weno_riemann"] = bench_adjoint(
                torch, P, scheme=dict(flux_euler=0, riemann_weno=1, rhs_visc=1), label="WENO5-Riemann + viscous")
            result["level"] = bench_level(torch, capi, P, n=n)
            result["sod_device_loop"] = bench_sod(torch, capi, P)
            result["channel"] = bench_channel(torch, capi, P)
        if not args.skip_large:
            result["large"] = bench_large(torch, capi, P, peak)
        if not args.skip_cpu:
            result["cpu_baseline"] = cpu_baseline_sample()
        result["summary"] = summary_of(result)
    return result


def fp64_peak(torch, h, local, seconds=1.5):
    """FP64 roofline denominator: the larger of (a) the DFMA-chain probe
    (amrs_probe_fp64_tflops_timed, one launch of about `seconds`) and (b) the
    nominal rate of the pipe, SMs x 2 DFMA lanes per clock x 2 flops x the
    median SM clock sampled over the probe's launch."""
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.2)
    tf, ms = h.probe_fp64_tflops(seconds=seconds)
    clk = clocks.stop()
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    info = {"probe_tflops": tf, "probe_ms": ms, "sms": nsm, "probe_sm_mhz_median": clk.get("sm_mhz"),
            "sm_max_mhz": clk.get("sm_max_mhz"), "probe_clock_reasons": clk.get("reasons"),
            "rule": "max(probe, nominal at the sampled SM clock); FMA = 2 flops"}
    nominal = None
    if mhz:
        nominal = nsm * 2 * 2 * mhz * 1e6 / 1e12
        info["nominal_tflops_at_sampled_mhz"] = nominal
        info["probe_frac_of_nominal"] = tf / nominal
        info["probe_ms_x_mhz"] = ms * mhz
    if clk.get("sm_max_mhz"):
        info["nominal_tflops_at_max_mhz"] = nsm * 4 * clk["sm_max_mhz"] * 1e6 / 1e12
    peak = max(tf, nominal or 0.0)
    info["chosen"] = "probe" if peak == tf else "nominal at sampled clock"
    # what four products per 16 FMAs cost beside a full FP64 pipe: hardware
    # products take FP64 slots, the integer-pipe product (part of the kernels'
    # products) overlaps with the FMAs
    ip = [h.probe_intpipe(m) for m in (0, 1, 2)]
    info["intpipe_probe_ms"] = {"fma_only": ip[0], "fma_plus_hw_products": ip[1],
                                "fma_plus_intpipe_products": ip[2]}
    return peak, info


def summary_of(result):
    """A compact digest of the metric's numbers, printed as the line's last
    key: cell-updates/s batched vs per box, adjoint / forward step time, and
    the roofline fractions (of the FP64 peak in `roofline.peak`)."""
    out = {"headline_cell_updates_per_s": result.get("value"), "headline_e2e": result["e2e"]["value"],
           "face_kernel_frac": result["roofline"]["frac"], "fp64_peak_tflops": result["roofline"]["peak"]}
    b = result.get("batched")
    if b:
        out["batched_graph_cell_updates_per_s"] = b["batched_graph_cell_updates_per_s"]
        out["per_box_cell_updates_per_s"] = b["per_box_cell_updates_per_s"]
        out["batched_speedup"] = b["speedup"]
        if "tuned" in b:
            out["batched_tuned_over_default"] = b["tuned"].get("tuned_over_default")
    lv = result.get("level")
    if lv and "tuned" in lv:
        out["level_64x32cubed_tuned_over_default"] = lv["tuned"]["tuned_over_default"]
    e = result.get("ensemble")
    if e:
        out["ensemble_cell_updates_per_s"] = e["cell_updates_per_s"]
    a = result.get("adjoint")
    if a:
        out["adjoint_over_forward_keep4_tgv64"] = a.get("adjoint_over_forward")
    c = result.get("adjoint_checkpointed")
    if c:
        out["checkpointed_200_steps_adjoint_over_forward"] = c.get("adjoint_over_forward")
    lg = result.get("large")
    if lg:
        for k in ("weno_reference_order", "weno_fast", "keep4_visc"):
            if k in lg:
                out["large_256_%s_frac" % k] = lg[k].get("frac_of_fp64_peak")
                out["large_256_%s_cell_updates_per_s" % k] = lg[k].get("cell_updates_per_s")
        if "weno_reference_order" in lg:
            out["large_256_adjoint_over_forward"] = lg["weno_reference_order"].get("adjoint_over_forward")
    return out


def read_traffic(path):
    """(traffic_bytes_per_launch, cells_per_launch) of a profiles/ summary."""
    tr, cells = None, None
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                tr = float(line.split(":")[1])
            elif line.startswith("cells_per_launch:"):
                cells = float(line.split(":")[1])
    except Exception:
        pass
    return tr, cells or 96.0 ** 3


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-large", action="store_true", help="skip the 256^3 WENO5 + viscous section")
    ap.add_argument("--scheme", default="keep4", choices=sorted(SCHEMES),
                    help="scheme of the TGV line (keep4 is the headline; weno* for profiling the WENO path)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=128, help="TGV box edge (128 for the headline; smaller for profiling)")
    ap.add_argument("--vjp-only", action="store_true",
                    help="only the adjoint-step timings (TGV 64^3) of every scheme with a reverse pass, one JSON "
                         "line; used to profile the reverse kernels")
    args = ap.parse_args()
    if args.vjp_only:
        return run_vjp_only()
    rank, world, local = dist_env()
    if world > 1:
        import torch
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            torch.cuda.set_device(local)
        torch.distributed.init_process_group(backend)
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
    else:
        res = run_gpu(args, rank, world, local)
        if rank == 0 and res is not None:
            print(json.dumps(res), flush=True)
        rc = 0
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
