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
  cpu_baseline  the CPU oracle on the host cores (bounded sample).

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
WORKLOAD = "Taylor-Green vortex 128^3 periodic, M=0.1 Re=1600 Pr=0.71, KEEP4 + viscous, SSPRK3"


# --------------------------------------------------------------- helpers --
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


def face_kernel_flops(orc, scheme, closures, n, prog_flops_per_comp):
    """Algorithmic FP64 flops of one fused face-kernel launch over an n^3 box:
    the oracle's operation counts (+,-,*,/,sqrt each 1; no FMA in the oracle)
    of the Euler face fluxes, viscous face averages and divergence, per face
    and per cell, scaled to the box, plus the stage program."""
    from amrsolver_gb300 import problems as P
    m = 16
    U, dx = P.tgv(m)
    per = orc.rhs_counts(scheme, closures, U, [1.0 / h for h in dx], per_phase=True)
    f = lambda d: d["add"] + d["mul"] + d["div"] + d["sqrt"]
    faces_m = 3 * (m + 1) * m * m
    faces_n = 3 * (n + 1) * n * n
    per_face = (f(per["euler_faces"]) + f(per["visc_faces"])) / faces_m
    per_cell_div = f(per["divergence"]) / m ** 3
    total = per_face * faces_n + (per_cell_div + 5 * prog_flops_per_comp) * n ** 3
    return total, per


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
        "config": {"workload": WORKLOAD, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "full 128^3 SSPRK3 steps, OpenMP over k-planes on %d threads" % cores},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- GPU arm --
def cpu_baseline_sample():
    """Bounded CPU sample: TGV 64^3 SSPRK3 steps with the oracle, all cores."""
    from oracle import pyoracle
    from amrsolver_gb300 import problems as P
    orc = pyoracle.oracle()
    cores = len(os.sched_getaffinity(0))
    n = 64
    U, dx = P.tgv(n)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
    dxinv = [1.0 / h for h in dx]
    S = orc.advance(sc, cl, U, dxinv, (-1, -1, -1), (-1, -1, -1), 1e-3, nthreads=cores)
    steps = 0
    t0 = time.perf_counter()
    while True:
        S = orc.advance(sc, cl, S, dxinv, (-1, -1, -1), (-1, -1, -1), 1e-3, nthreads=cores)
        steps += 1
        if time.perf_counter() - t0 > 8.0 or steps >= 40:
            break
    el = time.perf_counter() - t0
    return {"value": n ** 3 * steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "TGV 64^3 KEEP4+viscous, %d SSPRK3 steps, %d OpenMP threads" % (steps, cores)}


def bench_batched(torch, capi, P, nboxes=512, steps=3, warmup=2):
    """Config: 512 uneven boxes (edges {8..64}), one SSPRK3 step; persistent
    box-list launches in a CUDA graph vs per-box launches (one box list of
    one box each)."""
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
    bl.close()
    return {"workload": "512 uneven boxes, edges from {8,16,24,32,48,64}, KEEP4 + viscous, one SSPRK3 step",
            "cells": cells, "batched_graph_cell_updates_per_s": cells / (ms_b * 1e-3),
            "per_box_cell_updates_per_s": cells / (ms_p * 1e-3), "ms_batched": ms_b, "ms_per_box": ms_p,
            "speedup": ms_p / ms_b}


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


def bench_adjoint(torch, P, steps=3):
    """TGV 64^3, M=0.1, Re=400: one SSPRK3 step forward (keeping the stage
    inputs the adjoint needs) vs the step's VJP (three stage VJPs)."""
    from amrsolver_gb300 import adjoint, cns
    n = 64
    U, dx = P.tgv(n, mach=0.1)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
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
    return {"workload": "TGV 64^3 M=0.1 Re=400, one SSPRK3 step", "forward_ms": fwd,
            "forward_keeping_stages_ms": fwd_save, "adjoint_ms": adj, "adjoint_over_forward": adj / fwd}


def run_gpu(args, rank, world, local):
    import torch
    from amrsolver_gb300 import capi, cns
    from amrsolver_gb300 import problems as P
    torch.cuda.set_device(local)
    capi.load(build_if_missing=True)
    n = args.n
    U, dx = P.tgv(n)
    cl = P.Closures.nondimensional(1.0 / 1600.0)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
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
    ms_all = ms
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_all = float(t.item())
    value = world * n ** 3 / (ms_all * 1e-3)

    # ---- end to end through the public API with host buffers
    pin_in = torch.from_numpy(lev.state_host()).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    for _ in range(2):
        lev.S.copy_(pin_in, non_blocking=True)
        lev.advance(lev.time, dt)
        pin_out.copy_(lev.S, non_blocking=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        lev.S.copy_(pin_in, non_blocking=True)
        lev.advance(lev.time, dt)
        pin_out.copy_(lev.S, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    nbytes = pin_in.numel() * 8

    result = None
    if rank == 0:
        # ---- dominant kernel: fused face kernel, timed alone on the stream
        from oracle import pyoracle
        orc = pyoracle.oracle()
        progs = capi.rk_program(3, 3, dt)
        # stage 2 program: Xpay (2 flops) + LinComb (3 flops) per component
        face_flops, per = face_kernel_flops(orc, sc, cl, n, 5)
        peak = lev.h.probe_fp64_tflops()
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
                    "traffic": None, "kernel": "keep_face_kernel<4,true>",
                    "peak_source": "measured: DFMA-chain probe kernel (amrs_probe_fp64_tflops), FMA = 2 flops",
                    "algorithmic_flops_per_launch": face_flops, "ms_per_launch": tf,
                    "stage_kernel_ms": {"prims": kms[0], "visc_cells": kms[1], "faces": kms[2]},
                    "hbm_peak_gbs_measured": None}
        try:
            mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
            roofline["hbm_peak_gbs_measured"] = mp.get("hbm_gbs")
        except Exception:
            pass
        algo_bytes_face = n ** 3 * (3 * 40)  # reads U_s, U^n, writes U_{s+1}: 120 B/cell
        roofline["hbm_achieved_gbs_algorithmic"] = algo_bytes_face / (tf * 1e-3) / 1e9
        prof = os.path.join(ROOT, "profiles", "keep_face_kernel_tgv96.md")
        t96 = read_traffic(prof)
        # traffic grows with the cells processed: scale the 96^3 capture to this box
        roofline["traffic"] = None if t96 is None else t96 * (n ** 3) / 96 ** 3
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_all, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": n ** 3, "l2": "inputs larger than L2 (3 ghosted states + "
                       "scratch ~0.7 GB)", "parallelism": "replicas" if world > 1 else "single GPU",
                       "tma": lev.h.tma_enabled()},
            "e2e": {"value": world * n ** 3 / (ms_e2e * 1e-3), "unit": UNIT, "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "roofline": roofline,
            "gpu_launches": args.steps * 3 * 4,
            "clocks": clk,
        }
        if not args.skip_batched:
            result["batched"] = bench_batched(torch, capi, P)
            result["ensemble"] = bench_ensemble(torch, capi, P)
            result["adjoint"] = bench_adjoint(torch, P)
        if not args.skip_cpu:
            result["cpu_baseline"] = cpu_baseline_sample()
    return result


def read_traffic(path):
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except Exception:
        pass
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=128, help="TGV box edge (128 for the headline; smaller for profiling)")
    args = ap.parse_args()
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
