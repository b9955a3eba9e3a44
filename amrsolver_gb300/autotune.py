"""Autotuner of the fused face kernel's tile shape per box-size class.

The fused KEEP face kernel tiles each box's (x, y) extent into tx x ty
columns (tx * ty <= 256 threads) and streams z through shared memory.  Which
shape wastes the fewest FP64 lanes depends on the box's nx and ny: partial
tiles idle lanes, narrow tiles recompute more x/y pair terms at tile edges.
For every (nx, ny) class present in a box list the tuner times one RK stage
of a probe box of that class for each candidate shape, keeps the fastest,
and applies the winners with amrs_boxlist_set_tile.  Results are cached in a
JSON file keyed by (order, nx, ny, device name).
"""
from __future__ import annotations

import json
import os

import torch

from . import capi
from .problems import BoxSpec, NGHOST, random_state

CANDIDATES = ((32, 8), (16, 16), (24, 10), (8, 30), (16, 8), (8, 16), (8, 8), (32, 4), (24, 8))
DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")


def _key(order, nx, ny):
    return "%s|o%d|%dx%d" % (torch.cuda.get_device_name(), order, nx, ny)


def load_cache(path=DEFAULT_CACHE):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def save_cache(cache, path=DEFAULT_CACHE):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _time_probe(handle, n, tile, reps=3, nz_probe=None):
    """Average ms of one SSPRK3 step of a single-box list of extents n."""
    nz = nz_probe or n[2]
    U = random_state((n[0], n[1], nz), seed=7)
    slots = [[torch.from_numpy(U).cuda() for _ in range(3)]]
    bl = capi.BoxList(handle, [(0, 0, 0)], slots, (64.0, 64.0, 64.0))
    try:
        bl.set_tile((0, 0, 0), tile[0], tile[1], nz)
    except capi.AmrsError:
        bl.close()
        return None
    bl.step(3, 3, 1e-4, use_graph=False)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        bl.step(3, 3, 1e-4, use_graph=False)
    e1.record()
    torch.cuda.synchronize()
    bl.close()
    return e0.elapsed_time(e1) / reps


def tune_class(handle, nx, ny, nz_probe=32, candidates=CANDIDATES, cache=None):
    """Best (tx, ty) for boxes with this (nx, ny); cached."""
    order = handle.scheme.order_keep
    key = _key(order, nx, ny)
    if cache is not None and key in cache:
        return tuple(cache[key]["tile"])
    results = {}
    for t in candidates:
        ms = _time_probe(handle, (nx, ny, nz_probe), t)
        if ms is not None:
            results[t] = ms
    best = min(results, key=results.get)
    if cache is not None:
        cache[key] = {"tile": list(best), "ms": results[best],
                      "sweep": {"%dx%d" % k: v for k, v in results.items()}}
    return best


def tune_boxlist(boxlist, specs, cache_path=DEFAULT_CACHE, nz_probe=32):
    """Tune every (nx, ny) class of `specs` (BoxSpec list) and apply the
    winning tiles to `boxlist`.  Returns {(nx, ny): (tx, ty)}."""
    cache = load_cache(cache_path)
    handle = boxlist.handle
    classes = sorted({(s.shape[0], s.shape[1]) for s in specs})
    choice = {}
    for nx, ny in classes:
        choice[(nx, ny)] = tune_class(handle, nx, ny, nz_probe=nz_probe, cache=cache)
    save_cache(cache, cache_path)
    boxlist.set_tiles([choice[(s.shape[0], s.shape[1])] + (s.shape[2],) for s in specs])
    return choice
