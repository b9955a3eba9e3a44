"""Autotuner of the fused face kernel: tile shape per box-size class and the
schedule's thread coarsening, timed on the real box list.

The fused KEEP face kernel tiles each box's (x, y) extent into tx x ty
columns (tx * ty <= 256 threads) and streams z through shared memory; a
host-built schedule cuts the (tile column x plane) work of all boxes into
`waves` x (resident CTAs) shares.  Two knobs therefore set how the work
maps onto threads:

* tile shape per (nx, ny) class: partial tiles idle lanes, narrow tiles
  recompute more x/y pair terms at tile edges;
* waves (z coarsening): one wave gives every CTA one long z run, so each
  thread streams the most planes per z prologue; more waves give shorter
  runs that CTAs pick up as others finish.

The reference has no counterpart: its only tiling knob is MFIter over the
boxes of max_grid_size (src/tim/CNS_advance.cpp:200).

`tune_level` times whole SSPRK3 steps of the list itself (its CUDA graph,
CUDA events, best of a few), so the balanced schedule and the interplay of
all boxes are in every measurement.  It starts from the library's default
tiles, sweeps the waves, then one shape for all boxes, then each of the
classes that carry the most work, keeping a change only when it saves more
than the timing noise; finally the winner is timed against the default once
more and the faster of the two is applied, so the tuned list is never
slower than the default by more than the noise.  Steps read state slot `s1`
and write only the two work slots, so the caller's state is not changed.
Results are cached in JSON keyed by device, order and the box-size multiset.
"""
from __future__ import annotations

import hashlib
import json
import os

import torch

from . import capi

CANDIDATES = ((32, 8), (16, 16), (24, 10), (8, 30), (16, 8), (8, 16), (8, 8), (32, 4), (24, 8))
WAVES = (1, 2, 3, 4)
DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")


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


def _level_key(order, shapes):
    h = hashlib.sha1(repr(sorted(shapes)).encode()).hexdigest()[:16]
    return "%s|o%d|%d boxes|%s" % (torch.cuda.get_device_name(), order, len(shapes), h)


class _Timer:
    """Best-of-`reps` time (ms) of one SSPRK3 step of the list through its
    graph, after one untimed step that records the graph."""

    def __init__(self, bl, s1, w1, w2, dt, reps):
        self.bl, self.args, self.dt, self.reps = bl, (s1, w1, w2), dt, reps
        self.count = 0

    def __call__(self):
        s1, w1, w2 = self.args
        self.bl.step(3, 3, self.dt, s1, w1, w2, use_graph=True)
        torch.cuda.synchronize()
        best = float("inf")
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        for _ in range(self.reps):
            e0.record()
            self.bl.step(3, 3, self.dt, s1, w1, w2, use_graph=True)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        self.count += 1
        return best


def tune_level(bl, shapes, s1=0, w1=1, w2=2, dt=1e-4, reps=3, max_classes=4, min_gain=0.005,
               cache_path=DEFAULT_CACHE, use_cache=True):
    """Tune tiles per (nx, ny) class and the schedule's waves of box list `bl`
    whose boxes have valid extents `shapes` ((nx, ny, nz) per box), apply the
    winner and return a report: default and tuned ms per step, the choice
    and every timed candidate."""
    order = bl.handle.scheme.order_keep
    key = _level_key(order, [tuple(s) for s in shapes])
    cache = load_cache(cache_path) if use_cache else {}
    timer = _Timer(bl, s1, w1, w2, dt, reps)
    default_tiles = bl.get_tiles()
    classes = {}
    for b, s in enumerate(shapes):
        classes.setdefault((s[0], s[1]), []).append(b)
    work = {c: sum(shapes[b][0] * shapes[b][1] * shapes[b][2] for b in bs) for c, bs in classes.items()}

    def apply(tiles, waves):
        try:
            bl.set_tiles(tiles)
            bl.set_schedule(waves)
            return True
        except capi.AmrsError:
            return False

    if use_cache and key in cache:
        ent = cache[key]
        tiles = [tuple(t) for t in ent["tiles"]]
        if apply(tiles, ent["waves"]):
            return dict(ent, cached=True)
    sweep = []

    def measure(tiles, waves, label):
        if not apply(tiles, waves):
            return None
        ms = timer()
        sweep.append({"candidate": label, "waves": waves, "ms": ms})
        return ms

    t_default = measure(default_tiles, 1, "default")
    best_tiles, best_w, best_ms = list(default_tiles), 1, t_default
    for w in WAVES[1:]:
        ms = measure(best_tiles, w, "default")
        if ms is not None and ms < best_ms * (1 - min_gain):
            best_w, best_ms = w, ms
    for t in CANDIDATES:
        tiles = [(t[0], t[1], kc) for (_, _, kc) in default_tiles]
        ms = measure(tiles, best_w, "all %dx%d" % t)
        if ms is not None and ms < best_ms * (1 - min_gain):
            best_tiles, best_ms = tiles, ms
    top = sorted(classes, key=lambda c: -work[c])[:max_classes]
    for c in top:
        for t in CANDIDATES:
            tiles = list(best_tiles)
            for b in classes[c]:
                tiles[b] = (t[0], t[1], tiles[b][2])
            if tiles == best_tiles:
                continue
            ms = measure(tiles, best_w, "class %dx%d -> %dx%d" % (c[0], c[1], t[0], t[1]))
            if ms is not None and ms < best_ms * (1 - min_gain):
                best_tiles, best_ms = tiles, ms
    for w in WAVES:
        if w == best_w:
            continue
        ms = measure(best_tiles, w, "tuned tiles")
        if ms is not None and ms < best_ms * (1 - min_gain):
            best_w, best_ms = w, ms
    # the winner against the default, timed once more each
    t_def2 = measure(default_tiles, 1, "default (final)")
    t_best2 = measure(best_tiles, best_w, "tuned (final)")
    if t_best2 > t_def2:
        best_tiles, best_w, t_best2 = list(default_tiles), 1, t_def2
    apply(best_tiles, best_w)
    choice = {}
    for c, bs in classes.items():
        choice["%dx%d" % c] = list(best_tiles[bs[0]][:2])
    rep = {"default_ms": t_def2, "tuned_ms": t_best2, "tuned_over_default": t_def2 / t_best2,
           "waves": best_w, "class_tiles": choice, "tiles": [list(t) for t in best_tiles],
           "candidates_timed": timer.count, "sweep": sweep, "cached": False}
    if use_cache:
        cache[key] = {k: rep[k] for k in ("default_ms", "tuned_ms", "tuned_over_default", "waves", "class_tiles",
                                          "tiles", "candidates_timed")}
        save_cache(cache, cache_path)
    return rep


def tune_boxlist(boxlist, specs, cache_path=DEFAULT_CACHE, **kw):
    """tune_level for a list built from `specs` (problems.BoxSpec); returns
    {(nx, ny): (tx, ty)}."""
    kw.pop("nz_probe", None)
    rep = tune_level(boxlist, [tuple(s.shape) for s in specs], cache_path=cache_path, **kw)
    return {tuple(int(v) for v in c.split("x")): tuple(t) for c, t in rep["class_tiles"].items()}
