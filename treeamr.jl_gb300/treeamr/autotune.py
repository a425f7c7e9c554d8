"""A per-schedule autotuner for the fused fill.

The reference has no tuning: its device fill is one launch per group with
KernelAbstractions' default workgroup.  Here each uploaded schedule carries
launch options (``tam_schedule_set_option``) that change speed but never a
result: the box points per warp tile, the threads per CTA, and whether the
Float64 multiplies by short weight products run on the integer pipe.  The
tuner times every candidate on the caller's own field set (CUDA events on the
fill's stream, best of a few fills after a warm-up), keeps the fastest, and
caches the choice per schedule and variable count.
"""
from __future__ import annotations

import itertools
from typing import Dict, Iterable, Optional

import torch

from .ghosts import device_schedule, fill_ghosts
from .schedule import GhostSchedule
from .storage import FieldSet

TILE_ITEMS = (32, 64, 128, 256, 512)
THREADS = (128, 256, 512)


def _time_fill(fs: FieldSet, sched: GhostSchedule, reps: int) -> float:
    stream = torch.cuda.current_stream(fs.work.device)
    fill_ghosts(fs, sched)                                    # warm-up
    best = float("inf")
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fill_ghosts(fs, sched)
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def autotune(fs: FieldSet, sched: GhostSchedule, *, reps: int = 3,
             tile_items: Iterable[int] = TILE_ITEMS, threads: Iterable[int] = THREADS,
             int_mul: Optional[Iterable[int]] = None) -> Dict[str, int]:
    """Pick the fastest launch options for filling ``fs`` with ``sched`` and
    leave them set.  The field set's contents are overwritten by fills (the
    ghosts only: a fill never writes an owned point)."""
    ds = device_schedule(sched, fs.work.device.index or 0)
    cache = sched.__dict__.setdefault("_tuned", {})
    key = (fs.work.device.index, fs.nvars)
    if key in cache:
        for k, v in cache[key].items():
            ds.set_option(k, v)
        return dict(cache[key])
    if int_mul is None:
        int_mul = (0, 1) if fs.T.itemsize == 8 else (0,)
    # every combination: the best tile and CTA size differ between the two
    # multiply paths, so neither is chosen before the other
    results = []
    for im, ti, th in itertools.product(int_mul, tile_items, threads):
        ds.set_option("tile_items", ti)
        ds.set_option("threads", th)
        ds.set_option("int_mul", im)
        results.append((_time_fill(fs, sched, reps), {"tile_items": ti, "threads": th,
                                                      "int_mul": im}))
    best_t, best = min(results, key=lambda r: r[0])
    for k, v in best.items():
        ds.set_option(k, v)
    cache[key] = dict(best)
    sched._tuned_ms = best_t
    return dict(best)
