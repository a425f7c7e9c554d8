"""A per-schedule autotuner for the fused fill.

The reference has no tuning: its device fill is one launch per group with
KernelAbstractions' default workgroup.  Here each uploaded schedule carries
launch options (``tam_schedule_set_option``) that change speed but never a
result: the box points per warp tile (copies and stencils apart), the threads
per CTA, whether the Float64 stencil multiplies (and a quarter of the adds)
run on the integer pipe, and the grouping and order of the work (stage
groups, stencil tiles grouped by their path through the kernel or by target
block, the order the blocks are visited in, points a lane of the copy kernel
takes at once, the copies' share of the multiprocessors beside the
stencils).  The tuner times every candidate on the caller's own field set
(CUDA events on the fill's stream, best of a few fills after a warm-up; the
data should be representative, since zeros and specials send the
integer-pipe multiplies' points back to the FP64 pipe), keeps the fastest,
and caches the choice per schedule and variable count.  The default grid runs in
the library (``tam_autotune``); other candidate sets are timed from here.
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
    if tuple(tile_items) == TILE_ITEMS and tuple(threads) == THREADS and int_mul is None:
        # the native tuner (tam_autotune): the same grid, timed in the library
        import ctypes as C
        out = [C.c_int64(), C.c_int64(), C.c_int64()]
        ms = C.c_double()
        s = torch.cuda.current_stream(fs.work.device)
        rc = ds.lib.tam_autotune(ds.handle, C.c_void_p(fs.work.data_ptr()), fs.nvars,
                                 fs.nblocks(), C.c_void_p(fs.factors.data_ptr()), reps,
                                 C.c_void_p(s.cuda_stream), C.byref(out[0]), C.byref(out[1]),
                                 C.byref(out[2]), C.byref(ms))
        from . import _native
        _native.check(rc, ds.ctx, "tam_autotune")
        best = {"tile_items": out[0].value, "threads": out[1].value, "int_mul": out[2].value}
        opts = ds.options()
        for k in ("merge_stages", "path_tiles", "staged", "pair_vars", "block_order",
                  "copy_points", "copy_share", "soft_add", "stencil_tile"):
            best[k] = opts[k]
        cache[key] = dict(best)
        sched._tuned_ms = ms.value
        return dict(best)
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
