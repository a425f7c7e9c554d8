"""Ghost-fill benchmark: GB/s of the batched fused fill on the walls mesh, one GB300.

Workload (the default): the walls mesh, 3-D vertex-centred, 8^3 roots over
the unit cube, N = 32, G = 2, low faces reflecting and high faces outflow,
five levels nested around two seeded points, 8 Float64 variables (5 even, a
vector's 3 components odd in their own dimension), point-value operators of
order 4 (2,374 blocks, 7.7 GB of field data), filled with its stated data
(Gaussian bumps of width 0.05 plus seeded uniform noise in [-1, 1]).  A step
is one whole ghost fill, stages P and 0 included.  ``value`` counts the
reference's algorithmic bytes (one read plus one write per ghost
point-variable written, ``bench/copies.jl:17-21``) per second with the field
data resident in HBM; ``e2e`` is the same through the C ABI with the field
data copied from pinned host memory and back every step.  The field data are
far larger than L2 (129 MB), so no flush is needed between steps.  The
sphere mesh, the adjoint's mesh, the walls mesh in the other element type,
the batch of 64 forests and the other parts of the path are measured in the
same line under ``workloads``.

``--impl reference`` times the CPU restatement of the reference's threaded
fill (the oracle, ``oracle/fill_oracle.c``) on this machine's host cores, on
the same mesh and data: the reference itself is Julia, which this machine
does not have.

Launch: ``python bench.py [--gpus N] [--steps K] [--warmup W]``; N > 1 under
torchrun runs N independent replicas, one a GPU (a fill is one forest's, on one GPU).
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "treeamr.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "ghost-fill GB/s (batched fused fill, algorithmic bytes)"
UNIT = "GB/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--method", choices=["fused", "plain"], default="fused")
    ap.add_argument("--roots", type=int, default=8)
    ap.add_argument("--levels", type=int, default=3)
    ap.add_argument("--nvars", type=int, default=4)
    ap.add_argument("--walls-levels", type=int, default=5,
                    help="refinement levels of the walls mesh (5 as stated; fewer for profiling)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-walls", action="store_true")
    ap.add_argument("--no-fp64-peak", action="store_true",
                    help="skip the DGEMM measurement of the FP64 rate (the fp64 roofline)")
    ap.add_argument("--options", default=None,
                    help="fixed launch options instead of the autotuner's, e.g. "
                         "tile_items=64,threads=128,int_mul=1")
    ap.add_argument("--workload", choices=["sphere", "walls", "batch"], default="walls",
                    help="walls: the headline line (the walls mesh); sphere, batch: time only "
                         "the sphere mesh or the batch of forests and print its entry")
    ap.add_argument("--forests", type=int, default=64,
                    help="forests of the batch (64 as stated; fewer for profiling)")
    ap.add_argument("--dtype", choices=["float32", "float64"], default="float64",
                    help="element type of the walls mesh")
    ap.add_argument("--sector-minimum", default=None, metavar="TAG",
                    help="count, on the CPU, the 32-byte sectors the unit copies of stage TAG "
                         "of the walls mesh read and write, print them and exit; 'all': every "
                         "stage, stencils with their whole source windows, and the whole fill's "
                         "least traffic against its algorithmic bytes")
    ap.add_argument("--sector-unit", type=int, default=32,
                    help="the access unit --sector-minimum counts in bytes (32: an L2 "
                         "sector; 64: the DRAM's access unit)")
    return ap.parse_args()


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's time: every rank's replica is timed alone, and the
    job's time is the maximum (an all-reduce on ``device``, which is a CUDA
    device under NCCL and the CPU under gloo)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def stencil_flops(sched, nvars, one_tap=True):
    """Algorithmic FP64/FP32 operations of each stage's stencil transfers: per
    target point-variable one multiply and one add per tap the reference's
    sum takes (src/ghosts.jl:75-118), with the CPU form's one tap along a
    dimension whose weight column has a single nonzero weight.  Copies have
    none."""
    out = {}
    for gr in sched.groups:
        if gr.unit():
            continue
        taps = 1
        for st in gr.stencils:
            nz = np.count_nonzero(st.weights, axis=0)
            eff = np.where((nz == 1) & one_tap, 1, st.order)
            taps *= int(eff.sum())               # a tensor-product box: product of sums
        out[gr.stage] = out.get(gr.stage, 0) + 2 * taps * gr.ntransfers() * nvars
    return out


def fused_launches(sched, ds=None):
    """Kernel launches of one fused fill: per stage (or stage group, when the
    uploaded schedule ``ds`` runs consecutive stages as one) a copy launch
    when it has unit copies and a stencil launch when it has stencils."""
    tags = sorted({gr.stage for gr in sched.groups})
    merged = []
    if ds is not None and ds.options().get("merge_stages", 0):
        ng, nin = ds.stage_groups()
        merged = [ng, nin]
    n = 0
    for tag in tags:
        grs = [gr for gr in sched.groups if gr.stage == tag]
        n += any(gr.unit() for gr in grs) + any(not gr.unit() for gr in grs)
    if merged and merged[0]:
        # a group of k prolongation stages runs one stencil launch instead of
        # k (their stencils only, on the walls and sphere meshes)
        n -= merged[1] - merged[0]
    return n


def fp64_peak_tflops(dev):
    """cuBLAS DGEMM, 4096^3, best of 5 (CUDA events): the FP64 rate the
    stencil stages are compared with."""
    import torch
    n = 4096
    a = torch.rand(n, n, dtype=torch.float64, device=dev)
    b = torch.rand(n, n, dtype=torch.float64, device=dev)
    c = a @ b
    best = None
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del a, b, c
    return 2 * n ** 3 / (best * 1e-3) / 1e12


def fp64_roofline(flops, stage_ms, peak_tf):
    """The FP64-pipe view of the stencil stages: algorithmic operations (a
    multiply and an add per tap, no fused multiply-add, as the reference's
    rounding requires) per second against the measured DGEMM rate, which
    counts a fused multiply-add as two.  Stages without stencils are left
    out."""
    ms = {k: statistics.mean(v) for k, v in stage_ms.items() if k in flops}
    tot_ms = sum(ms.values())
    tot = sum(flops[k] for k in ms)
    ach = tot / (tot_ms * 1e-3) / 1e12 if tot_ms else 0.0
    return {"bound": "fp64", "achieved": ach, "peak": peak_tf, "unit": "TFLOP/s",
            "frac": ach / peak_tf if peak_tf else None,
            "peak_source": "measured here: cuBLAS DGEMM 4096^3, best of 5",
            "stage_tflops": {str(k): flops[k] / (ms[k] * 1e-3) / 1e12 for k in ms},
            "stage_flops": {str(k): flops[k] for k in ms}}


def measure_batch(dev, timed, args, peak):
    """The uneven batch: 64 independent periodic cell-centred forests (roots per
    side from {2..6}^3, N from {8, 16}, 1-4 levels around seeded points), G=2,
    2 Float32 variables (u, v), PV(4,4).  The batched fill (one launch per stage
    for all forests) against 64 separate fills; 10 RK4 steps of the wave
    equation replayed from one CUDA graph against the same steps launched
    eagerly; and the adjoint sweep through the 10 steps with checkpoints every
    2 steps."""
    import torch
    from treeamr import fill_ghosts, meshes
    from treeamr.wave import WaveSolver
    fss, scheds, batch = meshes.forest_batch_setup(n=args.forests, device=dev)
    g = torch.Generator(device=dev).manual_seed(9)
    batch.arena.uniform_(-1.0, 1.0, generator=g)
    esize = 4
    bytes_per_fill = 2 * batch.ghost_points() * esize
    if args.options:
        for kv in args.options.split(","):
            k, v = kv.split("=")
            batch.set_option(k.strip(), int(v))
        tuned = dict(batch.options)
    else:
        tuned = batch.autotune()
    batch.arena.uniform_(-1.0, 1.0, generator=g)
    for _ in range(args.warmup):
        batch.fill()
    steps = max(3, args.steps // 2)
    ms = timed(batch.fill, steps)
    # each stage's launches for every forest, CUDA events on the launching stream
    stream = torch.cuda.current_stream(dev)
    tags = sorted({gr.stage for s in scheds for gr in s.groups})
    evs = []
    for _ in range(3):
        for tag in tags:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            batch._run("tam_batch_fill_ex", batch.arena, tag, tag, stream)
            b.record(stream)
            evs.append((tag, a, b))
    torch.cuda.synchronize(dev)
    stage_ms = {}
    for tag, a, b in evs:
        stage_ms.setdefault(str(tag), []).append(a.elapsed_time(b))
    stage_ms = {k: statistics.mean(v) for k, v in stage_ms.items()}
    stage_bytes = {str(tag): 2 * esize * batch.nvars * sum(
        int(np.prod(gr.boxsize())) * gr.ntransfers() for s in scheds for gr in s.groups
        if gr.stage == tag) for tag in tags}
    if args.workload == "batch":
        return {"forests": len(fss), "blocks": sum(fs.forest.nleaves() for fs in fss),
                "ms_per_fill": ms, "value": bytes_per_fill / (ms * 1e-3) / 1e9,
                "stage_ms": stage_ms, "stage_bytes": stage_bytes, "tuned": tuned}

    def separate():
        for fs, s in zip(fss, scheds):
            fill_ghosts(fs, s)
    separate()
    ms_sep = timed(separate, max(2, steps // 2))
    solver = WaveSolver(batch)
    y = batch.arena
    y.mul_(1e-3)
    eager_ms = timed(lambda: [solver.step(y) for _ in range(10)], 1)
    graph = solver.capture(y, steps=10)
    graph.replay()
    graph_ms = timed(graph.replay, 2)
    y0 = y.clone()
    w = torch.rand(y.shape, dtype=y.dtype, device=dev, generator=g)
    solver.gradient(y0, 2, lambda v: 2 * w * v, checkpoint=2)      # prepares the adjoints
    bwd_ms = timed(lambda: solver.gradient(y0, 10, lambda v: 2 * w * v, checkpoint=2), 1)
    out = {
        "workload": "batch64: 64 periodic cell-centred forests, roots per side from {2..6}^3, "
                    "N from {8,16}, 1-4 levels, G=2, 2 vars F32 (u, v), PV(4,4)",
        "dtype": "float32", "forests": len(fss),
        "blocks": sum(fs.forest.nleaves() for fs in fss),
        "field_bytes": batch.arena.numel() * esize,
        "value": bytes_per_fill / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_fill": ms,
        "separate_fills": {"ms_per_fill": ms_sep, "speedup_batched": ms_sep / ms},
        "rk4_10_steps": {"graph_ms": graph_ms, "eager_ms": eager_ms,
                         "fills": 40, "dt": solver.dt},
        "adjoint_10_steps_checkpoint_2_ms": bwd_ms,
        "stage_ms": stage_ms, "stage_bytes": stage_bytes, "tuned": tuned,
        "roofline": {"bound": "hbm", "achieved": bytes_per_fill / (ms * 1e-3) / 1e9,
                     "peak": peak, "unit": "GB/s",
                     "frac": bytes_per_fill / (ms * 1e-3) / 1e9 / peak},
    }
    del graph, solver, batch
    torch.cuda.empty_cache()
    return out


def measure_walls(T, dev, timed, args, peak):
    """The walls mesh: 3-D vertex-centred, 8^3 roots over the unit cube, N=32, G=2,
    low faces reflecting and high faces outflow, five levels nested around two
    seeded points, 8 variables (5 even, a vector's 3 components odd in their
    own dimension), PV(4,4).  Fused (autotuned) and plain fills, per-stage
    launches of the fused kernel for the roofline."""
    import statistics
    import torch
    from treeamr import GhostSchedule, fill_ghosts, meshes
    from treeamr.autotune import autotune
    from treeamr.ghosts import device_schedule
    f, fs, ops = meshes.walls_setup(device=dev, T=T, roots=args.roots, levels=args.walls_levels)
    sched = GhostSchedule(fs, ops)
    meshes.config_fill(fs, "walls", seed=3)
    esize = np.dtype(T).itemsize
    bytes_per_fill = 2 * sched.ghost_items(fs.nvars) * esize
    if args.options:
        ds0 = device_schedule(sched, dev.index)
        for kv in args.options.split(","):
            k, v = kv.split("=")
            ds0.set_option(k.strip(), int(v))
        tuned = ds0.options()
    else:
        tuned = autotune(fs, sched)
        meshes.config_fill(fs, "walls", seed=3)
    for _ in range(args.warmup):
        fill_ghosts(fs, sched)
    steps = max(3, args.steps // 2)
    ms = timed(lambda: fill_ghosts(fs, sched), steps)
    # the fill's deviation from a wider evaluation of the same stencils
    filled = fs.work.cpu().numpy()
    err = fill_error(sched, filled, filled, fs.nvars, fs.factors_host)
    del filled
    fill_ghosts(fs, sched, method="plain")
    ms_plain = timed(lambda: fill_ghosts(fs, sched, method="plain"), max(2, steps // 2))
    # unify! of the set (stages P and 0 alone: every secondary copy of a
    # shared point takes its primary's value)
    from treeamr.unify import unify
    unify(fs, sched)
    ms_unify = timed(lambda: unify(fs, sched), max(2, steps // 2))
    unify_bytes = 2 * esize * fs.nvars * sum(int(np.prod(g.boxsize())) * g.ntransfers()
                                             for g in sched.groups if g.stage <= 0)
    ds = device_schedule(sched, dev.index)
    stream = torch.cuda.current_stream(dev)
    tags = sorted({gr.stage for gr in sched.groups})
    stage_ms = {}
    evs = []
    for _ in range(3):
        for tag in tags:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ds.run(fs, tag, tag, "fused")
            b.record(stream)
            evs.append((tag, a, b))
    torch.cuda.synchronize(dev)
    for tag, a, b in evs:
        stage_ms.setdefault(tag, []).append(a.elapsed_time(b))
    kern_ms = sum(statistics.mean(v) for v in stage_ms.values())
    achieved = bytes_per_fill / (kern_ms * 1e-3) / 1e9
    fp = None
    if T == np.float64 and getattr(args, "fp64_peak", None):
        fp = fp64_roofline(stencil_flops(sched, fs.nvars), stage_ms, args.fp64_peak)
    out = {
        "workload": "walls: 3-D vertex, 8^3 roots, N=32, G=2, reflecting low / outflow high "
                    "faces, 5 levels around 2 seeded points, 8 vars (5 even, 3 odd), PV(4,4)",
        "data": "Gaussian bumps of width 0.05 at the 2 seeded refinement centres + seeded "
                "U[-1,1]",
        "dtype": np.dtype(T).name, "blocks": f.nleaves(), "groups": len(sched.groups),
        "field_bytes": fs.work.numel() * esize,
        "value": bytes_per_fill / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms,
        "plain": {"value": bytes_per_fill / (ms_plain * 1e-3) / 1e9, "ms_per_step": ms_plain,
                  "speedup_fused_vs_plain": ms_plain / ms},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "stage_ms": {str(k): statistics.mean(v) for k, v in stage_ms.items()},
                     "kernels": kernel_rooflines(sched, stage_ms, {
                         t: 2 * esize * fs.nvars * sum(int(np.prod(g.boxsize())) * g.ntransfers()
                                                       for g in sched.groups if g.stage == t)
                         for t in tags}, peak)},
        "fp64": fp,
        "error": err,
        "unify": {"ms": ms_unify, "bytes": unify_bytes,
                  "gbs": unify_bytes / (ms_unify * 1e-3) / 1e9},
        "tuned": tuned,
        "gpu_launches_per_fill": fused_launches(sched, ds),
    }
    del fs, sched, ds
    torch.cuda.empty_cache()
    return out


def measure_hook(dev, timed, args):
    """The device boundary hook (CellBoundary with a built-in quadratic
    polynomial): the sphere mesh without periodic faces, 4^3 roots, N=16,
    G=3, 3 levels, 4 Float64 variables; the fill with the hook against the
    same stages without it."""
    import torch
    from treeamr import FieldSet, GhostSchedule, Operators, fill_ghosts, meshes
    from treeamr.boundary import CellBoundary, Polynomial
    from treeamr.ghosts import device_schedule
    from treeamr import _native
    f = meshes.sphere_forest(roots=4, N=16, levels=3, periodic=False)
    fs = FieldSet(f, args.nvars, G=3, T=np.float64, device=dev)
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    fs.work.uniform_(-1.0, 1.0)
    terms = {(0, 0, 0): [1.0] * args.nvars, (1, 0, 0): [0.5] * args.nvars,
             (0, 1, 0): [-0.25] * args.nvars, (0, 0, 2): [0.125] * args.nvars}
    hook = CellBoundary(Polynomial(terms))
    fill_ghosts(fs, sched, boundary=hook)
    steps = max(3, args.steps // 2)
    ms_hook = timed(lambda: fill_ghosts(fs, sched, boundary=hook), steps)
    ms_plain = timed(lambda: fill_ghosts(fs, sched), steps)
    pts = sum(int(np.prod([z - a + 1 for a, z in r.region])) for r in sched.boundaries)
    out = {"workload": "sphere without periodic faces: 4^3 roots, N=16, G=3, 3 levels, "
                       f"{args.nvars} vars F64, PV(4,4), quadratic polynomial boundary",
           "blocks": f.nleaves(), "regions": len(sched.boundaries),
           "hook_points_per_var": pts, "fill_with_hook_ms": ms_hook,
           "fill_without_hook_ms": ms_plain, "hook_ms": ms_hook - ms_plain}
    del fs, sched
    torch.cuda.empty_cache()
    return out


def measure_pv6(dev, timed, args):
    """The sphere mesh with the order-6 variant of its operators, PV(6,6):
    the same 8^3 periodic roots, N=16, G=3, 3 levels and 4 Float64
    variables; fused (autotuned) and plain fills, and the stated error."""
    import torch
    from treeamr import GhostSchedule, fill_ghosts, meshes
    from treeamr.autotune import autotune
    f, fs, ops = meshes.sphere_setup(device=dev, nvars=args.nvars, roots=args.roots,
                                     levels=args.levels, p=6)
    sched = GhostSchedule(fs, ops)
    # tuned on the stated data: on zeros the integer-pipe multiplies hand
    # every point back to the FP64 pipe and would look slower than they are
    meshes.config_fill(fs, "sphere", seed=11)
    tuned = autotune(fs, sched)
    meshes.config_fill(fs, "sphere", seed=11)
    bytes_per_fill = 2 * sched.ghost_items(fs.nvars) * 8
    fill_ghosts(fs, sched)
    steps = max(3, args.steps // 2)
    ms = timed(lambda: fill_ghosts(fs, sched), steps)
    filled = fs.work.cpu().numpy()
    err = fill_error(sched, filled, filled, fs.nvars, fs.factors_host, per_group=1)
    del filled
    fill_ghosts(fs, sched, method="plain")
    ms_plain = timed(lambda: fill_ghosts(fs, sched, method="plain"), max(2, steps // 2))
    out = {"workload": f"sphere, PV(6,6): {args.roots}^3 periodic roots, N=16, G=3, "
                       f"{args.levels} levels, {args.nvars} vars F64",
           "blocks": f.nleaves(), "groups": len(sched.groups),
           "value": bytes_per_fill / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms,
           "plain": {"ms_per_step": ms_plain, "speedup_fused_vs_plain": ms_plain / ms},
           # the stencils' algorithmic FP64 operations over the whole fill's
           # time (copies included): a lower bound of the stencil stages' rate
           "fp64_tflops_over_fill": sum(stencil_flops(sched, fs.nvars).values()) / (ms * 1e-3)
           / 1e12,
           "error": err, "tuned": tuned}
    del fs, sched
    torch.cuda.empty_cache()
    return out


def measure_regrid(dev, timed, args):
    """The regrid transfer (``regrid!``'s move of the own points) on the
    sphere mesh: every level-0 leaf with x < 0.25 refined and a tenth of the
    finest families coarsened, then balanced; 4 Float64 variables, PV(4,4).
    Algorithmic bytes: one read and one write per new own point-variable."""
    import torch
    from treeamr import Operators, meshes
    from treeamr.forest import parentkey, sortedchildkeys
    from treeamr.regrid import RegridTransfer
    f = meshes.sphere_forest(roots=args.roots, N=16, levels=args.levels)
    old = list(f.leaves)
    refine = [k for k in old if k.level == 0 and f.block_extent(k)[0][1] <= 0.25]
    top = max(k.level for k in old)
    index = set(old)
    fams = sorted({parentkey(k) for k in old if k.level == top})
    fams = [p for p in fams if all(c in index for c in sortedchildkeys(p))][::10]
    f.refine(refine)
    f.coarsen(fams)
    f.balance()
    t = RegridTransfer(f, old, 3, ("cell",) * 3, np.float64,
                       Operators(prolongation=4, restriction=4))
    S = t.stored
    a = torch.empty((len(old), args.nvars) + tuple(reversed(S)), dtype=torch.float64, device=dev)
    a.uniform_(-1.0, 1.0)
    b = torch.zeros((f.nleaves(), args.nvars) + tuple(reversed(S)), dtype=torch.float64,
                    device=dev)
    t.run(a, b, args.nvars)
    ms = timed(lambda: t.run(a, b, args.nvars), max(3, args.steps // 2))
    pts = f.nleaves() * 16 ** 3 * args.nvars
    out = {"workload": f"sphere {args.roots}^3 roots, {args.levels} levels: {len(refine)} "
                       f"level-0 leaves refined, {len(fams)} finest families coarsened",
           "old_blocks": len(old), "new_blocks": f.nleaves(), "transfers": t.counts(),
           "ms": ms, "gbs": 2 * 8 * pts / (ms * 1e-3) / 1e9}
    del a, b, t
    torch.cuda.empty_cache()
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms.

    nvidia-smi takes a moment to start, longer than a short timed region, so
    ``wait_first`` runs the step (untimed) until the first sample is written,
    and ``hold`` keeps the GPU on the same step after the timed region until
    the window is long enough for several samples: every sample is taken
    under the timed work's load."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.path = None
        self.proc = None
        self.t0 = None
        self.before = 0
        self.held = 0

    def wait_first(self, fn, sync, timeout: float = 3.0, batch: int = 10):
        """Run ``fn`` in batches of ``batch`` until the first sample is written
        (or ``timeout`` seconds pass, or nvidia-smi is not running)."""
        t = time.time()
        while self.proc is not None and time.time() - t < timeout:
            if self.proc.poll() is not None:
                break
            try:
                if os.path.getsize(self.path) > 0:
                    break
            except OSError:
                pass
            for _ in range(batch):
                fn()
            sync()
            self.before += batch
        self.t0 = time.time()

    def hold(self, fn, sync, seconds: float = 1.0, batch: int = 10):
        """Run ``fn`` (the timed step, untimed here) in batches of ``batch``
        until ``seconds`` have passed since the load window started."""
        if self.proc is None:
            return
        if self.t0 is None:
            self.t0 = time.time()
        while time.time() - self.t0 < seconds:
            for _ in range(batch):
                fn()
            sync()
            self.held += batch

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        with os.fdopen(fd, "w") as out:  # the child keeps its own descriptor
            try:
                self.proc = subprocess.Popen(
                    ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits", "-lms", "200"],
                    stdout=out, stderr=subprocess.DEVNULL)
            except Exception:
                self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.path is None or not os.path.exists(self.path):
            if self.path is not None and os.path.exists(self.path):
                os.unlink(self.path)
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
               "reasons": sorted(reasons)}
        if self.before or self.held:
            out["window"] = (f"the timed region, with {self.before} of the same steps before it "
                             f"and {self.held} after it, untimed, holding its load while "
                             "nvidia-smi samples")
        return out


def dot_test(work, fill, adjoint, seed: int) -> dict:
    """<A x, y> = <x, A^T y> with x and y seeded uniform over the whole array:
    ``fill(work)`` applies A to ``work`` in place and ``adjoint(t)`` applies
    A^T to ``t`` in place.  Each inner product is summed in float64 chunks,
    the chunks summed exactly.  ``work`` keeps its contents."""
    import math
    import torch
    keep = work.clone()
    g = torch.Generator(device=work.device).manual_seed(seed)
    x = torch.empty_like(work).uniform_(-1.0, 1.0, generator=g)
    y = torch.empty_like(work).uniform_(-1.0, 1.0, generator=g)
    work.copy_(x)
    fill(work)
    aty = y.clone()
    adjoint(aty)

    def dot(a, b):
        a, b = a.reshape(-1), b.reshape(-1)
        step = 1 << 22
        return math.fsum(float(torch.dot(a[i:i + step].double(), b[i:i + step].double()))
                         for i in range(0, a.numel(), step))
    lhs, rhs = dot(work, y), dot(x, aty)
    work.copy_(keep)
    bound = 1e-13 if work.dtype == torch.float64 else 1e-5
    return {"lhs": lhs, "rhs": rhs,
            "relative_residual": abs(lhs - rhs) / max(abs(lhs), abs(rhs)), "bound": bound}


def run_side(workloads: dict, name: str, world: int, fn, *args):
    """``workloads[name] = fn(*args)``.  On one GPU a side workload that raises
    records its error in the line instead of costing the headline; under
    torchrun it raises (a rank that skipped it would leave the others waiting
    in the next barrier)."""
    if world > 1:
        workloads[name] = fn(*args)
        return
    try:
        workloads[name] = fn(*args)
    except Exception as e:  # noqa: BLE001
        workloads[name] = {"error": f"{type(e).__name__}: {e}"}
        import torch
        if torch.cuda.is_available():
            torch.cuda.empty_cache()


def _split(a):
    """Veltkamp's split of float64 ``a`` into two halves of 26 bits."""
    c = 134217729.0 * a
    hi = c - (c - a)
    return hi, a - hi


def _two_prod(a, b):
    """``a * b`` as an unevaluated float64 sum, exactly (Dekker)."""
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    return p, ((ah * bh - p) + ah * bl + al * bh) + al * bl


def _two_sum(a, b):
    """``a + b`` as an unevaluated float64 sum, exactly (Knuth)."""
    s_ = a + b
    bb = s_ - a
    return s_, (a - (s_ - bb)) + (b - bb)


def fill_error(sched, inp, out, nvars, factors, per_group=2, seed=0):
    """The fill's deviation from a wider evaluation of the same stencils on
    the same data: a sample of up to ``per_group`` transfers of every group,
    all their points and variables, with the stored weights and the factor
    column.  Float32 results are checked against float64 sums (its products
    of Float32 values are exact); Float64 ones against double-double sums
    (products and sums by error-free transformations, about 106 bits).
    ``inp`` is the data the fill read (a filled array: every source a fill
    reads is a fixed point of it), ``out`` the result.  Returns the largest
    absolute deviation, and the largest in units of the last place, in the
    result's type, of the sum of the terms' magnitudes (a sum's rounding
    lives on that scale; a result near zero by cancellation has no last
    place of its own to measure against)."""
    dd = out.dtype == np.float64
    rng = np.random.default_rng(seed)
    D = sched.forest.D
    worst_abs, worst_ulp, n = 0.0, 0.0, 0
    for g in sched.groups:
        if getattr(g, "bounded", 0) or getattr(g, "orientation", 0) or g.stage < 1:
            continue
        nt = g.ntransfers()
        pick = rng.choice(nt, size=min(per_group, nt), replace=False)
        st = g.stencils
        tsl = tuple(slice(s_.targetfirst - 1, s_.targetfirst - 1 + s_.ntarget)
                    for s_ in reversed(st))
        fcol = (factors[:, g.factorcol - 1].astype(np.float64).reshape((nvars,) + (1,) * D)
                if g.factorcol else None)
        shape_t = (nvars,) + tuple(s_.ntarget for s_ in reversed(st))
        for t in pick:
            tb, sb = int(g.targetblocks[t]) - 1, int(g.sourceblocks[t]) - 1
            src = inp[sb].astype(np.float64)              # every variable at once
            hi = np.zeros(shape_t)
            lo = np.zeros(shape_t)
            mag = np.zeros(shape_t)
            # the tensor-product sum over each dimension's taps
            for taps in itertools.product(*[range(s_.order) for s_ in st]):
                wh = np.ones(shape_t[1:])
                wl = np.zeros(shape_t[1:])
                idx = []
                for d, s_ in enumerate(st):
                    shape = [1] * D
                    shape[D - 1 - d] = s_.ntarget
                    wd = s_.weights[taps[d], :].astype(np.float64).reshape(shape)
                    if dd:
                        ph, pl = _two_prod(wh, wd)
                        wh, wl = ph, pl + wl * wd
                    else:
                        wh = wh * wd
                    idx.append((s_.srcstart - 1 + taps[d]).astype(np.int64))
                u = src[(slice(None),) + np.ix_(*reversed(idx))]
                if dd:
                    th, tl = _two_prod(wh, u)
                    tl = tl + wl * u
                    s1, e1 = _two_sum(hi, th)
                    e1 = e1 + lo + tl
                    hi, lo = _two_sum(s1, e1)
                    mag = mag + np.abs(th)
                else:
                    term = wh * u
                    hi = hi + term
                    mag = mag + np.abs(term)
            if fcol is not None:
                hi, lo = hi * fcol, lo * fcol
            got = out[(tb, slice(None)) + tsl].astype(np.float64)
            dev = np.abs((got - hi) - lo)
            ulp = dev / np.spacing(mag.astype(out.dtype)).astype(np.float64)
            worst_abs = max(worst_abs, float(dev.max()))
            worst_ulp = max(worst_ulp, float(ulp.max()))
            n += hi.size
    return {"max_abs": worst_abs, "max_ulp_of_terms": worst_ulp, "points": n,
            "against": "double-double" if dd else "float64",
            "sample": f"up to {per_group} transfers of every copy, restriction and "
                      "prolongation group, every point and variable"}


def footprint_points(sched):
    """Per variable, the points a fill writes (every target, once) and the
    distinct points it reads (the union of every transfer's source windows,
    per source block)."""
    S = sched.stored
    nb = sched.forest.nleaves()
    wr = np.zeros((nb,) + tuple(reversed(S)), bool)
    rd = np.zeros_like(wr)
    for g in sched.groups:
        tbox, sbox = [], []
        for st in g.stencils:
            win = st.order // 2 if getattr(g, "bounded", 0) == 2 else st.order
            tbox.append(slice(st.targetfirst - 1, st.targetfirst - 1 + st.ntarget))
            sbox.append(slice(int(st.srcstart.min()) - 1, int(st.srcstart.max()) - 1 + win))
        tbox, sbox = tuple(reversed(tbox)), tuple(reversed(sbox))
        for t, src in zip(g.targetblocks, g.sourceblocks):
            wr[(int(t) - 1,) + tbox] = True
            rd[(int(src) - 1,) + sbox] = True
    return int(wr.sum()), int(rd.sum())


def sector_minimum(sched, nvars: int, esize: int, tag: int, stencils: bool = False,
                   unit: int = 32):
    """The least DRAM traffic of the unit copies of stage ``tag`` (with
    ``stencils``, of all its transfers, a stencil reading its whole source
    window) that the layout allows: every distinct ``unit``-byte sector they
    read fetched once, every sector they write stored once, and (with
    read-modify-write) every partly written sector fetched once too.  Per
    variable plane, in bytes."""
    S1, S2, S3 = (tuple(sched.stored) + (1, 1))[:3]
    vol = S1 * S2 * S3
    groups = [g for g in sched.groups if g.stage == tag and (g.unit() or stencils)]
    rd_s = wr_s = part_s = rp_s = 0
    alg = 0
    for v in range(nvars):
        rd, wr = [], []
        for g in groups:
            st = list(g.stencils) + [None] * (3 - len(g.stencils))
            tx = [np.arange(x.targetfirst - 1, x.targetfirst - 1 + x.ntarget) if x else
                  np.zeros(1, np.int64) for x in st]
            if g.unit():
                sx = [np.asarray(x.srcstart, np.int64) - 1 if x else np.zeros(1, np.int64)
                      for x in st]
            else:  # the window every column of the group reads
                sx = [np.arange(int(x.srcstart.min()) - 1, int(x.srcstart.max()) - 1 + x.order)
                      if x else np.zeros(1, np.int64) for x in st]
            toff = (tx[2][:, None, None] * S2 + tx[1][None, :, None]) * S1 + tx[0][None, None, :]
            soff = (sx[2][:, None, None] * S2 + sx[1][None, :, None]) * S1 + sx[0][None, None, :]
            tb = np.asarray(g.targetblocks, np.int64) - 1
            sb = np.asarray(g.sourceblocks, np.int64) - 1
            wr.append(((tb[:, None] * nvars + v) * vol + toff.ravel()[None, :]).ravel())
            rd.append(((sb[:, None] * nvars + v) * vol + soff.ravel()[None, :]).ravel())
        if not wr:
            break
        w = np.concatenate(wr) * esize
        r = np.concatenate(rd) * esize
        alg += 2 * w.size * esize              # a read and a write per point written
        ws, wc = np.unique(w // unit, return_counts=True)
        rs = np.unique(r // unit)
        partial = ws[wc < unit // esize]
        wr_s += ws.size
        rd_s += rs.size
        part_s += partial.size
        rp_s += np.union1d(rs, partial).size
    return {"stage": tag, "groups": len(groups), "unit_bytes": unit, "algorithmic_bytes": alg,
            "sectors_read_bytes": rd_s * unit, "sectors_written_bytes": wr_s * unit,
            "partly_written_bytes": part_s * unit,
            "minimum_bytes": (rd_s + wr_s) * unit,
            "minimum_bytes_with_rmw": (rp_s + wr_s) * unit}


def cpu_fill_rate(sched, fs_host_work, nvars, factors, bytes_per_fill, budget_s=15.0,
                  max_runs=5):
    """The oracle's threaded fill on every host core: (GB/s, seconds per
    fill, runs, threads)."""
    import oracle
    threads = os.cpu_count() or 1
    work = fs_host_work
    oracle.fill(sched, work, nvars, factors, nthreads=threads)          # warm-up
    times = []
    t_all = time.perf_counter()
    while len(times) < max_runs and (time.perf_counter() - t_all) < budget_s:
        t0 = time.perf_counter()
        oracle.fill(sched, work, nvars, factors, nthreads=threads)
        times.append(time.perf_counter() - t0)
    best = min(times)
    return bytes_per_fill / best / 1e9, best, len(times), threads


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def kernel_rooflines(sched, stage_ms, stage_bytes, peak):
    """The HBM roofline of each fused kernel over the stages that run it
    alone: the copy kernel over the stages that hold only unit copies, the
    stencil kernel over those that hold only stencils (a stage with both runs
    the two side by side and is left out)."""
    import statistics
    kinds = {}
    for g in sched.groups:
        kinds.setdefault(g.stage, set()).add("copy" if g.unit() else "stencil")
    out = {}
    for name, kind in (("fused_copy_kernel", "copy"), ("fused_stage_kernel", "stencil")):
        tags = [t for t, k in kinds.items() if k == {kind} and t in stage_ms]
        if not tags:
            continue
        ms = sum(statistics.mean(stage_ms[t]) for t in tags)
        b = sum(stage_bytes[t] for t in tags)
        out[name] = {"stages": sorted(tags), "ms": ms, "algorithmic_bytes": b,
                     "achieved": b / (ms * 1e-3) / 1e9, "frac": b / (ms * 1e-3) / 1e9 / peak}
    return out


def stage_times(ds, fs, sched, stream, dev, reps):
    """Per stage tag, the fused launches' times (CUDA events on the launching
    stream, ``reps`` fills' worth), and the algorithmic bytes of the stage."""
    import torch
    tags = sorted({gr.stage for gr in sched.groups})
    esize = fs.T.itemsize
    stage_bytes = {tag: 2 * esize * fs.nvars * sum(int(np.prod(gr.boxsize())) * gr.ntransfers()
                                                  for gr in sched.groups if gr.stage == tag)
                   for tag in tags}
    evs = []
    torch.cuda.synchronize(dev)
    for _ in range(reps):
        for tag in tags:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ds.run(fs, tag, tag, "fused")
            b.record(stream)
            evs.append((tag, a, b))
    torch.cuda.synchronize(dev)
    stage_ms = {}
    for tag, a, b in evs:
        stage_ms.setdefault(tag, []).append(a.elapsed_time(b))
    return stage_ms, stage_bytes


def measure_sphere(dev, timed, args, peak, world):
    """The sphere mesh with its stated data: 3-D, 8^3 periodic roots, N=16,
    G=3, cell-centred, 4 Float64 variables, PV(4,4), three levels around
    |x - 1/2| = 0.25, filled with sin(2 pi x) sin(2 pi y) sin(2 pi z) plus
    seeded noise of 1e-3.  Fused (autotuned) and plain fills, the per-stage
    HBM and FP64 rooflines, the fill's stated error, and the state vector's
    copies (scatter!/gather!) on the same mesh."""
    import torch
    from treeamr import FieldSet, GhostSchedule, Operators, fill_ghosts, meshes
    from treeamr.autotune import autotune
    from treeamr.ghosts import device_schedule
    f = meshes.sphere_forest(roots=args.roots, N=16, levels=args.levels)
    fs = FieldSet(f, 4, G=3, T=np.float64, device=dev)
    meshes.config_fill(fs, "sphere", seed=1)
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    nvars = fs.nvars
    bytes_per_fill = 2 * sched.ghost_items(nvars) * 8
    if args.options:
        ds0 = device_schedule(sched, dev.index)
        for kv in args.options.split(","):
            k, v = kv.split("=")
            ds0.set_option(k.strip(), int(v))
        tuned = ds0.options()
    else:
        tuned = autotune(fs, sched)
    for _ in range(args.warmup):
        fill_ghosts(fs, sched)
    steps = max(3, args.steps // 2)
    ms = timed(lambda: fill_ghosts(fs, sched), steps)
    filled = fs.work.cpu().numpy()
    error = fill_error(sched, filled, filled, nvars, fs.factors_host)
    del filled
    fill_ghosts(fs, sched, method="plain")
    ms_plain = timed(lambda: fill_ghosts(fs, sched, method="plain"), max(3, steps // 2))
    ds = device_schedule(sched, dev.index)
    stream = torch.cuda.current_stream(dev)
    stage_ms, stage_bytes = stage_times(ds, fs, sched, stream, dev, 3)
    kern_ms = sum(statistics.mean(v) for v in stage_ms.values())
    achieved = sum(stage_bytes.values()) / (kern_ms * 1e-3) / 1e9
    fp64 = fp64_roofline(stencil_flops(sched, nvars), stage_ms, args.fp64_peak) \
        if args.fp64_peak else None
    # the state vector's copies and one right-hand side's scatter + fill
    from treeamr.state import gather, scatter, scatter_fill, statevector
    u = statevector(fs)
    gather(u, fs)
    state_bytes = 2 * u.numel() * u.element_size()
    ms_scatter = timed(lambda: scatter(fs, u), steps)
    ms_gather = timed(lambda: gather(u, fs), steps)
    ms_sf = timed(lambda: scatter_fill(fs, sched, u), steps)
    state = {"entries": u.numel(), "bytes_per_copy": state_bytes,
             "scatter_ms": ms_scatter, "gather_ms": ms_gather,
             "scatter_gbs": state_bytes / (ms_scatter * 1e-3) / 1e9,
             "gather_gbs": state_bytes / (ms_gather * 1e-3) / 1e9,
             "scatter_frac_of_hbm": state_bytes / (ms_scatter * 1e-3) / 1e9 / peak,
             "scatter_fill_ms": ms_sf}
    del u
    wr, rd = footprint_points(sched)
    out = {
        "workload": "sphere: 3-D 8^3 periodic roots, N=16, G=3, cell, 4 vars F64, PV(4,4), "
                    "3 levels nested around |x-1/2|=0.25",
        "data": "sin(2 pi x) sin(2 pi y) sin(2 pi z) + seeded 1e-3 U[-1,1]",
        "dtype": "float64", "blocks": f.nleaves(), "groups": len(sched.groups),
        "field_bytes": fs.work.numel() * 8,
        "value": world * bytes_per_fill / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms,
        "plain": {"value": world * bytes_per_fill / (ms_plain * 1e-3) / 1e9,
                  "ms_per_step": ms_plain, "speedup_fused_vs_plain": ms_plain / ms},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "stage_ms": {str(k): statistics.mean(v) for k, v in stage_ms.items()},
                     "stage_bytes": {str(k): v for k, v in stage_bytes.items()},
                     "kernels": kernel_rooflines(sched, stage_ms, stage_bytes, peak)},
        "fp64": fp64,
        "error": error,
        "footprint": {"written_points": wr, "read_points": rd,
                      "bytes": (wr + rd) * nvars * 8},
        "ghost_points_per_s": sched.ghost_items(1) / (ms * 1e-3),
        "state": state,
        "tuned": tuned,
        "gpu_launches_per_fill": fused_launches(sched, ds),
    }
    del fs, sched, ds
    torch.cuda.empty_cache()
    return out


def measure_adjoint_sphere(dev, timed, args):
    """The adjoint's workload: the sphere mesh with 2 Float64 variables.  The
    transposed fill's time against the forward fill's on the same field set,
    and the dot-product test <A x, y> = <x, A^T y> with seeded uniform x, y
    (each inner product summed in float64 chunks, the chunks summed exactly)."""
    import math
    import torch
    from treeamr import FieldSet, GhostSchedule, Operators, fill_ghosts, meshes
    from treeamr.adjoint import fill_ghosts_adjoint
    from treeamr.autotune import autotune
    f = meshes.sphere_forest(roots=args.roots, N=16, levels=args.levels)
    fs = FieldSet(f, 2, G=3, T=np.float64, device=dev)
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    g = torch.Generator(device=dev).manual_seed(21)
    x = torch.empty_like(fs.work).uniform_(-1.0, 1.0, generator=g)
    y = torch.empty_like(fs.work).uniform_(-1.0, 1.0, generator=g)
    fs.work.copy_(x)
    autotune(fs, sched)
    fs.work.copy_(x)
    fill_ghosts(fs, sched)
    aty = y.clone()
    fill_ghosts_adjoint(fs, sched, aty)                    # prepares the transpose

    def dot(a, b):
        a, b = a.reshape(-1), b.reshape(-1)
        step = 1 << 22
        return math.fsum(float(torch.dot(a[i:i + step], b[i:i + step]))
                         for i in range(0, a.numel(), step))
    lhs, rhs = dot(fs.work, y), dot(x, aty)
    steps = max(3, args.steps // 2)
    work = fs.work.clone()
    ms_fwd = timed(lambda: fill_ghosts(fs, sched), steps)
    ms_adj = timed(lambda: fill_ghosts_adjoint(fs, sched, work), steps)
    bytes_per_fill = 2 * sched.ghost_items(fs.nvars) * 8
    out = {"workload": "sphere (8^3 periodic roots, N=16, G=3, 3 levels), 2 vars F64, PV(4,4)",
           "forward_ms": ms_fwd, "adjoint_ms": ms_adj, "time_vs_forward": ms_adj / ms_fwd,
           "value": bytes_per_fill / (ms_adj * 1e-3) / 1e9, "unit": UNIT,
           "dot_test": {"lhs": lhs, "rhs": rhs,
                        "relative_residual": abs(lhs - rhs) / max(abs(lhs), abs(rhs)),
                        "bound": 1e-13}}
    del fs, sched, x, y, aty, work
    torch.cuda.empty_cache()
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        return run_reference(args)

    if args.sector_minimum is not None:
        from treeamr import GhostSchedule, meshes
        T = np.dtype(args.dtype).type
        f, fs, ops = meshes.walls_setup(T=T, roots=args.roots, levels=args.walls_levels)
        sched = GhostSchedule(fs, ops)
        esize = np.dtype(T).itemsize
        if args.sector_minimum == "all":
            tags = sorted({g.stage for g in sched.groups})
            per = [sector_minimum(sched, fs.nvars, esize, t, stencils=True,
                                  unit=args.sector_unit) for t in tags]
            alg = sum(p["algorithmic_bytes"] for p in per)
            least = sum(p["minimum_bytes_with_rmw"] for p in per)
            out = {"stages": per, "algorithmic_bytes": alg, "minimum_bytes_with_rmw": least,
                   "ceiling_frac_of_peak": alg / least}
        else:
            out = sector_minimum(sched, fs.nvars, esize, int(args.sector_minimum),
                                 unit=args.sector_unit)
        out.update({"roots": args.roots, "dtype": args.dtype, "blocks": f.nleaves(),
                    "levels": args.walls_levels})
        print(json.dumps(out), flush=True)
        return 0

    import torch
    import torch.distributed as dist
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    from treeamr import GhostSchedule, fill_ghosts, meshes
    from treeamr.ghosts import device_schedule

    peaks = load_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            dist.barrier()

    def timed(fn, steps):
        torch.cuda.synchronize(dev)
        barrier()
        torch.cuda.synchronize(dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize(dev)
        barrier()
        return max_over_ranks(a.elapsed_time(b), world, dev) / steps

    if args.workload == "sphere":
        args.fp64_peak = None
        print(json.dumps(measure_sphere(dev, timed, args, peak, world)), flush=True)
        return 0
    if args.workload == "batch":
        print(json.dumps(measure_batch(dev, timed, args, peak)), flush=True)
        return 0

    # ---- the headline: the walls mesh (vertex-centred, reflecting low and
    # outflow high faces, stages P and 0), its stated data
    T = np.dtype(args.dtype).type
    esize = np.dtype(T).itemsize
    f, fs, ops = meshes.walls_setup(device=dev, T=T, roots=args.roots, levels=args.walls_levels)
    meshes.config_fill(fs, "walls", seed=3 + rank)
    sched = GhostSchedule(fs, ops)
    nvars = fs.nvars
    points = sched.ghost_items(nvars)
    bytes_per_fill = 2 * points * esize                # one read + one write per point-variable
    field_bytes = fs.work.numel() * esize
    ds = device_schedule(sched, dev.index)
    cfg = {"workload": "walls: 3-D vertex, 8^3 roots, N=32, G=2, reflecting low / outflow high "
                       f"faces, 5 levels around 2 seeded points, 8 vars (5 even, 3 odd) "
                       f"{'F64' if esize == 8 else 'F32'}, PV(4,4)"
           if (args.roots, args.walls_levels) == (8, 5) else
           f"walls: {args.roots}^3 roots, {args.walls_levels} levels",
           "blocks": f.nleaves(), "groups": len(sched.groups),
           "ghost_points_per_var": int(sched.ghost_items(1)), "nvars": nvars,
           "field_bytes": field_bytes,
           "l2": f"inputs larger than L2 ({field_bytes / 1e9:.1f} GB field data vs 129 MB L2); "
                 "no flush"}
    method = args.method
    if method == "fused" and args.options:
        for kv in args.options.split(","):
            k, v = kv.split("=")
            ds.set_option(k.strip(), int(v))
        cfg["options"] = ds.options()
    elif method == "fused":
        from treeamr.autotune import autotune
        cfg["tuned"] = autotune(fs, sched)
        meshes.config_fill(fs, "walls", seed=3 + rank)
    for _ in range(args.warmup):
        fill_ghosts(fs, sched, method=method)
    with ClockSampler(dev.index) as clk:
        step = lambda: fill_ghosts(fs, sched, method=method)  # noqa: E731
        sync = lambda: torch.cuda.synchronize(dev)  # noqa: E731
        clk.wait_first(step, sync)
        ms = timed(step, args.steps)
        clk.hold(step, sync)
    clocks = clk.summary()
    value = world * bytes_per_fill / (ms * 1e-3) / 1e9
    filled = fs.work.cpu().numpy() if rank == 0 else None
    error = fill_error(sched, filled, filled, nvars, fs.factors_host) if rank == 0 else None
    del filled

    # the plain one-launch-per-group fill on the same data
    fill_ghosts(fs, sched, method="plain")
    ms_plain = timed(lambda: fill_ghosts(fs, sched, method="plain"), max(3, args.steps // 2))

    # the adjoint of the same fill
    from treeamr.adjoint import fill_ghosts_adjoint
    yadj = fs.work.clone()
    fill_ghosts_adjoint(fs, sched, yadj)
    ms_adj = timed(lambda: fill_ghosts_adjoint(fs, sched, yadj), max(3, args.steps // 2))
    # and stage by stage (the transposes run in reverse stage order)
    adj_evs = []
    for _ in range(3):
        for tag in sorted({g.stage for g in sched.groups}, reverse=True):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ds.run_adjoint(yadj, nvars, fs.factors, tag, tag, stream)
            b.record(stream)
            adj_evs.append((tag, a, b))
    torch.cuda.synchronize(dev)
    adj_stage_ms = {}
    for tag, a, b in adj_evs:
        adj_stage_ms.setdefault(str(tag), []).append(a.elapsed_time(b))
    adj_stage_ms = {k: statistics.mean(v) for k, v in adj_stage_ms.items()}
    del yadj
    # and its dot-product test at full size (the field data kept)
    try:
        adj_dot = dot_test(fs.work, lambda t: fill_ghosts(fs, sched, method=method),
                           lambda t: fill_ghosts_adjoint(fs, sched, t), 22)
    except Exception as e:  # noqa: BLE001
        adj_dot = {"error": f"{type(e).__name__}: {e}"}
    torch.cuda.empty_cache()

    stage_ms, stage_bytes = stage_times(ds, fs, sched, stream, dev, max(3, args.steps // 2))
    kern_ms = sum(statistics.mean(v) for v in stage_ms.values())
    achieved = sum(stage_bytes.values()) / (kern_ms * 1e-3) / 1e9
    args.fp64_peak = None if (args.no_fp64_peak or esize != 8) else fp64_peak_tflops(dev)
    fp64 = fp64_roofline(stencil_flops(sched, nvars), stage_ms, args.fp64_peak) \
        if args.fp64_peak else None
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "walls_fill_traffic.json")))
        traffic = prof.get("traffic_bytes_per_fill_" + np.dtype(T).name)
    except Exception:
        pass

    # end to end through the C ABI from page-locked host buffers
    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(fs, sched, timed, stream, args, world, bytes_per_fill, field_bytes)

    # the other workloads, each on its own mesh
    host_data = fs.work.cpu().numpy() if (not args.no_cpu and rank == 0) else None
    factors_host = fs.factors_host
    workloads = {}
    if not args.no_walls:
        del fs
        torch.cuda.empty_cache()
        run_side(workloads, "sphere_float64", world, measure_sphere, dev, timed, args, peak,
                 world)
        run_side(workloads, "adjoint_sphere_2vars", world, measure_adjoint_sphere, dev, timed,
                 args)
        other = np.float32 if esize == 8 else np.float64
        run_side(workloads, "walls_" + np.dtype(other).name, world, measure_walls, other, dev,
                 timed, args, peak)
        run_side(workloads, "batch64_float32", world, measure_batch, dev, timed, args, peak)
        run_side(workloads, "boundary_hook", world, measure_hook, dev, timed, args)
        run_side(workloads, "regrid", world, measure_regrid, dev, timed, args)
        run_side(workloads, "sphere_pv6", world, measure_pv6, dev, timed, args)

    cpu = None
    if host_data is not None:
        gbs, best, runs, threads = cpu_fill_rate(sched, host_data, nvars, factors_host,
                                                 bytes_per_fill)
        cpu = {"value": gbs, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"whole fills of the same mesh and data, best of {runs} after one "
                         f"warm-up ({best:.3f} s a fill), oracle/fill_oracle.c with "
                         f"{threads} OpenMP threads"}

    if rank == 0:
        wr, rd = footprint_points(sched)
        fp_bytes = (wr + rd) * nvars * esize
        throughput = {
            "ghost_points_per_s": world * sched.ghost_items(1) / (ms * 1e-3),
            "ghost_point_variables_per_s": world * points / (ms * 1e-3),
            "footprint": {"written_points": wr, "read_points": rd, "bytes": fp_bytes,
                          "gbs": world * fp_bytes / (ms * 1e-3) / 1e9,
                          "frac": fp_bytes / (ms * 1e-3) / 1e9 / peak}}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if esize == 8 else "f32",
            "data": "synthetic: the walls mesh's stated data (Gaussian bumps of width 0.05 at "
                    "the 2 seeded refinement centres + seeded U[-1,1])",
            "config": dict(cfg, method=method, parallelism=f"replicas{world}"),
            "plain": {"value": world * bytes_per_fill / (ms_plain * 1e-3) / 1e9, "unit": UNIT,
                      "ms_per_step": ms_plain, "speedup_fused_vs_plain": ms_plain / ms},
            "adjoint": {"value": world * bytes_per_fill / (ms_adj * 1e-3) / 1e9, "unit": UNIT,
                        "ms_per_step": ms_adj, "time_vs_forward": ms_adj / ms,
                        "stage_ms": adj_stage_ms, "dot_test": adj_dot},
            "throughput": throughput,
            "error": error,
            "workloads": workloads,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum "
                                           "of every launch of one fill, captured on the walls "
                                           "mesh at 4^3 roots and scaled by the algorithmic "
                                           "bytes (profiles/walls_fill_traffic.json)"
                         if traffic else None,
                         "peak_source": peak_src,
                         "scope": "the whole fill: algorithmic bytes over the sum of the "
                                  "stages' fused launches (CUDA events)",
                         "stage_ms": {str(k): statistics.mean(v) for k, v in stage_ms.items()},
                         "stage_bytes": {str(k): v for k, v in stage_bytes.items()},
                         "kernels": kernel_rooflines(sched, stage_ms, stage_bytes, peak)},
            "fp64": fp64,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": args.steps * fused_launches(sched, ds) if method == "fused" else
            args.steps * len(sched.groups),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def measure_e2e(fs, sched, timed, stream, args, world, bytes_per_fill, field_bytes):
    """The fill of a host-resident field through the C ABI from page-locked
    host buffers, copies inside the timed region.

    - ``value``: three independent fills in flight (``HostPipeline``, each
      step's upload, fill and download on its own stream and device buffer),
      the own points uploaded (``tam_fill_host_own``).
    - ``dependent``: what a solver gets, each step's input the previous
      step's output, upload, fill and download on one stream, one after the
      other (``tam_fill_host_own``).
    - ``full_upload_ms_per_step``: the pipelined steps uploading the whole
      array (``tam_fill_host``)."""
    import torch
    from treeamr.host import HostPipeline
    host_in = torch.empty_like(fs.work, device="cpu").pin_memory()
    host_in.copy_(fs.work)
    host_out = [torch.empty_like(host_in).pin_memory() for _ in range(2)]
    own = not sched.boundaries
    e2e_steps = max(6, min(args.steps, 12))

    def e2e_pipeline(pipe):
        def run(n):
            pipe.wait_on(stream)
            for i in range(n):
                pipe.submit(host_in, host_out[i % 2])
            pipe.join(stream)
        run(3)
        return timed(lambda: run(e2e_steps), 1) / e2e_steps
    pipe = HostPipeline(fs, sched, depth=3)
    ms_full = e2e_pipeline(pipe)
    del pipe
    ms_e2e, h2d = ms_full, field_bytes
    if own:
        pipe = HostPipeline(fs, sched, depth=3, own=True)
        ms_e2e, h2d = e2e_pipeline(pipe), pipe.own_bytes()
        del pipe
    # dependent steps: the output of one is the input of the next
    pipe1 = HostPipeline(fs, sched, depth=1, own=own)
    a, b = host_out

    def chain(n):
        pipe1.wait_on(stream)
        src, dst = host_in, a
        for _ in range(n):
            pipe1.submit(src, dst)
            src, dst = dst, (b if dst is a else a)
        pipe1.join(stream)
    chain(2)
    dep_steps = 4
    ms_dep = timed(lambda: chain(dep_steps), 1) / dep_steps
    h2d_dep = pipe1.own_bytes() if own else field_bytes
    del pipe1
    out = {"value": world * bytes_per_fill / (ms_e2e * 1e-3) / 1e9, "unit": UNIT,
           "ms_per_step": ms_e2e, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": field_bytes, "steps": e2e_steps,
           "api": ("tam_fill_host_own (C ABI, page-locked host buffers: the own points up, "
                   "read by a kernel, the filled array down)" if own else
                   "tam_fill_host (C ABI, host buffers)") +
                  " through treeamr.host.HostPipeline, 3 independent steps in flight",
           "full_upload_ms_per_step": ms_full,
           "dependent": {"value": world * bytes_per_fill / (ms_dep * 1e-3) / 1e9, "unit": UNIT,
                         "ms_per_step": ms_dep, "steps": dep_steps,
                         "h2d_bytes_per_step": h2d_dep, "d2h_bytes_per_step": field_bytes,
                         "what": "each step's input is the previous step's output: upload, "
                                 "fill and download one after the other on one stream, what "
                                 "a time-stepping solver holding its state on the host gets"}}
    torch.cuda.empty_cache()
    # the host link's own rate
    dbuf = torch.empty_like(fs.work)
    s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()

    def link(up=True, down=True):
        s_up.wait_stream(stream)
        s_down.wait_stream(stream)
        if up:
            with torch.cuda.stream(s_up):
                dbuf.copy_(host_in, non_blocking=True)
        if down:
            with torch.cuda.stream(s_down):
                host_out[0].copy_(fs.work, non_blocking=True)
        stream.wait_stream(s_up)
        stream.wait_stream(s_down)
    link()
    ms_up = timed(lambda: link(down=False), 3)
    ms_down = timed(lambda: link(up=False), 3)
    ms_both = timed(link, 3)
    gb = field_bytes / 1e9
    floor = min(ms_up + ms_down, ms_both)
    out["host_link"] = {"h2d_gbs": gb / (ms_up * 1e-3), "d2h_gbs": gb / (ms_down * 1e-3),
                        "both_each_way_gbs": gb / (ms_both * 1e-3),
                        "serial_floor_ms": ms_up + ms_down, "concurrent_floor_ms": ms_both,
                        "floor_ms_per_step": floor, "frac": floor / ms_full}
    del dbuf, host_in, host_out
    torch.cuda.empty_cache()
    return out


def run_reference(args):
    """The CPU restatement of the reference's threaded fill (the oracle) on
    every host core, on the headline's walls mesh and data."""
    from treeamr import GhostSchedule, meshes
    import oracle
    T = np.dtype(args.dtype).type
    esize = np.dtype(T).itemsize
    f, fs, ops = meshes.walls_setup(T=T, roots=args.roots, levels=args.walls_levels)
    meshes.config_fill(fs, "walls", seed=3)
    sched = GhostSchedule(fs, ops)
    nvars = fs.nvars
    bytes_per_fill = 2 * sched.ghost_items(nvars) * esize
    cfg = {"workload": "walls: 3-D vertex, 8^3 roots, N=32, G=2, reflecting low / outflow high "
                       f"faces, 5 levels around 2 seeded points, 8 vars (5 even, 3 odd) "
                       f"{'F64' if esize == 8 else 'F32'}, PV(4,4)"
           if (args.roots, args.walls_levels) == (8, 5) else
           f"walls: {args.roots}^3 roots, {args.walls_levels} levels",
           "blocks": f.nleaves(), "groups": len(sched.groups),
           "ghost_points_per_var": int(sched.ghost_items(1)), "nvars": nvars,
           "field_bytes": fs.work.numel() * esize}
    host = fs.work.numpy()
    threads = os.cpu_count() or 1
    oracle.build()
    t0 = time.perf_counter()
    oracle.fill(sched, host, nvars, fs.factors_host, nthreads=threads)
    one = time.perf_counter() - t0
    warm = max(0, min(args.warmup - 1, int(20 / max(one, 1e-3))))
    for _ in range(warm):
        oracle.fill(sched, host, nvars, fs.factors_host, nthreads=threads)
    steps = max(1, min(args.steps, int(90 / max(one, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(steps):
        oracle.fill(sched, host, nvars, fs.factors_host, nthreads=threads)
    sec = (time.perf_counter() - t0) / steps
    value = bytes_per_fill / sec / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": steps, "steps_requested": args.steps, "warmup": warm + 1,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if esize == 8 else "f32",
        "data": "synthetic: the walls mesh's stated data (Gaussian bumps of width 0.05 at the "
                "2 seeded refinement centres + seeded U[-1,1])",
        "config": dict(cfg, method="cpu threaded fill", parallelism="host threads"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} whole fills after {warm + 1} warm-up, "
                                   "oracle/fill_oracle.c (the reference is Julia, absent here)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
