"""``fill_ghosts``: replay a GhostSchedule on the GPU through libtreeamr_cuda.so.

Mirrors the reference's entry point ``fill_ghosts!(fs, schedule; boundary)``
(``src/ghosts.jl:1783-1794``) with its checks (``check_fill``,
``src/ghosts.jl:2058-2101``) and stage order (``exchange_ghosts!``,
``src/ghosts.jl:1099-1160``): stage W (a hook that prescribes the wall
planes), stage P, stage 0, phase 1, the boundary hook, then the
prolongations coarsest target level first.  The stages run on the
device; only the hook, when one is given, runs between two library calls.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Optional

import numpy as np
import torch

from . import _native
from .schedule import GhostSchedule, PHASE1_TAG
from .storage import FieldSet

METHODS = ("fused", "plain")


class DeviceSchedule:
    """A schedule uploaded to one device (``tam_schedule_upload``).  Freed
    with the object."""

    def __init__(self, schedule: GhostSchedule, device: int):
        self.lib = _native.lib()
        self.ctx = _native.context(device)
        self.desc = _native.Descriptor(schedule)
        handle = C.c_void_p()
        _native.check(self.lib.tam_schedule_upload(self.ctx, self.desc.ref(), C.byref(handle)),
                      self.ctx, "tam_schedule_upload")
        self.handle = handle
        self.device = device
        ng, nt, pts = C.c_int64(), C.c_int64(), C.c_int64()
        ns = C.c_int32()
        self.lib.tam_schedule_info(handle, C.byref(ng), C.byref(nt), C.byref(pts), C.byref(ns))
        self.ngroups, self.ntransfers, self.points, self.nstages = ng.value, nt.value, pts.value, ns.value

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.tam_schedule_free(h)
            except Exception:
                pass
            self.handle = None

    def run(self, fs: FieldSet, first: int, last: int, method: str = "fused",
            stream: Optional[torch.cuda.Stream] = None, alt: Optional[torch.Tensor] = None,
            factors: Optional[torch.Tensor] = None, rotvars: Optional[torch.Tensor] = None):
        """Stages ``[first, last]`` on ``fs.work``; a RotationPair member's
        fill passes the pair's tables and its partner's array ``alt``."""
        s = stream if stream is not None else torch.cuda.current_stream(fs.work.device)
        if rotvars is None:
            rotvars = getattr(fs, "rotvars", None)
        if factors is None:
            factors = fs.factors
        if rotvars is not None or alt is not None:
            # turned transfers across a seam read the variable table, and an
            # odd orientation the alternate array (tam_fill_ex)
            rc = self.lib.tam_fill_ex(
                self.handle, C.c_void_p(fs.work.data_ptr()),
                C.c_void_p(alt.data_ptr() if alt is not None else 0), fs.nvars, fs.nblocks(),
                C.c_void_p(factors.data_ptr()),
                C.c_void_p(rotvars.data_ptr() if rotvars is not None else 0), first, last,
                _native.TAM_METHOD_PLAIN if method == "plain" else _native.TAM_METHOD_FUSED,
                C.c_void_p(s.cuda_stream))
            _native.check(rc, self.ctx, f"tam_fill_ex ({method})")
            return
        fn = {"fused": self.lib.tam_fill, "plain": self.lib.tam_fill_plain}[method]
        rc = fn(self.handle, C.c_void_p(fs.work.data_ptr()), fs.nvars, fs.nblocks(),
                C.c_void_p(fs.factors.data_ptr()), first, last, C.c_void_p(s.cuda_stream))
        _native.check(rc, self.ctx, f"tam_fill ({method})")

    def run_adjoint(self, y: torch.Tensor, nvars: int, factors: torch.Tensor, first: int,
                    last: int, stream: Optional[torch.cuda.Stream] = None,
                    scratch: Optional[torch.Tensor] = None,
                    rotvars: Optional[torch.Tensor] = None,
                    alt: Optional[torch.Tensor] = None):
        """``y <- A^T y`` in place (``tam_fill_adjoint``), or with the caller's
        scratch tensor (``tam_fill_adjoint_scratch``); a schedule across a
        seam passes the variable table (``tam_fill_adjoint_ex``), and a
        RotationPair member its partner's cotangent ``alt``, onto which its
        odd turns' transposes add (``tam_fill_adjoint_alt``)."""
        s = stream if stream is not None else torch.cuda.current_stream(y.device)
        if rotvars is not None or alt is not None:
            rc = self.lib.tam_fill_adjoint_alt(
                self.handle, C.c_void_p(y.data_ptr()),
                C.c_void_p(alt.data_ptr() if alt is not None else 0), nvars, y.shape[0],
                C.c_void_p(factors.data_ptr()),
                C.c_void_p(rotvars.data_ptr() if rotvars is not None else 0), first, last,
                C.c_void_p(scratch.data_ptr() if scratch is not None else 0),
                0 if scratch is None else scratch.numel() * scratch.element_size(),
                C.c_void_p(s.cuda_stream))
            _native.check(rc, self.ctx, "tam_fill_adjoint_alt")
            return
        if scratch is None:
            rc = self.lib.tam_fill_adjoint(self.handle, C.c_void_p(y.data_ptr()), nvars,
                                           y.shape[0], C.c_void_p(factors.data_ptr()), first,
                                           last, C.c_void_p(s.cuda_stream))
        else:
            rc = self.lib.tam_fill_adjoint_scratch(
                self.handle, C.c_void_p(y.data_ptr()), nvars, y.shape[0],
                C.c_void_p(factors.data_ptr()), first, last, C.c_void_p(scratch.data_ptr()),
                scratch.numel() * scratch.element_size(), C.c_void_p(s.cuda_stream))
        _native.check(rc, self.ctx, "tam_fill_adjoint")

    def stage_groups(self):
        """(stage groups, stages they hold): consecutive prolongation stages a
        fill runs as one launch pair (``tam_schedule_stage_groups``)."""
        g, n = C.c_int32(), C.c_int32()
        _native.check(self.lib.tam_schedule_stage_groups(self.handle, C.byref(g), C.byref(n)),
                      self.ctx, "tam_schedule_stage_groups")
        return g.value, n.value

    def adjoint_scratch_bytes(self, nvars: int) -> int:
        b = C.c_size_t()
        _native.check(self.lib.tam_adjoint_scratch_bytes(self.handle, nvars, C.byref(b)),
                      self.ctx, "tam_adjoint_scratch_bytes")
        return b.value

    # one_tap picks the form of the sum (1: the reference's CPU form, 0: its
    # device form; the same bits for finite data), the others speed only.
    OPTIONS = {"tile_items": 1, "threads": 2, "int_mul": 3, "one_tap": 4, "copy_points": 5,
               "block_order": 6, "path_tiles": 7, "merge_stages": 8,
               "staged": 9, "pair_vars": 10, "copy_share": 11,
               "soft_add": 12, "stencil_tile": 13}

    def set_option(self, name: str, value: int):
        _native.check(self.lib.tam_schedule_set_option(self.handle, self.OPTIONS[name], int(value)),
                      self.ctx, f"tam_schedule_set_option({name})")

    def get_option(self, name: str) -> int:
        v = C.c_int64()
        _native.check(self.lib.tam_schedule_get_option(self.handle, self.OPTIONS[name],
                                                       C.byref(v)), self.ctx,
                      f"tam_schedule_get_option({name})")
        return v.value

    def options(self):
        return {k: self.get_option(k) for k in self.OPTIONS}

    def status(self, fs: FieldSet) -> int:
        code = C.c_int32()
        s = torch.cuda.current_stream(fs.work.device)
        _native.check(self.lib.tam_device_status(self.handle, C.c_void_p(s.cuda_stream),
                                                 C.byref(code)), self.ctx, "tam_device_status")
        return code.value


def device_schedule(schedule: GhostSchedule, device: int) -> DeviceSchedule:
    """The schedule's upload to ``device``, made once and cached on it."""
    cache = schedule.__dict__.setdefault("_device", {})
    if device not in cache:
        cache[device] = DeviceSchedule(schedule, device)
    return cache[device]


def check_fill(fs: FieldSet, schedule: GhostSchedule, pair: bool = False):
    """The reference's refusals before any launch (``src/ghosts.jl:2058-2101``)."""
    if fs.forest is not schedule.forest:
        raise ValueError("the field set and the schedule are over different forests")
    if schedule.isstale():
        raise ValueError("the schedule is stale: the forest changed since it was built; "
                         "rebuild it (GhostSchedule(fs, ops))")
    if fs.generation != schedule.forest.generation:
        raise ValueError("the field set is stale: the forest changed since it was allocated")
    if fs.G != schedule.G:
        raise ValueError(f"the schedule was built for G={schedule.G}, the field set has G={fs.G}")
    if fs.centering != schedule.centering:
        raise ValueError(f"the schedule was built for centering {schedule.centering}, "
                         f"the field set has {fs.centering}")
    if fs.T != schedule.T:
        raise ValueError(f"the schedule was built for {schedule.T}, the field set holds {fs.T}")
    if schedule.selfimage and schedule.parities and fs.parities != schedule.parities:
        raise ValueError("the schedule's stage P was built for other variable parities than "
                         "the field set's; build the schedule from this field set")
    if fs.work.device.type != "cuda":
        raise ValueError("fill_ghosts runs on the GPU: the field set must live on a CUDA device")
    if getattr(schedule, "odd_turns", False) and not pair:
        from .storage import symmetric_layout
        if not symmetric_layout(fs.forest, fs.G, fs.c):
            raise ValueError(
                "this field set's layout is not symmetric in the rotating seam's dimensions "
                f"{fs.forest.rotating_dims()} (G = {fs.G}, centering {fs.centering}), so its "
                "ghosts across the seam are its partner's data, turned: fill it together with "
                "the set of the swapped layout as a RotationPair (src/ghosts.jl:1960-1980)")
    if getattr(schedule, "turned", False) and fs.rotvars is None and not pair:
        raise ValueError("this schedule turns ghosts across a seam, but the field set has no "
                         "variable table to turn them with: build it over the same forest, "
                         "with `rotation` (or `halfturn`)")


def turns_variables(fs: FieldSet) -> bool:
    """Whether the set's map across its forest's seam turns any variable:
    where it does not, the axis projection is the identity
    (``src/ghosts.jl:774-778``)."""
    m = fs.halfturn if fs.forest.ishalfturn() else fs.rotation
    return m is not None and list(m) != list(range(1, fs.nvars + 1))


def axis_transposed_tables(fs: FieldSet):
    """The tables of the axis projection's transpose.  The projection maps an
    axis point's variables ``u`` to ``(1/M) sum_r f[v, r] u[sigma_r(v)]``
    (``f[v, r]`` the factor at column ``3^D r``, ``sigma_r`` the variable
    table's column ``r``), so its transpose maps ``y`` to ``(1/M) sum_r
    f[sigma_r^-1(w), r] y[sigma_r^-1(w)]``: the same form, with column ``r``
    of the variable table inverted and each factor moved with its variable."""
    fac = np.asarray(fs.factors_host)
    rv = np.asarray(fs.rotvars_host)
    nvars, ncol = fs.nvars, 3 ** fs.D
    ft = np.zeros_like(fac)
    rt = np.empty_like(rv)
    for r in range(rv.shape[1]):
        sigma = rv[:, r].astype(np.int64) - 1
        if sorted(sigma.tolist()) != list(range(nvars)):
            raise ValueError(f"column {r} of the variable table is not a permutation, so the "
                             "axis projection has no transpose of its own form")
        for v in range(nvars):
            rt[sigma[v], r] = v + 1
            ft[sigma[v], ncol * r] = fac[v, ncol * r]
    return ft, rt


def run_axis(fs: FieldSet, schedule: GhostSchedule, stream=None, *,
             work: Optional[torch.Tensor] = None, transpose: bool = False):
    """A seam's axis projection on the device (``tam_axis_project``), stage
    P's axis part, between stage P and stage 0 (``src/ghosts.jl:1111-1116``),
    on ``work`` (default: the set's own array); ``transpose``: the
    projection's transpose, for the adjoint fill."""
    if not schedule.axis or not turns_variables(fs):
        return
    work = fs.work if work is None else work
    dev = work.device
    cache = schedule.__dict__.setdefault("_axis_device", {})
    key = (dev.index, fs.nvars, fs.T.name)
    if key not in cache:
        S = schedule.stored
        vol = int(np.prod(S))
        offs = []
        for b, idx in schedule.axis:
            o = 0
            for d in reversed(range(fs.D)):
                o = o * S[d] + (idx[d] - 1)
            offs.append(b * fs.nvars * vol + o)
        pts = torch.tensor(offs, dtype=torch.int64, device=dev)
        buf = torch.empty(len(offs) * fs.nvars, dtype=work.dtype, device=dev)
        cache[key] = (pts, buf, vol)
    pts, buf, vol = cache[key]
    if transpose:
        tcache = fs.__dict__.setdefault("_axis_transposed", {})
        if dev.index not in tcache:
            ft, rt = axis_transposed_tables(fs)
            col = lambda a: torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).to(dev)
            tcache[dev.index] = (col(ft), col(rt))
        factors, rotvars = tcache[dev.index]
    else:
        factors, rotvars = fs.factors, fs.rotvars
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    rc = _native.lib().tam_axis_project(
        _native.TAM_F64 if fs.T == np.float64 else _native.TAM_F32,
        C.c_void_p(pts.data_ptr()), pts.numel(), len(schedule.axis_orbit),
        C.c_void_p(work.data_ptr()), fs.nvars, vol, C.c_void_p(factors.data_ptr()),
        3 ** fs.D, C.c_void_p(rotvars.data_ptr()), C.c_void_p(buf.data_ptr()),
        C.c_void_p(s.cuda_stream))
    if rc != 0:
        raise _native.TamError(f"tam_axis_project failed ({rc})")


def _runner(ds, fs, schedule, method, stream):
    """``ds.run`` over a stage range, with a seam's axis projection inserted
    between stage P and stage 0 where the range covers both."""
    from .schedule import SELFIMAGE_TAG, UNIFY_TAG

    def run(first, last):
        if schedule.axis and first <= SELFIMAGE_TAG and last >= UNIFY_TAG:
            ds.run(fs, first, SELFIMAGE_TAG, method, stream)
            run_axis(fs, schedule, stream)
            ds.run(fs, UNIFY_TAG, last, method, stream)
        else:
            ds.run(fs, first, last, method, stream)
    return run


def fill_pair(pair, schedules, *, boundary=None, method: str = "fused",
              stream: Optional[torch.cuda.Stream] = None):
    """``fill_ghosts!(pair, (sa, sb); boundary)`` (``src/ghosts.jl:2117-2180``):
    the two schedules' stages merged by (stage, member), each member's
    turned transfers of odd orientation reading its partner's array through
    the pair's tables; the hooks (one for both, or one each) after phase 1
    of both, before the prolongations."""
    from .storage import RotationPair
    if not isinstance(pair, RotationPair):
        raise TypeError("fill_pair takes a RotationPair")
    sa, sb = schedules
    if method not in METHODS:
        raise ValueError(f"method must be one of {METHODS}")
    a, b = pair.a, pair.b
    check_fill(a, sa, pair=True)
    check_fill(b, sb, pair=True)
    hooks = boundary if isinstance(boundary, tuple) else (boundary, boundary)
    members = [(a, sa, pair.afactors, pair.arotvars, b.work, hooks[0]),
               (b, sb, pair.bfactors, pair.brotvars, a.work, hooks[1])]
    dss = [device_schedule(s, x.work.device.index or 0) for x, s, *_ in members]
    tags = sorted(set(sa.stage_tags) | set(sb.stage_tags))

    def run(i, tag):
        fs, s, fac, rv, alt, _ = members[i]
        if tag in s.stage_tags:
            dss[i].run(fs, tag, tag, method, stream, alt=alt, factors=fac, rotvars=rv)
    for tag in [t for t in tags if t <= PHASE1_TAG]:
        run(0, tag)
        run(1, tag)
    for i in (0, 1):
        fs, s, *_, hook = members[i]
        if hook is None or not s.boundaries:
            continue
        from .boundary import CellBoundary
        if isinstance(hook, CellBoundary):
            hook.apply(fs, s, stream, slot=PHASE1_TAG) if hook.relative else \
                hook.apply(fs, s, stream)
        else:
            hook(fs, s.boundaries)
    for tag in [t for t in tags if t > PHASE1_TAG]:
        run(0, tag)
        run(1, tag)
    return pair


def fill_ghosts(fs: FieldSet, schedule: GhostSchedule, *, boundary: Optional[Callable] = None,
                method: str = "fused", stream: Optional[torch.cuda.Stream] = None) -> FieldSet:
    """Fill every ghost of ``fs`` from its neighbours (``fill_ghosts!``).

    ``boundary(fs, regions)`` fills the regions facing out through outer faces;
    it runs after phase 1 and before the prolongations, as the reference's
    hook does (``src/ghosts.jl:1129-1136``).  ``method`` picks the fused
    batched launch (default) or the plain one-launch-per-group replay.
    ``fill_ghosts(pair, (schedule_a, schedule_b))`` fills a RotationPair."""
    from .storage import RotationPair
    if isinstance(fs, RotationPair):
        return fill_pair(fs, schedule, boundary=boundary, method=method, stream=stream)
    if method not in METHODS:
        raise ValueError(f"method must be one of {METHODS}")
    check_fill(fs, schedule)
    ds = device_schedule(schedule, fs.work.device.index or 0)
    from .boundary import CellBoundary
    if isinstance(boundary, CellBoundary):
        # stage W: a hook that prescribes the wall planes writes their
        # primaries before stage P and stage 0 (src/ghosts.jl:1111-1113)
        boundary.apply_walls(fs, schedule, stream)
    run = _runner(ds, fs, schedule, method, stream)
    if boundary is None or not schedule.boundaries:
        run(_native.TAM_STAGE_ALL_FIRST, _native.TAM_STAGE_ALL_LAST)
        return fs
    if isinstance(boundary, CellBoundary) and boundary.relative:
        # the relative form in parts, each after the stage that fills the
        # ghosts it reads (src/ghosts.jl:1146-1160)
        run(_native.TAM_STAGE_ALL_FIRST, PHASE1_TAG)
        slots = set(boundary.slots(schedule))
        boundary.apply(fs, schedule, stream, slot=PHASE1_TAG)
        for tag in [t for t in schedule.stage_tags if t > PHASE1_TAG]:
            ds.run(fs, tag, tag, method, stream)
            if tag in slots:
                boundary.apply(fs, schedule, stream, slot=tag)
        return fs
    run(_native.TAM_STAGE_ALL_FIRST, PHASE1_TAG)
    if isinstance(boundary, CellBoundary):
        boundary.apply(fs, schedule, stream)        # the device hook
    else:
        boundary(fs, schedule.boundaries)           # the region form, on the host
    ds.run(fs, PHASE1_TAG + 1, _native.TAM_STAGE_ALL_LAST, method, stream)
    return fs


def boundary_by_coordinates(fn: Callable):
    """A hook that sets every outer-face ghost to ``fn(x, v)`` at its position
    (``src/ghosts.jl:1400-1440``, the form the reference's tests use)."""
    def hook(fs: FieldSet, regions):
        host = fs.work.detach().cpu().numpy()
        for r in regions:
            pos = fs.positions(r.block)
            axes = [pos[d][a - 1:z] for d, (a, z) in enumerate(r.region)]
            grids = np.meshgrid(*axes, indexing="ij")
            sl = tuple(slice(a - 1, z) for a, z in reversed(r.region))
            for v in range(fs.nvars):
                vals = np.broadcast_to(np.asarray(fn(tuple(grids), v), dtype=np.float64),
                                       grids[0].shape)
                host[(r.block, v) + sl] = vals.astype(fs.T).transpose()
        fs.work.copy_(torch.from_numpy(host).to(fs.work.device))
    return hook
