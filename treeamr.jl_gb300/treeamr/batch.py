"""Many independent forests filled together: ``ForestBatch``.

The reference fills one field set per call (``fill_ghosts!``,
``src/ghosts.jl:1783``).  A batch lays the field data of several field sets --
forests of any size and block extent, one element type and variable count --
out in one arena, 256-byte aligned member by member, and fills all of them
with one launch per stage (``tam_batch_fill``).  Each member's ``FieldSet``
keeps working on its own: its ``work`` is a view into the arena.

Members may turn ghosts across a seam (sets symmetric in the seam's plane:
a RotationPair reads its partner's array and is filled as a pair) or bound
their prolongations; their solo groups run after each stage's fused
launches, one launch for all members.  Turned members share one variable
table, and a seam's axis projection runs between stage P and stage 0.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import torch

from . import _native
from .ghosts import check_fill, device_schedule, run_axis, turns_variables
from .schedule import GhostSchedule, SELFIMAGE_TAG, UNIFY_TAG
from .storage import FieldSet, _TORCH

ALIGN_BYTES = 256


class ForestBatch:
    def __init__(self, fieldsets: Sequence[FieldSet], schedules: Sequence[GhostSchedule],
                 device="cuda"):
        if len(fieldsets) != len(schedules) or not fieldsets:
            raise ValueError("a batch needs one schedule per field set, and at least one")
        T = fieldsets[0].T
        nvars = fieldsets[0].nvars
        D = fieldsets[0].D
        for fs, s in zip(fieldsets, schedules):
            if fs.T != T or fs.nvars != nvars or fs.D != D:
                raise ValueError("the field sets of a batch share element type, variable count "
                                 "and dimension")
        self.device = torch.device(device)
        self.T, self.nvars, self.D = T, nvars, D
        align = ALIGN_BYTES // T.itemsize
        offs, total = [], 0
        for fs in fieldsets:
            offs.append(total)
            n = fs.work.numel()
            total += (n + align - 1) // align * align
        # each member's factor table: nvars x 3^D, or nvars x 4 * 3^D over a seam
        fsizes = [fs.factors.numel() for fs in fieldsets]
        self.arena = torch.zeros(max(total, 1), dtype=_TORCH[T], device=self.device)
        self.factor_arena = torch.zeros(max(sum(fsizes), 1), dtype=_TORCH[T],
                                        device=self.device)
        foffs = []
        for m, fs in enumerate(fieldsets):
            host = fs.work.detach().cpu()
            view = self.arena[offs[m]:offs[m] + fs.work.numel()].view(tuple(fs.work.shape))
            view.copy_(host)
            fs.work = view
            fo = sum(fsizes[:m])
            fview = self.factor_arena[fo:fo + fsizes[m]]
            fview.copy_(fs.factors.detach().cpu())
            fs.factors = fview
            foffs.append(fo)
        self.fieldsets = list(fieldsets)
        self.schedules = list(schedules)
        self.offsets = offs
        self.factor_offsets = foffs
        for fs, s in zip(fieldsets, schedules):
            check_fill(fs, s)
        # the variable table of the turned members, which they share
        self.rotvars = None
        for fs, s in zip(fieldsets, schedules):
            if not getattr(s, "turned", False):
                continue
            rv = fs.rotvars.detach().cpu()
            if self.rotvars is None:
                self.rotvars = rv
            elif not torch.equal(self.rotvars, rv):
                raise ValueError("the turned members of a batch share one variable table: "
                                 "build their field sets with the same rotation")
        if self.rotvars is not None:
            self.rotvars = self.rotvars.to(torch.int32).to(self.device)
        for fs in fieldsets:  # the axis projection reads each member's own table
            if getattr(fs, "rotvars", None) is not None:
                fs.rotvars = fs.rotvars.to(self.device)
        # members whose seam axis is projected between stage P and stage 0
        self.axis_members = [m for m, (fs, s) in enumerate(zip(fieldsets, schedules))
                             if s.axis and turns_variables(fs)]
        dev = self.device.index or 0
        self.uploads = [device_schedule(s, dev) for s in schedules]
        self.lib = _native.lib()
        self.ctx = _native.context(dev)
        handles = (C.c_void_p * len(fieldsets))(*[u.handle.value for u in self.uploads])
        wo = (C.c_int64 * len(offs))(*offs)
        fo = (C.c_int64 * len(foffs))(*foffs)
        h = C.c_void_p()
        _native.check(self.lib.tam_batch_create(self.ctx, handles, len(fieldsets), wo, fo,
                                                C.byref(h)), self.ctx, "tam_batch_create")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.tam_batch_free(h)
            except Exception:
                pass
            self.handle = None

    def nstages(self) -> int:
        return len({g.stage for s in self.schedules for g in s.groups})

    def _stream(self, stream):
        return stream if stream is not None else torch.cuda.current_stream(self.device)

    def _run(self, name: str, a: torch.Tensor, first: int, last: int, stream):
        rv = self.rotvars
        rc = getattr(self.lib, name)(
            self.handle, C.c_void_p(a.data_ptr()), a.numel(), self.nvars,
            C.c_void_p(self.factor_arena.data_ptr()), self.factor_arena.numel(),
            C.c_void_p(rv.data_ptr() if rv is not None else 0), first, last,
            C.c_void_p(self._stream(stream).cuda_stream))
        _native.check(rc, self.ctx, name)

    def _axis(self, a: torch.Tensor, stream, transpose: bool):
        for m in self.axis_members:
            run_axis(self.fieldsets[m], self.schedules[m], self._stream(stream),
                     work=self.member_view(a, m), transpose=transpose)

    def fill(self, arena: Optional[torch.Tensor] = None, stream=None):
        """Fill every member's ghosts; ``arena`` (default: the batch's own) is
        any tensor laid out like the batch's arena."""
        a = self.arena if arena is None else arena
        first, last = _native.TAM_STAGE_ALL_FIRST, _native.TAM_STAGE_ALL_LAST
        if self.axis_members:
            self._run("tam_batch_fill_ex", a, first, SELFIMAGE_TAG, stream)
            self._axis(a, stream, transpose=False)
            first = UNIFY_TAG
        self._run("tam_batch_fill_ex", a, first, last, stream)
        return a

    def fill_adjoint(self, y: torch.Tensor, stream=None):
        """``y <- A^T y`` for every member, ``y`` laid out like the arena."""
        first, last = _native.TAM_STAGE_ALL_FIRST, _native.TAM_STAGE_ALL_LAST
        if self.axis_members:
            self._run("tam_batch_fill_adjoint_ex", y, UNIFY_TAG, last, stream)
            self._axis(y, stream, transpose=True)
            last = SELFIMAGE_TAG
        self._run("tam_batch_fill_adjoint_ex", y, first, last, stream)
        return y

    def device_status(self, stream=None) -> int:
        """The solo launches' error word (nonzero: a variable table named no
        variable), read and cleared."""
        code = C.c_int32()
        _native.check(self.lib.tam_batch_device_status(
            self.handle, C.c_void_p(self._stream(stream).cuda_stream), C.byref(code)),
            self.ctx, "tam_batch_device_status")
        return code.value

    # the launch options a batch takes (TAM_OPT_*; the block order and stage
    # groups are a single schedule's)
    OPTIONS = {"tile_items": 1, "threads": 2, "int_mul": 3, "one_tap": 4, "copy_points": 5,
               "path_tiles": 7, "staged": 9, "pair_vars": 10,
               "copy_share": 11, "soft_add": 12, "stencil_tile": 13}

    def set_option(self, name: str, value: int):
        code = self.OPTIONS[name]
        _native.check(self.lib.tam_batch_set_option(self.handle, code, int(value)), self.ctx,
                      f"tam_batch_set_option({name})")
        self.options[name] = int(value)

    @property
    def options(self) -> dict:
        """The launch options set so far (the library's defaults until set)."""
        if "_options" not in self.__dict__:
            self._options = {"tile_items": 128, "threads": 256, "int_mul": 0, "one_tap": 1,
                             "copy_points": 1, "path_tiles": 1 if self.T.itemsize == 8 else 0,
                             "staged": 0, "pair_vars": 0, "copy_share": 0, "soft_add": 0,
                             "stencil_tile": 0}
        return self._options

    # the batch's tuning choices: every value of each, one option at a time
    TUNE = (("tile_items", (32, 64, 128, 256, 512)), ("threads", (128, 256, 512)),
            ("copy_points", (1, 2, 4)), ("copy_share", (0, 2, 4)), ("path_tiles", (0, 1)),
            ("stencil_tile", (0, 32, 64, 128)))

    def autotune(self, reps: int = 3, sweeps: int = 2) -> dict:
        """Pick the batch's launch options by timing whole fills (CUDA events,
        best of ``reps`` after a warm-up) one option at a time, ``sweeps``
        times over (for Float64 the integer-pipe multiply too).  The fills
        overwrite the arena's ghosts, never an own point; every choice gives
        the same bits.  Returns the options left set."""
        stream = torch.cuda.current_stream(self.device)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

        def timed() -> float:
            self.fill()
            best = float("inf")
            for _ in range(reps):
                start.record(stream)
                self.fill()
                end.record(stream)
                end.synchronize()
                best = min(best, start.elapsed_time(end))
            return best

        dims = list(self.TUNE)
        if self.T.itemsize == 8:
            dims += [("int_mul", (0, 1)), ("soft_add", (0, 1))]
        best = timed()
        for _ in range(sweeps):
            for name, values in dims:
                keep = self.options[name]
                for v in values:
                    if v == keep:
                        continue
                    self.set_option(name, v)
                    ms = timed()
                    if ms < best:
                        best, keep = ms, v
                self.set_option(name, keep)
        self.tuned_ms = best
        return dict(self.options)

    def member_view(self, arena: torch.Tensor, m: int) -> torch.Tensor:
        fs = self.fieldsets[m]
        o = self.offsets[m]
        return arena[o:o + fs.work.numel()].view(tuple(fs.work.shape))

    def ghost_points(self) -> int:
        return sum(s.ghost_items(self.nvars) for s in self.schedules)
