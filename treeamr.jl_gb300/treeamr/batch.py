"""Many independent forests filled together: ``ForestBatch``.

The reference fills one field set per call (``fill_ghosts!``,
``src/ghosts.jl:1783``).  A batch lays the field data of several field sets --
forests of any size and block extent, one element type and variable count --
out in one arena, 256-byte aligned member by member, and fills all of them
with one launch per stage (``tam_batch_fill``).  Each member's ``FieldSet``
keeps working on its own: its ``work`` is a view into the arena.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import torch

from . import _native
from .ghosts import check_fill, device_schedule
from .schedule import GhostSchedule
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
        ncols = 3 ** D
        self.arena = torch.zeros(max(total, 1), dtype=_TORCH[T], device=self.device)
        self.factor_arena = torch.zeros(len(fieldsets) * nvars * ncols, dtype=_TORCH[T],
                                        device=self.device)
        foffs = []
        for m, fs in enumerate(fieldsets):
            host = fs.work.detach().cpu()
            view = self.arena[offs[m]:offs[m] + fs.work.numel()].view(tuple(fs.work.shape))
            view.copy_(host)
            fs.work = view
            fo = m * nvars * ncols
            fview = self.factor_arena[fo:fo + nvars * ncols]
            fview.copy_(fs.factors.detach().cpu())
            fs.factors = fview
            foffs.append(fo)
        self.fieldsets = list(fieldsets)
        self.schedules = list(schedules)
        self.offsets = offs
        self.factor_offsets = foffs
        for fs, s in zip(fieldsets, schedules):
            check_fill(fs, s)
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

    def fill(self, arena: Optional[torch.Tensor] = None, stream=None):
        """Fill every member's ghosts; ``arena`` (default: the batch's own) is
        any tensor laid out like the batch's arena."""
        a = self.arena if arena is None else arena
        rc = self.lib.tam_batch_fill(self.handle, C.c_void_p(a.data_ptr()), a.numel(), self.nvars,
                                     C.c_void_p(self.factor_arena.data_ptr()),
                                     self.factor_arena.numel(), _native.TAM_STAGE_ALL_FIRST,
                                     _native.TAM_STAGE_ALL_LAST,
                                     C.c_void_p(self._stream(stream).cuda_stream))
        _native.check(rc, self.ctx, "tam_batch_fill")
        return a

    def fill_adjoint(self, y: torch.Tensor, stream=None):
        """``y <- A^T y`` for every member, ``y`` laid out like the arena."""
        rc = self.lib.tam_batch_fill_adjoint(
            self.handle, C.c_void_p(y.data_ptr()), y.numel(), self.nvars,
            C.c_void_p(self.factor_arena.data_ptr()), self.factor_arena.numel(),
            _native.TAM_STAGE_ALL_FIRST, _native.TAM_STAGE_ALL_LAST,
            C.c_void_p(self._stream(stream).cuda_stream))
        _native.check(rc, self.ctx, "tam_batch_fill_adjoint")
        return y

    def set_option(self, name: str, value: int):
        code = {"tile_items": 1, "threads": 2, "int_mul": 3, "one_tap": 4}[name]
        _native.check(self.lib.tam_batch_set_option(self.handle, code, int(value)), self.ctx,
                      f"tam_batch_set_option({name})")

    def member_view(self, arena: torch.Tensor, m: int) -> torch.Tensor:
        fs = self.fieldsets[m]
        o = self.offsets[m]
        return arena[o:o + fs.work.numel()].view(tuple(fs.work.shape))

    def ghost_points(self) -> int:
        return sum(s.ghost_items(self.nvars) for s in self.schedules)
