"""The regrid transfer (``src/regrid.jl:585-756, 942-955``): moving a field
set's own points from the leaves before a refinement or coarsening to the
leaves after.

Every new leaf takes its data from where they were: a kept leaf by a copy,
a created child by a prolongation from its parent, a coarsened parent by a
restriction from each of its children.  The transfers are the ghost fill's
with direction zero, grouped by ``(kind, child offset)`` under the same
``GroupKey`` and built by the same stencil builders, and they run through
the same kernels, reading the old array and writing the new one
(``tam_regrid_upload``, ``tam_regrid_transfer``).  The ghosts are left to
the next fill, as in the reference.  ``regrid`` wraps the serial
``regrid!`` of one field set: fill, move the forest, transfer, swap arrays.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native
from .forest import Forest, MortonKey, childoffset, parentkey, sortedchildkeys
from .schedule import (COPY, PROLONG, RESTRICT, GroupKey, TransferGroup, _nospan,
                       kind_stencil)
from .storage import FieldSet

REGRID_TAG = 50                     # the reference's stage tag of the transfer


def regrid_sources(oldleaves: Sequence[MortonKey], newleaves: Sequence[MortonKey]):
    """``GroupKey -> (targets, sources)``, 1-based new and old leaf indices,
    targets ascending (``src/regrid.jl:585-656``)."""
    index = {k: i for i, k in enumerate(oldleaves)}
    D = len(newleaves[0].coords) if newleaves else 1
    zero = (0,) * D
    nomirror = (0,) * D
    nospan = _nospan(D)
    pairs: Dict[GroupKey, Tuple[List[int], List[int]]] = {}

    def push(kind, offset, t, s):
        key = GroupKey(kind, zero, offset, 0, nomirror, nospan)
        tb, sb = pairs.setdefault(key, ([], []))
        tb.append(t + 1)
        sb.append(s + 1)

    for t, kn in enumerate(newleaves):
        same = index.get(kn)
        if same is not None:
            push(COPY, zero, t, same)
            continue
        parent = index.get(parentkey(kn)) if kn.level > 0 else None
        if parent is not None:
            push(PROLONG, childoffset(kn), t, parent)
            continue
        for kc in sortedchildkeys(kn):
            child = index.get(kc)
            if child is None:
                raise ValueError(f"cannot rebuild {kn}: neither it, its parent, nor its child "
                                 f"{kc} was a leaf before regridding. A single regrid may move "
                                 "a block by at most one level, which holds when the previous "
                                 "tree was 2:1 balanced.")
            push(RESTRICT, childoffset(kc), t, child)
    return pairs


class RegridTransfer:
    """The serial regrid transfer's groups (``transfer_groups``,
    ``src/regrid.jl:942-955``) for one layout: built from the old and new
    leaf arrays, uploaded once per device."""

    def __init__(self, forest: Forest, oldleaves: Sequence[MortonKey], G, centering, T,
                 operators):
        from .storage import ghostwidths, staggers
        D, N = forest.D, forest.N
        self.forest = forest                     # holds the new leaves
        self.generation = forest.generation
        self.G = ghostwidths(G, D)
        self.c = staggers(centering)
        self.centering = tuple(centering)
        self.T = np.dtype(T)
        self.stored = tuple(N + 2 * g + cd for g, cd in zip(self.G, self.c))
        self.nold = len(oldleaves)
        self.nnew = forest.nleaves()
        pairs = regrid_sources(list(oldleaves), forest.leaves)
        groups = []
        for key in sorted(pairs, key=GroupKey.order):
            tb, sb = pairs[key]
            st = tuple(kind_stencil(self.T, N, self.G[d], self.c[d], key.kind, 0, key.offset[d],
                                    operators) for d in range(D))
            groups.append(TransferGroup(key, st, tb, sb, 0, REGRID_TAG))
        self.groups = groups
        self._device = {}

    def all_groups(self):
        return list(self.groups)

    def counts(self):
        out = {COPY: 0, PROLONG: 0, RESTRICT: 0}
        for g in self.groups:
            out[g.kind] += g.ntransfers()
        return out

    def _upload(self, device: int):
        if device not in self._device:
            lib = _native.lib()
            ctx = _native.context(device)
            desc = _native.Descriptor(self)
            h = C.c_void_p()
            _native.check(lib.tam_regrid_upload(ctx, desc.ref(), self.nold, C.byref(h)), ctx,
                          "tam_regrid_upload")
            self._device[device] = (lib, ctx, desc, h)
        return self._device[device]

    def __del__(self):
        for lib, ctx, desc, h in getattr(self, "_device", {}).values():
            try:
                lib.tam_schedule_free(h)
            except Exception:
                pass

    def run(self, old_work: torch.Tensor, new_work: torch.Tensor, nvars: int,
            stream: Optional[torch.cuda.Stream] = None):
        """The transfer from ``old_work`` (old leaves) into ``new_work``'s own
        points (new leaves), on the device."""
        if old_work.device.type != "cuda" or new_work.device != old_work.device:
            raise ValueError("the old and new arrays must be on one CUDA device")
        if old_work.shape[0] != self.nold or new_work.shape[0] != self.nnew:
            raise ValueError("the arrays' block counts differ from the transfer's")
        lib, ctx, desc, h = self._upload(old_work.device.index or 0)
        s = stream if stream is not None else torch.cuda.current_stream(old_work.device)
        rc = lib.tam_regrid_transfer(h, C.c_void_p(old_work.data_ptr()), self.nold,
                                     C.c_void_p(new_work.data_ptr()), self.nnew, nvars,
                                     C.c_void_p(s.cuda_stream))
        _native.check(rc, ctx, "tam_regrid_transfer")


def regrid(fs: FieldSet, operators, *, refine: Sequence[MortonKey] = (),
           coarsen: Sequence[MortonKey] = (), schedule=None) -> RegridTransfer:
    """The serial ``regrid!`` of one field set (``src/regrid.jl:1269-1418``):
    fill its ghosts (the prolongations of created blocks read them), refine
    ``refine`` and coarsen ``coarsen`` (parents whose children are leaves),
    2:1 balance, move the own points to the new leaves, and give the field
    set the new array.  Returns the transfer, which the caller may replay."""
    from .ghosts import fill_ghosts
    from .schedule import GhostSchedule
    forest = fs.forest
    if schedule is None:
        schedule = GhostSchedule(fs, operators)
    fill_ghosts(fs, schedule)
    oldleaves = list(forest.leaves)
    if refine:
        forest.refine(list(refine))
    if coarsen:
        forest.coarsen(list(coarsen))
    forest.balance()
    t = RegridTransfer(forest, oldleaves, fs.G, fs.centering, fs.T, operators)
    new = torch.zeros((forest.nleaves(),) + tuple(fs.work.shape[1:]), dtype=fs.work.dtype,
                      device=fs.work.device)
    t.run(fs.work, new, fs.nvars)
    fs.work = new
    fs.generation = forest.generation
    return t
