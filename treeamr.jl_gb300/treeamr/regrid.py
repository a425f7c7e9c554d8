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

A set with a vertex-like dimension takes a second stage, the
kept-over-created pass (``src/regrid.jl:788-905``): a created block's copy
of a point that a kept block holds at the finest level holding it takes
the kept block's value, so that the next fill's stage 0 cannot carry a
prolongated value over an evolved one.  Its transfers are same-level
copies of closed sub-pieces within the new array, uploaded as an ordinary
schedule and run by ``tam_fill`` over its stage tag alone.
"""
from __future__ import annotations

import ctypes as C
import itertools
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native
from .forest import Forest, MortonKey, childoffset, parentkey, sortedchildkeys
from .schedule import (COPY, PROLONG, RESTRICT, GroupKey, NeighbourTable, TransferGroup,
                       _nospan, copy_stencil, kind_stencil, merged_transfers, piece_copies,
                       piece_of, piece_primary, subpiece_list, subpiece_values)
from .forest import axismap
from .operators import boundedmode
from .storage import FieldSet, mirrorcolumn

REGRID_TAG = 50                     # the reference's stage tag of the transfer
REGRID_KEPT_TAG = 51                # and of its kept-over-created pass


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


def regrid_kept_pairs(forest: Forest, oldleaves: Sequence[MortonKey], c):
    """``GroupKey -> (targets, sources)`` of the kept-over-created pass, both
    1-based new leaf indices (``regrid_kept_pairs``, ``src/regrid.jl:826-881``).

    ``forest`` holds the new leaves.  For every created leaf with a kept
    neighbour of its own level across a face, edge or corner of a
    vertex-like dimension, every closed sub-piece but the open interior
    that the created leaf holds at the finest level holding it, and that a
    kept leaf of that level also holds, is copied from the kept holder that
    would be the primary among the kept holders; the sub-pieces merge into
    boxes per source as stage 0's do."""
    D = len(c)
    pairs: Dict[GroupKey, Tuple[List[int], List[int]]] = {}
    if not any(cd == 1 for cd in c):
        return pairs
    old = set(oldleaves)
    newleaves = forest.leaves
    kept = [k in old for k in newleaves]
    allowed = subpiece_values(c, forest.N)
    subs = subpiece_list(c, forest.N)
    steps = list(itertools.product(*[(-1, 0, 1) if cd == 1 else (0,) for cd in c]))
    nomirror = (0,) * D
    for j, k in enumerate(newleaves):
        if kept[j]:
            continue
        t = NeighbourTable(forest, j)
        found = False
        for delta in steps:
            if all(x == 0 for x in delta):
                continue
            lvl, nbrs = t.neighbours(delta)
            if lvl == t.level and any(kept[x[0]] for x in nbrs):
                found = True
                break
        if not found:
            continue
        entries = []
        for sub in subs:
            if all(x == 1 for x in piece_of(sub)):       # the open interior
                continue
            copies = piece_copies(t, sub, c)
            finest = max(x[0] for x in copies)
            if t.level != finest:
                continue
            holders = [x for x in copies if x[0] == finest and kept[x[1]]]
            if not holders:
                continue
            _, s, _, delta, o, r = piece_primary(holders)[:6]
            entries.append((sub, COPY, s, delta, o, r))
        for kind, s, delta, o, spans, r in merged_transfers(entries, allowed):
            key = GroupKey(kind, delta, o, 0, nomirror, spans, r)
            tb, sb = pairs.setdefault(key, ([], []))
            tb.append(j + 1)
            sb.append(s + 1)
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
            # a bounded operator bounds the regrid's children too
            # (src/regrid.jl:765-778)
            mode = boundedmode(operators, key.kind, key.mirror, self.c)
            st = tuple(kind_stencil(self.T, N, self.G[d], self.c[d], key.kind, 0, key.offset[d],
                                    operators, -1, mode) for d in range(D))
            groups.append(TransferGroup(key, st, tb, sb, 0, REGRID_TAG, None, mode))
        self.groups = groups
        kept = regrid_kept_pairs(forest, oldleaves, self.c)
        self.kept_groups = []
        for key in sorted(kept, key=GroupKey.order):
            tb, sb = kept[key]
            st = tuple(copy_stencil(self.T, N, self.G[d], self.c[d], key.direction[d],
                                    span=key.span[d]) for d in range(D))
            # across a seam the turned copy, with the turn's axis map and sign
            # column (src/regrid.jl:918-920)
            axes = axismap(key.orientation, *forest.seam_plane(), D) if key.orientation \
                else None
            fcol = mirrorcolumn((0,) * D) + 3 ** D * key.orientation if key.orientation else 0
            self.kept_groups.append(TransferGroup(key, st, tb, sb, fcol, REGRID_KEPT_TAG, axes))
        self._device = {}
        self._kept_device = {}

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

    def kept_counts(self):
        """The kept-over-created pass's transfers and points."""
        n = sum(g.ntransfers() for g in self.kept_groups)
        pts = sum(g.ntransfers() * int(np.prod(g.boxsize())) for g in self.kept_groups)
        return n, pts

    def _upload_kept(self, device: int):
        if device not in self._kept_device:
            lib = _native.lib()
            ctx = _native.context(device)
            desc = _native.Descriptor(self, groups=self.kept_groups)
            h = C.c_void_p()
            _native.check(lib.tam_schedule_upload(ctx, desc.ref(), C.byref(h)), ctx,
                          "tam_schedule_upload (kept-over-created pass)")
            self._kept_device[device] = (lib, ctx, desc, h)
        return self._kept_device[device]

    def __del__(self):
        for table in (getattr(self, "_device", {}), getattr(self, "_kept_device", {})):
            for lib, ctx, desc, h in table.values():
                try:
                    lib.tam_schedule_free(h)
                except Exception:
                    pass

    def run(self, old_work: torch.Tensor, new_work: torch.Tensor, nvars: int,
            stream: Optional[torch.cuda.Stream] = None, factors=None, rotvars=None):
        """The transfer from ``old_work`` (old leaves) into ``new_work``'s own
        points (new leaves), then the kept-over-created pass within
        ``new_work``, on the device."""
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
        if self.kept_groups:
            self.run_kept(new_work, nvars, stream=s, factors=factors, rotvars=rotvars)

    def run_kept(self, new_work: torch.Tensor, nvars: int,
                 stream: Optional[torch.cuda.Stream] = None, factors=None, rotvars=None):
        """The kept-over-created pass alone, within ``new_work``; a copy across
        a seam reads the field set's factor and variable tables."""
        if new_work.device.type != "cuda" or new_work.shape[0] != self.nnew:
            raise ValueError("the new array must be on a CUDA device and hold the new leaves")
        if not self.kept_groups:
            return
        lib, ctx, desc, h = self._upload_kept(new_work.device.index or 0)
        s = stream if stream is not None else torch.cuda.current_stream(new_work.device)
        if any(g.orientation for g in self.kept_groups):
            if factors is None or rotvars is None:
                raise ValueError("this regrid's kept-over-created pass turns copies across a "
                                 "seam: pass the field set's factors and rotvars")
            rc = lib.tam_fill_ex(h, C.c_void_p(new_work.data_ptr()), None, nvars, self.nnew,
                                 C.c_void_p(factors.data_ptr()), C.c_void_p(rotvars.data_ptr()),
                                 REGRID_KEPT_TAG, REGRID_KEPT_TAG, _native.TAM_METHOD_FUSED,
                                 C.c_void_p(s.cuda_stream))
        else:
            rc = lib.tam_fill(h, C.c_void_p(new_work.data_ptr()), nvars, self.nnew, None,
                              REGRID_KEPT_TAG, REGRID_KEPT_TAG, C.c_void_p(s.cuda_stream))
        _native.check(rc, ctx, "tam_fill (kept-over-created pass)")


def regrid(fs: FieldSet, operators, *, refine: Sequence[MortonKey] = (),
           coarsen: Sequence[MortonKey] = (), schedule=None, boundary=None) -> RegridTransfer:
    """The serial ``regrid!`` of one field set (``src/regrid.jl:1269-1418``):
    fill its ghosts (the prolongations of created blocks read them), refine
    ``refine`` and coarsen ``coarsen`` (parents whose children are leaves),
    2:1 balance, move the own points to the new leaves, and give the field
    set the new array.  ``boundary`` is the fill's hook, applied whole, as
    every fill applies it.  Returns the transfer, which the caller may
    replay."""
    from .ghosts import fill_ghosts
    from .schedule import GhostSchedule
    forest = fs.forest
    if schedule is None:
        schedule = GhostSchedule(fs, operators)
    fill_ghosts(fs, schedule, boundary=boundary)
    oldleaves = list(forest.leaves)
    if refine:
        forest.refine(list(refine))
    if coarsen:
        forest.coarsen(list(coarsen))
    forest.balance()
    t = RegridTransfer(forest, oldleaves, fs.G, fs.centering, fs.T, operators)
    new = torch.zeros((forest.nleaves(),) + tuple(fs.work.shape[1:]), dtype=fs.work.dtype,
                      device=fs.work.device)
    t.run(fs.work, new, fs.nvars, factors=fs.factors, rotvars=getattr(fs, "rotvars", None))
    fs.work = new
    fs.generation = forest.generation
    return t
