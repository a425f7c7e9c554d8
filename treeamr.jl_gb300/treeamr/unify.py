"""Stage 0 of a fill alone: ``UnifySchedule`` and ``unify``
(``src/unify.jl:1-175``, ``src/ghosts.jl:1836-1906, 2003-2044``).

A set with a vertex-like dimension owns both face planes of its blocks, so a
point on a block face has a copy on every block that holds it.  Stage 0 gives
every secondary copy its primary's value: a copy from a block of its own
level, the restriction from a finer one, with the restriction the geometry
fixes (injection along a vertex-like dimension, the exact two-cell average
along a cell-like one).  On a flux that is the interface restriction a
conservative scheme needs at coarse-fine faces.  Over a forest with
reflecting faces the schedule also holds stage P, the wall-plane parity
projection.  The transfers run on the device through the same library and
kernels as the ghost fill: ``tam_fill`` over stage tags -1 and 0, on the
working array, or on a state vector through a copy of the schedule whose
indices are those of the own box.
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Union

import numpy as np
import torch

from .schedule import (GhostSchedule, GroupKey, NeighbourTable, SELFIMAGE_TAG, Stencil1D,
                       TransferGroup, UNIFY_TAG, selfimage_sources, unify_sources,
                       unify_stencil)
from .storage import FieldSet


class UnifySchedule:
    """Stages P and 0 of a fill for a set with a vertex-like dimension
    (``src/unify.jl:59-175``).  ``UnifySchedule(fs)``; replayed by ``unify``.
    Takes no operators: the restriction is the geometry's, order 2."""

    def __init__(self, fs: FieldSet):
        c = fs.c
        D = fs.forest.D
        if not any(cd == 1 for cd in c):
            raise ValueError(
                "a cell-centred field set has no shared point to unify: the fixup replaces "
                "the values lying on a block's boundary face, and a cell-centred field has "
                f"none. Build it over the field set that holds the face quantity, whose "
                f"centering is vertex-like in the face dimension (facecentered({D}, d)).")
        forest = fs.forest
        self.forest = forest
        self.generation = forest.generation
        self.G = fs.G
        self.centering = fs.centering
        self.c = c
        self.T = fs.T
        self.parities = fs.parities
        N = forest.N
        self.stored = tuple(N + 2 * g + cd for g, cd in zip(fs.G, c))
        self.own = tuple(N + cd for cd in c)
        pairs, ppairs = {}, {}
        bits = [0] * forest.nleaves()
        for b in range(forest.nleaves()):
            bits[b] = unify_sources(pairs, forest, c, b, NeighbourTable(forest, b))
        for b in range(forest.nleaves()):
            selfimage_sources(ppairs, forest, c, b, fs.parities or [], bits[b])
        self.primary_bits = bits
        built = {}

        def build(key):
            if key not in built:
                built[key] = tuple(unify_stencil(fs.T, N, fs.G[d], c[d], key, d, 2)
                                   for d in range(D))
            return built[key]

        from .storage import mirrorcolumn

        def factorcol(key):
            signs = tuple(0 if m == 3 else m for m in key.mirror)
            return mirrorcolumn(signs) if any(signs) else 0

        groups = []
        for key in sorted(ppairs, key=GroupKey.order):
            tb, sb = ppairs[key]
            groups.append(TransferGroup(key, build(key), tb, sb, factorcol(key), SELFIMAGE_TAG))
        for key in sorted(pairs, key=GroupKey.order):
            tb, sb = pairs[key]
            groups.append(TransferGroup(key, build(key), tb, sb, factorcol(key), UNIFY_TAG))
        self.groups = groups
        self.selfimage = [g for g in groups if g.stage == SELFIMAGE_TAG]
        self.unify = [g for g in groups if g.stage == UNIFY_TAG]
        self.stage_tags = sorted({g.stage for g in groups})
        self.boundaries = []
        self._state = None

    def isstale(self) -> bool:
        return self.forest.generation != self.generation

    def all_groups(self) -> List[TransferGroup]:
        return sorted(self.groups, key=lambda g: g.stage)

    def ghost_items(self, nvars: int) -> int:
        return sum(int(np.prod(g.boxsize())) * g.ntransfers() for g in self.groups) * nvars

    def __repr__(self):
        kinds = {}
        for g in self.unify:
            kinds[g.kind] = kinds.get(g.kind, 0) + g.ntransfers()
        return (f"UnifySchedule{{{np.dtype(self.T).name},{self.forest.D}}}("
                f"{kinds.get('copy', 0)} copies, {kinds.get('restrict', 0)} restrictions)")


class _StateForm:
    """A schedule's stages P and 0 with every index moved into the own box:
    what ``unify`` replays on a state vector (``stateunify``,
    ``src/unify.jl:150-160``).  Stage 0 reads and writes own points only."""

    def __init__(self, schedule, groups: Sequence[TransferGroup], G, own):
        self.forest = schedule.forest
        self.T = schedule.T
        self.stored = tuple(own)
        moved = {}

        def shift(s: Stencil1D, g: int) -> Stencil1D:
            k = (id(s), g)
            if k not in moved:
                t = Stencil1D.__new__(Stencil1D)
                t.targetfirst = s.targetfirst - g
                t.srcstart = (s.srcstart - g).astype(np.int32)
                t.exact = s.exact
                t.weights = s.weights
                t.unit = s.unit
                moved[k] = t
            return moved[k]

        D = self.forest.D
        self.groups = [TransferGroup(gr.key, tuple(shift(gr.stencils[d], G[d]) for d in range(D)),
                                     gr.targetblocks, gr.sourceblocks, gr.factorcol, gr.stage)
                       for gr in groups]

    def all_groups(self):
        return sorted(self.groups, key=lambda g: g.stage)


def _unify_groups(schedule):
    return [g for g in schedule.all_groups() if g.stage in (SELFIMAGE_TAG, UNIFY_TAG)]


def check_unify(fs: FieldSet, schedule) -> None:
    """The layout checks of ``check_unify`` (``src/ghosts.jl:2003-2044``)."""
    if isinstance(schedule, GhostSchedule):
        from .ghosts import check_fill
        check_fill(fs, schedule)
        return
    if schedule.forest is not fs.forest:
        raise ValueError("unify schedule was built for a different forest than the field set")
    if schedule.isstale():
        raise ValueError(f"the forest changed since this unify schedule was built (generation "
                         f"{schedule.generation} -> {schedule.forest.generation}); rebuild it")
    if fs.nblocks() != schedule.forest.nleaves():
        raise ValueError(f"field set has {fs.nblocks()} blocks but the schedule's forest has "
                         f"{schedule.forest.nleaves()}; rebuild both")
    if tuple(fs.G) != tuple(schedule.G):
        raise ValueError(f"the field set has ghost width G={fs.G} but this unify schedule was "
                         f"built for G={schedule.G}; build one with UnifySchedule(fs)")
    if schedule.parities and list(schedule.parities) != list(fs.parities or []):
        raise ValueError(f"the field set's variables have the parities {fs.parities} but this "
                         f"unify schedule was built for {schedule.parities}; build one with "
                         "UnifySchedule(fs)")
    if tuple(fs.centering) != tuple(schedule.centering):
        raise ValueError(f"the field set has centering {fs.centering} but this unify schedule "
                         f"was built for {schedule.centering}; build one with UnifySchedule(fs)")
    if np.dtype(fs.T) != np.dtype(schedule.T):
        raise ValueError(f"the field set stores {np.dtype(fs.T).name} but this unify schedule "
                         f"carries {np.dtype(schedule.T).name} weights; build the schedule from "
                         "the field set itself, UnifySchedule(fs)")


def unify(a: Union[FieldSet, torch.Tensor], b=None, c=None, *,
          stream: Optional[torch.cuda.Stream] = None):
    """``unify!(fs, schedule)`` on the working array, or ``unify!(v, fs,
    schedule)`` on a state vector ``v`` (``src/ghosts.jl:1836-1858``):
    stages P and 0 of a ``UnifySchedule`` or a ``GhostSchedule``.  Returns
    what it was given."""
    from .ghosts import DeviceSchedule, device_schedule
    if isinstance(a, FieldSet):
        fs, schedule = a, b
        check_unify(fs, schedule)
        ds = device_schedule(schedule, fs.work.device.index or 0)
        ds.run(fs, SELFIMAGE_TAG, UNIFY_TAG, "fused", stream)
        return fs
    v, fs, schedule = a, b, c
    check_unify(fs, schedule)
    from .state import statearray, ownextents
    A = statearray(v, fs)
    if v.device != fs.work.device or not v.is_contiguous() or v.dtype != fs.work.dtype:
        raise ValueError("the state vector must be contiguous, of the field set's type and "
                         "on its device")
    cache = schedule.__dict__.setdefault("_state_device", {})
    dev = v.device.index or 0
    if dev not in cache:
        form = _StateForm(schedule, _unify_groups(schedule), fs.G, ownextents(fs))
        cache[dev] = DeviceSchedule(form, dev)
    ds = cache[dev]

    class _View:                     # the state array as the fill's working array
        work = A
        nvars = fs.nvars
        factors = fs.factors

        @staticmethod
        def nblocks():
            return fs.nblocks()
    ds.run(_View, SELFIMAGE_TAG, UNIFY_TAG, "fused", stream)
    return v
