"""The ghost-exchange schedule: built once per regrid, replayed every fill.

Restates the reference's schedule build (``src/schedule.jl``) for brick
forests of cell-centred layouts, with periodic, reflecting, outflow and
outer faces:

* ``Stencil1D`` -- ``src/schedule.jl:64-93``; ``TransferGroup`` -- ``:150-197``.
* ``GroupKey`` and its order -- ``src/schedule.jl:400-506``.
* ``target_range`` -- ``:929-938``; ``copy_stencil`` -- ``:960-965``;
  ``restrict_stencil_over`` -- ``:1002-1025``; ``source_direction`` --
  ``:1035-1036``; ``prolong_stencil_over`` -- ``:1047-1079``;
  ``conservative_prolong_stencil`` -- ``:1122-1143``.
* ``clamp_rows`` / ``mirror_rows`` / ``mirror_restriction`` -- ``:1337-1395``.
* ``block_sources!`` -- ``:1525-1610``; ``mirror_sources!`` -- ``:2237-2297``;
  ``boundary_region`` -- ``:2188-2221``.
* ``GhostSchedule`` -- ``:3075-3292`` (``build1``, ``factorcol``,
  ``transfer_stage`` ``:656-658``, ``local_groups`` ``:2970-2992``).

The schedule is host data.  ``tam_groups`` flattens it into the
struct-of-arrays descriptors the CUDA library uploads once.
"""
from __future__ import annotations

from fractions import Fraction
from typing import Dict, List, NamedTuple, Optional, Sequence, Tuple

import numpy as np

from .forest import Forest, MortonKey, OUTER, OUTFLOW, REFLECTING, alldirections, childoffset
from .operators import (Conservative, Operators, check_operators, conservative_prolong_weights,
                        interpolation_weights, round_weights)
from .storage import FieldSet, ghostwidths, mirrorcolumn, staggers, storedsize

COPY, RESTRICT, PROLONG = "copy", "restrict", "prolong"
KINDRANK = {COPY: 1, RESTRICT: 2, PROLONG: 3}
KINDCODE = {COPY: 1, RESTRICT: 2, PROLONG: 3}

SELFIMAGE_TAG = -1          # stage P (runs first)
UNIFY_TAG = 0               # stage 0
PHASE1_TAG = 1              # copies and restrictions


def prolongation_tag(lvl: int) -> int:
    """``src/schedule.jl:642``."""
    return 2 + int(lvl)


class Stencil1D:
    """One dimension of a transfer: per target row ``targetfirst + i - 1``
    the first source row ``srcstart[i]`` (1-based stored indices) and the
    ``order`` weights ``weights[:, i]`` in the element type."""

    __slots__ = ("targetfirst", "srcstart", "weights", "exact", "unit")

    def __init__(self, targetfirst: int, srcstart: Sequence[int], exact: Sequence[Sequence[Fraction]],
                 dtype):
        self.targetfirst = int(targetfirst)
        self.srcstart = np.asarray(srcstart, dtype=np.int32)
        self.exact = [tuple(col) for col in exact]              # per column, ``order`` rationals
        order = len(self.exact[0]) if self.exact else 1
        w = np.empty((order, len(self.exact)), dtype=dtype)
        for i, col in enumerate(self.exact):
            w[:, i] = round_weights(col, dtype)
        self.weights = w
        self.unit = order == 1 and all(col[0] == 1 for col in self.exact)

    @property
    def ntarget(self) -> int:
        return len(self.srcstart)

    @property
    def order(self) -> int:
        return self.weights.shape[0]

    def rows(self, rows: Sequence[int], targetfirst: int, dtype) -> "Stencil1D":
        """The stencil with its target rows remapped: new row ``i`` takes
        column ``rows[i]`` (1-based) of this one."""
        return Stencil1D(targetfirst, [self.srcstart[r - 1] for r in rows],
                         [self.exact[r - 1] for r in rows], dtype)


class GroupKey(NamedTuple):
    """What a ghost region needs: kind, direction, child offset, target level
    (prolongations only), and the mirror state per dimension
    (``src/schedule.jl:400-410``; no seam orientation or glue here)."""
    kind: str
    direction: Tuple[int, ...]
    offset: Tuple[int, ...]
    level: int
    mirror: Tuple[int, ...]
    span: Tuple[int, ...]

    def order(self):
        """``keyorder`` (``src/schedule.jl:495-497``)."""
        return (KINDRANK[self.kind], self.direction, self.offset, self.level, self.mirror,
                0, 0, self.span)


def isunify(key: GroupKey) -> bool:
    return all(s >= 0 for s in key.span)


def transfer_stage(key: GroupKey) -> int:
    """``src/schedule.jl:656-658``."""
    if isunify(key):
        return UNIFY_TAG
    return prolongation_tag(key.level) if key.kind == PROLONG else PHASE1_TAG


class TransferGroup:
    """All transfers sharing one set of 1-D stencils, as ``(target, source)``
    block pairs (1-based block indices, targets non-decreasing)."""

    def __init__(self, key: GroupKey, stencils, targetblocks, sourceblocks, factorcol: int,
                 stage: int):
        self.key = key
        self.kind = key.kind
        self.stencils = tuple(stencils)
        self.targetblocks = np.asarray(targetblocks, dtype=np.int32)
        self.sourceblocks = np.asarray(sourceblocks, dtype=np.int32)
        self.factorcol = int(factorcol)
        self.stage = int(stage)

    def boxsize(self) -> Tuple[int, ...]:
        return tuple(s.ntarget for s in self.stencils)

    def ntransfers(self) -> int:
        return len(self.targetblocks)

    def unit(self) -> bool:
        return all(s.unit for s in self.stencils)


class BoundaryRegion(NamedTuple):
    """A ghost region facing out of the domain through an outer face, filled
    by the boundary hook (``src/schedule.jl:200-232``).  ``block`` is
    0-based; ``region`` holds 1-based inclusive ``(first, last)`` per
    dimension."""
    block: int
    direction: Tuple[int, ...]
    region: Tuple[Tuple[int, int], ...]


# --- 1-D stencils -----------------------------------------------------------

def target_range(N: int, G: int, c: int, dd: int, od: int, halved: bool) -> range:
    if dd == 1:
        return range(G + N + c + 1, N + 2 * G + c + 1)
    if dd == -1:
        return range(1, G + 1)
    if halved:
        h = N // 2
        if c == 1:
            return range(G + 1, G + 2 + h) if od == 0 else range(G + 2 + h, G + N + 2)
        return range(G + 1 + od * h, G + (od + 1) * h + 1)
    return range(G + 1, G + N + c + 1)


def copy_stencil(T, N, G, c, dd) -> Stencil1D:
    rng = target_range(N, G, c, dd, 0, False)
    return Stencil1D(rng.start, [j - N * dd for j in rng], [(Fraction(1),)] * len(rng), T)


def restrict_stencil_over(T, rng: range, N, G, c, dd, od, p) -> Stencil1D:
    shift = -N * dd
    if c == 1:                                   # injection along a vertex-like dimension
        ss = [G + 1 + 2 * (j + shift - G - 1 - od * (N // 2)) for j in rng]
        return Stencil1D(rng.start, ss, [(Fraction(1),)] * len(rng), T)
    ss, ws = [], []
    for j in rng:
        q = j + shift - G - 1
        f0 = G + 1 + 2 * (q - od * (N // 2))
        lo = min(max(f0 - p // 2 + 1, G + 1), G + N - p + 1)
        ss.append(lo)
        ws.append(interpolation_weights(lo, p, f0 + Fraction(1, 2), "restriction"))
    return Stencil1D(rng.start, ss, ws, T)


def source_direction(dd: int, od: int) -> int:
    return 1 if (dd == 1 and od == 1) else -1 if (dd == -1 and od == 0) else 0


def _fld(a: int, b: int) -> int:
    return a // b


def _cld(a: int, b: int) -> int:
    return -((-a) // b)


def prolong_stencil_over(T, rng: range, N, G, c, dd, od, p) -> Stencil1D:
    stored = N + 2 * G + c
    ss, ws = [], []
    for j in rng:
        phi = od * N + j - G - 1
        origin = -N * source_direction(dd, od) + G + 1
        if c == 1:
            lo = min(max(_fld(phi, 2) - p // 2 + 1 + origin, 1), stored - p + 1)
            x = Fraction(phi, 2) + origin
        else:
            lo = min(max(_cld(phi, 2) - p // 2 + origin, 1), stored - p + 1)
            x = Fraction(phi, 2) - Fraction(1, 4) + origin
        ss.append(lo)
        ws.append(interpolation_weights(lo, p, x, "prolongation"))
    return Stencil1D(rng.start, ss, ws, T)


def conservative_prolong_stencil(T, N, G, c, dd, od, p) -> Stencil1D:
    rng = target_range(N, G, c, dd, od, False)
    low, high = conservative_prolong_weights(p)
    r = (p - 1) // 2
    ss, ws = [], []
    for j in rng:
        phi = od * N + j - G - 1
        cc = _fld(phi, 2)
        sub = phi - 2 * cc
        origin = -N * source_direction(dd, od) + G + 1
        ss.append(cc - r + origin)
        ws.append(low if sub == 0 else high)
    return Stencil1D(rng.start, ss, ws, T)


def kind_stencil(T, N, G, c, kind, dd, od, ops: Operators) -> Stencil1D:
    """``src/schedule.jl:1183-1195`` (no element sets)."""
    if kind == COPY:
        return copy_stencil(T, N, G, c, dd)
    if kind == RESTRICT:
        return restrict_stencil_over(T, target_range(N, G, c, dd, od, True), N, G, c, dd, od,
                                     ops.restriction)
    if ops.family == Conservative and c == 0:
        return conservative_prolong_stencil(T, N, G, c, dd, od, ops.prolongation)
    return prolong_stencil_over(T, target_range(N, G, c, dd, od, False), N, G, c, dd, od,
                                ops.vertex_order())


def clamp_range(N, G, c, dd) -> range:
    return range(1, G + 1) if dd < 0 else range(G + N + c + 1, N + 2 * G + c + 1)


def clamp_rows(s: Stencil1D, N, G, c, dd, T) -> Stencil1D:
    rng = clamp_range(N, G, c, dd)
    row = (G + 1 if dd < 0 else G + N + c) - s.targetfirst + 1
    if not (1 <= row <= s.ntarget):
        raise RuntimeError(f"clamped row {row} falls outside the tangential stencil's "
                           f"{s.ntarget} targets (N={N}, G={G}, c={c}, delta={dd})")
    return s.rows([row] * len(rng), rng.start, T)


def mirror_range(N, G, c, dd) -> range:
    return range(1, G + 1) if dd < 0 else range(G + N + 1 + c, N + 2 * G + c + 1)


def mirror_index(N, G, c, dd, j) -> int:
    return 2 * G + 1 + c - j if dd < 0 else 2 * (G + N) + 1 + c - j


def mirror_rows(s: Stencil1D, N, G, c, dd, T) -> Stencil1D:
    rng = mirror_range(N, G, c, dd)
    rows = [mirror_index(N, G, c, dd, j) - s.targetfirst + 1 for j in rng]
    if not all(1 <= r <= s.ntarget for r in rows):
        raise RuntimeError(f"mirror rows {rows} fall outside the tangential stencil's "
                           f"{s.ntarget} targets (N={N}, G={G}, c={c}, delta={dd})")
    return s.rows(rows, rng.start, T)


def mirror_restriction(T, N, G, od, p) -> Stencil1D:
    h = N // 2
    rng = range(G + 1, G + 2 + h) if od == 0 else range(G + 1 + h, G + N + 2)
    return restrict_stencil_over(T, rng, N, G, 1, 0, od, p)


# --- the neighbour search ---------------------------------------------------

NOSPAN = None


def _nospan(D):
    return (-1,) * D


def boundary_region(forest: Forest, k: MortonKey, b: int, delta, region) -> BoundaryRegion:
    return BoundaryRegion(b, tuple(delta), tuple((r.start, r.stop - 1) for r in region))


def block_sources(pairs: Dict[GroupKey, Tuple[List[int], List[int]]],
                  boundaries: List[BoundaryRegion], forest: Forest, G, c, b: int, dirs):
    """Every transfer block ``b``'s ghosts need (``src/schedule.jl:1525-1610``).
    ``b`` is 0-based; recorded block indices are 1-based."""
    k = forest.leaves[b]
    N, D = forest.N, forest.D
    zero = (0,) * D
    nomirror = (0,) * D
    nospan = _nospan(D)

    def record(kind, offset, lvl, s, delta):
        key = GroupKey(kind, delta, offset, lvl, nomirror, nospan)
        lst = pairs.get(key)
        if lst is None:
            lst = pairs[key] = ([], [])
        lst[0].append(b + 1)
        lst[1].append(s + 1)

    for delta in dirs:
        region = [target_range(N, G[d], c[d], delta[d], 0, False) for d in range(D)]
        if any(len(r) == 0 for r in region):
            continue
        dprime, faces = forest.wall_direction(k, delta)
        if any(f != OUTER for f in faces):
            mirror_sources(pairs, boundaries, forest, G, c, b, delta, dprime, faces, region)
            continue
        nbrs = forest.oriented_neighbors(k, delta)
        if not nbrs:
            boundaries.append(boundary_region(forest, k, b, delta, region))
            continue
        nbl = nbrs[0].level
        if nbl == k.level:
            record(COPY, zero, 0, forest.find_leaf(nbrs[0]), delta)
        elif nbl < k.level:
            record(PROLONG, childoffset(k), k.level, forest.find_leaf(nbrs[0]), delta)
        else:
            for nbr in nbrs:
                record(RESTRICT, childoffset(nbr), 0, forest.find_leaf(nbr), delta)


def mirror_sources(pairs, boundaries, forest: Forest, G, c, b, delta, dprime, walls, region):
    """A ghost region crossing a reflecting or outflow face
    (``src/schedule.jl:2237-2297``)."""
    k = forest.leaves[b]
    D = forest.D
    zero = (0,) * D
    mask = [w != OUTER for w in walls]
    state = tuple(0 if not mask[d] else 3 if walls[d] == OUTFLOW else 1 for d in range(D))
    nospan = _nospan(D)

    def record(kind, offset, lvl, s):
        key = GroupKey(kind, tuple(delta), offset, lvl, state, nospan)
        lst = pairs.get(key)
        if lst is None:
            lst = pairs[key] = ([], [])
        lst[0].append(b + 1)
        lst[1].append(s + 1)

    if dprime == zero:
        record(COPY, zero, 0, b)
        return
    nbrs = forest.oriented_neighbors(k, dprime)
    if not nbrs:
        boundaries.append(boundary_region(forest, k, b, delta, region))
        return
    nbl = nbrs[0].level
    if nbl == k.level:
        record(COPY, zero, 0, forest.find_leaf(nbrs[0]))
    elif nbl < k.level:
        record(PROLONG, childoffset(k), k.level, forest.find_leaf(nbrs[0]))
    else:
        wallside = [0 if delta[d] < 0 else 1 for d in range(D)]
        for nbr in nbrs:
            o = childoffset(nbr)
            if all((not mask[d]) or o[d] == wallside[d] for d in range(D)):
                record(RESTRICT, o, 0, forest.find_leaf(nbr))


# --- the schedule -------------------------------------------------------------

class GhostSchedule:
    """The precomputed ghost exchange for one forest and one layout
    (``src/schedule.jl:820-864``), replayed by ``fill_ghosts``.

    ``GhostSchedule(fs, ops)`` or ``GhostSchedule(forest, ops, G=..., centering=..., T=...)``.
    """

    def __init__(self, fs_or_forest, operators: Operators, *, G=None, centering=None, T=None,
                 parity=None):
        if isinstance(fs_or_forest, FieldSet):
            fs = fs_or_forest
            forest, G, centering, T = fs.forest, fs.G, fs.centering, fs.T
            parity = fs.parities
        else:
            forest = fs_or_forest
            if G is None:
                raise ValueError("GhostSchedule(forest, ops) needs the ghost width G")
            centering = centering or ("cell",) * forest.D
            T = T or np.float64
        D, N = forest.D, forest.N
        G = ghostwidths(G, D)
        c = staggers(centering)
        storedsize(N, G, c)
        check_operators(N, G, c, operators)
        if any(cd == 1 for cd in c):
            raise NotImplementedError(
                "vertex-like layouts need the closed-block stages 0 and P, which this "
                "schedule builder does not provide yet")
        T = np.dtype(T)
        self.forest = forest
        self.generation = forest.generation
        self.G = G
        self.centering = tuple(centering)
        self.c = c
        self.T = T
        self.operators = operators
        self.parities = parity
        self.stored = tuple(N + 2 * g + cd for g, cd in zip(G, c))

        dirs = alldirections(D)
        pairs: Dict[GroupKey, Tuple[List[int], List[int]]] = {}
        boundaries: List[BoundaryRegion] = []
        for b in range(forest.nleaves()):
            block_sources(pairs, boundaries, forest, G, c, b, dirs)
        self.boundaries = boundaries

        built = {}

        def build1(key: GroupKey, d: int) -> Stencil1D:
            dd, od, state = key.direction[d], key.offset[d], key.mirror[d]
            ds = dd if state == 0 else 0
            if state != 0 and key.kind == RESTRICT and c[d] == 1:
                s = mirror_restriction(T, N, G[d], od, operators.restriction)
            else:
                s = kind_stencil(T, N, G[d], c[d], key.kind, ds, od, operators)
            if state == 0:
                return s
            if state == 3:
                return clamp_rows(s, N, G[d], c[d], dd, T)
            return mirror_rows(s, N, G[d], c[d], dd, T)

        def build(key):
            if key not in built:
                built[key] = tuple(build1(key, d) for d in range(D))
            return built[key]

        def factorcol(key):
            signs = tuple(0 if m == 3 else m for m in key.mirror)
            return mirrorcolumn(signs) if any(signs) else 0

        groups = []
        for key in sorted(pairs, key=GroupKey.order):
            tb, sb = pairs[key]
            groups.append(TransferGroup(key, build(key), tb, sb, factorcol(key),
                                        transfer_stage(key)))
        self.groups = groups
        self.unify = [g for g in groups if g.stage == UNIFY_TAG]
        self.phase1 = [g for g in groups if g.stage == PHASE1_TAG]
        levels = sorted({g.key.level for g in groups if g.stage >= 2})
        self.levels = levels
        self.phase2 = [[g for g in groups if g.stage == prolongation_tag(l)] for l in levels]
        self.selfimage: List[TransferGroup] = []
        # every group in the order the fill runs them: stage P, stage 0,
        # phase 1, then the prolongations coarsest target level first
        self.stage_tags = sorted({g.stage for g in groups})

    # -- queries ---------------------------------------------------------------
    def isstale(self) -> bool:
        return self.forest.generation != self.generation

    def all_groups(self) -> List[TransferGroup]:
        return sorted(self.groups, key=lambda g: g.stage)

    def transfer_counts(self) -> Dict[str, int]:
        out = {COPY: 0, RESTRICT: 0, PROLONG: 0}
        for g in self.groups:
            out[g.kind] += g.ntransfers()
        return out

    def ghost_items(self, nvars: int) -> int:
        """Point-variables the fill writes: ``sum ntransfers * prod(box) * nvars``."""
        tot = 0
        for g in self.groups:
            n = 1
            for s in g.stencils:
                n *= s.ntarget
            tot += n * g.ntransfers()
        return tot * nvars

    def write_counts(self) -> np.ndarray:
        """How many times each stored point of each block is written by a
        transfer or a hook region (``test/ghost_oracles.jl:228-256``);
        shape ``(nblocks, S_D, ..., S_1)``."""
        D = self.forest.D
        counts = np.zeros((self.forest.nleaves(),) + tuple(reversed(self.stored)), dtype=np.int64)
        for g in self.groups:
            sl = tuple(slice(s.targetfirst - 1, s.targetfirst - 1 + s.ntarget)
                       for s in reversed(g.stencils))
            for tb in g.targetblocks:
                counts[(tb - 1,) + sl] += 1
        for r in self.boundaries:
            sl = tuple(slice(a - 1, z) for a, z in reversed(r.region))
            counts[(r.block,) + sl] += 1
        return counts

    def __repr__(self):
        cnt = self.transfer_counts()
        return (f"GhostSchedule(D={self.forest.D}, leaves={self.forest.nleaves()}, G={self.G}, "
                f"centering={self.centering}, T={self.T.name}, groups={len(self.groups)}, "
                f"copies={cnt[COPY]}, restrictions={cnt[RESTRICT]}, prolongations={cnt[PROLONG]}, "
                f"levels={self.levels})")
