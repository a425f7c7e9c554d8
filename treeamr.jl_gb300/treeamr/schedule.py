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
import itertools
from typing import Dict, List, NamedTuple, Optional, Sequence, Tuple

import numpy as np

from .forest import (Forest, MortonKey, OUTER, OUTFLOW, REFLECTING, alldirections, axismap,
                     childoffset, virtual_offset)
from .operators import (BOUNDED_POINTVALUE, UNBOUNDED, Conservative, Operators, boundedmode,
                        check_operators, conservative_prolong_weights,
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
    (prolongations only), the mirror state per dimension, and the orientation
    of a transfer across a rotating or half-turn seam
    (``src/schedule.jl:400-410``; no glue here)."""
    kind: str
    direction: Tuple[int, ...]
    offset: Tuple[int, ...]
    level: int
    mirror: Tuple[int, ...]
    span: Tuple[int, ...]
    orientation: int = 0     # quarter turns across a seam (0 off it)

    def order(self):
        """``keyorder`` (``src/schedule.jl:495-497``)."""
        return (KINDRANK[self.kind], self.direction, self.offset, self.level, self.mirror,
                self.orientation, 0, self.span)


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
                 stage: int, axes=None, bounded: int = 0):
        self.key = key
        self.kind = key.kind
        # how the kernel bounds the group's result (``boundedmode``): 0 not
        # at all, 1 the bounded conservative prolongation, 2 the point-value
        # sum clamped into its bracket (stencils with the linear rows stacked)
        self.bounded = int(bounded)
        # A turned group (across a seam) reads its real source through the
        # axis map ``(perm, flip)`` in gather form (0-based dimensions) and
        # the variable table's column ``orientation`` (``src/ghosts.jl:183-244``).
        self.orientation = int(key.orientation)
        D = len(key.direction)
        self.perm, self.flip = axes if axes is not None else \
            (tuple(range(D)), (False,) * D)
        self.turned = self.orientation != 0
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
    dimension.  For the relative hook, ``clamps`` is per dimension the
    stored index of the nearest evolved point along a component that leaves
    through an outer face (``G + N + c`` high, ``G + 1`` low) and 0 along the
    others, and ``slot`` the stage tag after which the ghosts it reads along
    those others are filled (phase 1, or the prolongations onto the block's
    level)."""
    block: int
    direction: Tuple[int, ...]
    region: Tuple[Tuple[int, int], ...]
    clamps: Tuple[int, ...] = ()
    slot: int = 1


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


def copy_stencil(T, N, G, c, dd, span: int = -1) -> Stencil1D:
    rng = piece_range(N, G, c, span) if span >= 0 else target_range(N, G, c, dd, 0, False)
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


LINEAR_OPERATORS = Operators(prolongation=2, restriction=2)


def stack_linear(s: Stencil1D, lin: Stencil1D, T) -> Stencil1D:
    """A bounded point-value stencil (``src/schedule.jl:1279-1300``): ``s``'s
    order-p weights in rows ``1:p`` and below them, in rows ``p+1:2p``, the
    linear stencil's weights over the same targets placed at their points'
    positions in ``s``'s window; the kernel clamps the order-p sum into the
    range of the points whose linear weight is nonzero, the bracket."""
    p, q, n = s.order, lin.order, s.ntarget
    if s.targetfirst != lin.targetfirst or lin.ntarget != n:
        raise RuntimeError(f"the linear stencil covers other targets than the order-{p} one")
    cols = []
    for i in range(n):
        col = list(s.exact[i]) + [Fraction(0)] * p
        for k in range(q):
            w = lin.exact[i][k]
            if w == 0:
                continue
            off = int(lin.srcstart[i]) + k - int(s.srcstart[i])
            if not 0 <= off < p:
                raise RuntimeError(f"the bracket of target {s.targetfirst + i} lies outside "
                                   f"its order-{p} window")
            col[p + off] = w
        cols.append(col)
    return Stencil1D(s.targetfirst, s.srcstart, cols, T)


def kind_stencil(T, N, G, c, kind, dd, od, ops: Operators, span: int = -1,
                 mode: int = UNBOUNDED) -> Stencil1D:
    """``src/schedule.jl:1183-1204`` (no element sets); ``span`` a sub-piece
    span along a tangential vertex-like dimension (``prolongation_stencil``);
    a bounded point-value group's stencil stacks the linear one."""
    s = _kind_stencil(T, N, G, c, kind, dd, od, ops, span)
    if mode != BOUNDED_POINTVALUE:
        return s
    return stack_linear(s, _kind_stencil(T, N, G, c, kind, dd, od, LINEAR_OPERATORS, span), T)


def _kind_stencil(T, N, G, c, kind, dd, od, ops: Operators, span: int = -1) -> Stencil1D:
    if kind == COPY:
        return copy_stencil(T, N, G, c, dd, span)
    if kind == PROLONG and span >= 0:
        return prolong_stencil_over(T, piece_range(N, G, c, span), N, G, c, dd, od,
                                    ops.vertex_order())
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


def mirror_restriction(T, N, G, od, p, mode: int = UNBOUNDED) -> Stencil1D:
    h = N // 2
    rng = range(G + 1, G + 2 + h) if od == 0 else range(G + 1 + h, G + N + 2)
    s = restrict_stencil_over(T, rng, N, G, 1, 0, od, p)
    if mode != BOUNDED_POINTVALUE:
        return s
    return stack_linear(s, restrict_stencil_over(T, rng, N, G, 1, 0, od, 2), T)


# --- the neighbour search ---------------------------------------------------

def _nospan(D):
    return (-1,) * D


def _record(pairs, key, b, s):
    lst = pairs.get(key)
    if lst is None:
        lst = pairs[key] = ([], [])
    lst[0].append(b + 1)
    lst[1].append(s + 1)


def boundary_region(forest: Forest, k: MortonKey, b: int, delta, region, G=None,
                    c=None) -> BoundaryRegion:
    """``src/schedule.jl:2188-2217``: the region, and the relative hook's
    clamps and stage slot."""
    D = forest.D
    N = forest.N

    def exits(d):
        if delta[d] == 0:
            return False
        step = tuple(delta[d] if e == d else 0 for e in range(D))
        _, faces = forest.wall_direction(k, step)
        return faces[d] == OUTER and not forest.oriented_neighbors(k, step)

    ex = [exits(d) for d in range(D)]
    d2 = tuple(0 if ex[d] else delta[d] for d in range(D))
    slot = PHASE1_TAG
    if any(x != 0 for x in d2):
        d3, _ = forest.wall_direction(k, d2)
        if any(x != 0 for x in d3):
            nbrs = forest.oriented_neighbors(k, d3)
            if not nbrs:
                ex = [x != 0 for x in delta]
            elif nbrs[0].level < k.level:
                slot = prolongation_tag(k.level)
    G = G if G is not None else (0,) * D
    c = c if c is not None else (0,) * D
    clamps = tuple((G[d] + N + c[d] if delta[d] > 0 else G[d] + 1) if ex[d] else 0
                   for d in range(D))
    return BoundaryRegion(b, tuple(delta), tuple((r.start, r.stop - 1) for r in region),
                          clamps, slot)


def wall_regions(forest: Forest, G, c, b: int, bits: int) -> List[BoundaryRegion]:
    """Stage W's regions on block ``b`` (``wall_regions!``,
    ``src/schedule.jl:2134-2170``): every piece of its closed box on an outer
    face of a vertex-like dimension whose copy is the primary, the piece's
    own range, with the outward direction along the outer faces it lies on.
    A hook that prescribes the wall writes them before stage 0, which
    carries them to every other copy.  The relative form's nearest evolved
    point is one plane in from the wall (``G + 2`` low, ``G + N`` high), a
    primary of the same block that stage W does not write."""
    D, N = forest.D, forest.N
    k = forest.leaves[b]

    def isouter(d, side):
        step = tuple(side if e == d else 0 for e in range(D))
        _, faces = forest.wall_direction(k, step)
        return faces[d] == OUTER and not forest.oriented_neighbors(k, step)

    outer = [(isouter(d, -1), isouter(d, 1)) if c[d] == 1 else (False, False)
             for d in range(D)]
    if not any(lo or hi for lo, hi in outer):
        return []
    out = []
    for cls in closed_pieces(c):
        delta = tuple(-1 if cls[d] == 0 and outer[d][0] else
                      1 if cls[d] == 2 and outer[d][1] else 0 for d in range(D))
        if all(x == 0 for x in delta):
            continue
        if not (bits >> piece_index(cls)) & 1:
            continue
        region = []
        for d in range(D):
            r = piece_range(N, G[d], c[d], piece_span(cls[d]))
            region.append((r.start, r.stop - 1))
        clamps = tuple(G[d] + 2 if delta[d] < 0 else G[d] + N if delta[d] > 0 else 0
                       for d in range(D))
        out.append(BoundaryRegion(b, delta, tuple(region), clamps, UNIFY_TAG))
    return out


def block_sources(pairs: Dict[GroupKey, Tuple[List[int], List[int]]],
                  boundaries: List[BoundaryRegion], forest: Forest, G, c, b: int, dirs,
                  table: Optional["NeighbourTable"] = None):
    """Every transfer block ``b``'s ghosts need (``src/schedule.jl:1525-1610``),
    and for a layout with a vertex-like dimension its stage-0 transfers
    (``unify_sources!``).  ``b`` is 0-based; recorded block indices are 1-based.
    Returns the block's primary bits (0 for a cell-centred layout)."""
    k = forest.leaves[b]
    N, D = forest.N, forest.D
    zero = (0,) * D
    nomirror = (0,) * D
    nospan = _nospan(D)
    closed = any(cd == 1 for cd in c)
    if closed and table is None:
        table = NeighbourTable(forest, b)

    def record(kind, offset, lvl, s, delta, span=nospan, turns=0):
        _record(pairs, GroupKey(kind, tuple(delta), offset, lvl, nomirror, span, turns), b, s)

    for delta in dirs:
        region = [target_range(N, G[d], c[d], delta[d], 0, False) for d in range(D)]
        if any(len(r) == 0 for r in region):
            continue
        dprime, faces = forest.wall_direction(k, delta)
        if any(f != OUTER for f in faces):
            mirror_sources(pairs, boundaries, forest, G, c, b, delta, dprime, faces, region)
            continue
        r, nbrs = forest.turned_neighbors(k, delta)
        if table is not None:
            table.remember(delta, nbrs, r)
        if not nbrs:
            boundaries.append(boundary_region(forest, k, b, delta, region, G, c))
            continue
        nbl = nbrs[0].level
        if nbl == k.level:
            record(COPY, zero, 0, forest.find_leaf(nbrs[0]), delta, turns=r)
        elif nbl < k.level:
            src = forest.find_leaf(nbrs[0])
            parts = ghost_plane_parts(forest, k, delta, delta, c, src) if closed else None
            if parts is None:
                record(PROLONG, childoffset(k), k.level, src, delta, turns=r)
            else:
                for kind, dirn, span, s, via in parts:
                    if kind == PROLONG:
                        record(PROLONG, childoffset(k), k.level, s, delta, span, turns=r)
                    else:
                        record(COPY, zero, 0, s, dirn, span, turns=via)
        else:
            # each finer neighbour by its offset in its virtual parent,
            # where this block sees it across a seam
            for nbr in nbrs:
                record(RESTRICT, seam_offset(forest, nbr, r), 0, forest.find_leaf(nbr), delta,
                       turns=r)
    if closed:
        return unify_sources(pairs, forest, c, b, table)
    return 0


def seam_offset(forest: Forest, nbr: MortonKey, r: int) -> Tuple[int, ...]:
    """A finer neighbour's child offset in the virtual frame
    (``src/schedule.jl:1411-1420``)."""
    o = childoffset(nbr)
    return virtual_offset(o, r, *forest.seam_plane()) if r else o


def mirror_sources(pairs, boundaries, forest: Forest, G, c, b, delta, dprime, walls, region):
    """A ghost region crossing a reflecting or outflow face
    (``src/schedule.jl:2237-2297``)."""
    k = forest.leaves[b]
    D = forest.D
    zero = (0,) * D
    mask = [w != OUTER for w in walls]
    state = tuple(0 if not mask[d] else 3 if walls[d] == OUTFLOW else 1 for d in range(D))
    nospan = _nospan(D)
    closed = any(cd == 1 for cd in c)

    def record(kind, offset, lvl, s, dirn=tuple(delta), span=nospan, turns=0):
        _record(pairs, GroupKey(kind, tuple(dirn), offset, lvl, state, span, turns), b, s)

    if dprime == zero:
        record(COPY, zero, 0, b)
        return
    # dprime may still cross a seam, the mirror being outside its plane:
    # the two compose, the source turned and then mirrored
    r, nbrs = forest.turned_neighbors(k, dprime)
    if not nbrs:
        boundaries.append(boundary_region(forest, k, b, delta, region, G, c))
        return
    nbl = nbrs[0].level
    if nbl == k.level:
        record(COPY, zero, 0, forest.find_leaf(nbrs[0]), turns=r)
    elif nbl < k.level:
        src = forest.find_leaf(nbrs[0])
        parts = ghost_plane_parts(forest, k, tuple(delta), dprime, c, src) if closed else None
        if parts is None:
            record(PROLONG, childoffset(k), k.level, src, turns=r)
        else:
            for kind, dirn, span, s, via in parts:
                if kind == PROLONG:
                    record(PROLONG, childoffset(k), k.level, s, tuple(delta), span, turns=r)
                else:
                    record(COPY, zero, 0, s, dirn, span, turns=via)
    else:
        wallside = [0 if delta[d] < 0 else 1 for d in range(D)]
        for nbr in nbrs:
            o = seam_offset(forest, nbr, r)
            if all((not mask[d]) or o[d] == wallside[d] for d in range(D)):
                record(RESTRICT, o, 0, forest.find_leaf(nbr), turns=r)


# --- closed blocks: the primary of a shared point (vertex-like layouts) ---
#
# A point on a block face of a vertex-like dimension is held by every block
# whose closed box contains it; one copy is the primary and stage 0 gives
# the others its value (src/schedule.jl:1612-1990).  A block's closed box
# falls into pieces by class per dimension (0 low face plane, 1 open
# interior, 2 high face plane; 1 along a cell-like dimension) and finer into
# sub-pieces (0 low plane, 1 lower open half, 2 mid-plane, 3 upper open
# half, 4 high plane; 1 and 3 along a cell-like dimension).  The primary is
# the copy on the finest level holding the point, and among those the one
# with the greatest class tuple, dimension 1 first.

def span_code(lo: int, hi: int) -> int:
    return 8 * lo + hi


def span_classes(code: int) -> Tuple[int, int]:
    return code >> 3, code & 7


def piece_range(N: int, G: int, c: int, code: int) -> range:
    """Stored range of a span of sub-pieces (``src/schedule.jl:942-950``)."""
    lo, hi = span_classes(code)
    h = N // 2
    if c == 0:
        first = G + 1 if lo == 1 else G + h + 1
        last = G + h if hi == 1 else G + N
        return range(first, last + 1)
    first = (G + 1, G + 2, G + h + 1, G + h + 2, G + N + 1)[lo]
    last = (G + 1, G + h, G + h + 1, G + N, G + N + 1)[hi]
    return range(first, last + 1)


def piece_index(cls) -> int:
    return sum(x * 3 ** d for d, x in enumerate(cls))


def _product_dim1_fastest(values):
    for rev in itertools.product(*reversed(values)):
        yield tuple(reversed(rev))


def closed_pieces(c):
    return list(_product_dim1_fastest([(0, 1, 2) if cd == 1 else (1,) for cd in c]))


def subpiece_values(c, N):
    return [(1, 3) if cd == 0 else (0, 2, 4) if N == 2 else (0, 1, 2, 3, 4) for cd in c]


def subpiece_list(c, N):
    return list(_product_dim1_fastest(subpiece_values(c, N)))


def piece_class(sub: int) -> int:
    return 0 if sub == 0 else 2 if sub == 4 else 1


def piece_of(sub):
    return tuple(piece_class(x) for x in sub)


def piece_representative(cls, c):
    return tuple(1 if cd == 0 else 2 * x for x, cd in zip(cls, c))


def piece_span(cls: int) -> int:
    return span_code(0, 0) if cls == 0 else span_code(4, 4) if cls == 2 else span_code(1, 3)


class NeighbourTable:
    """The neighbours of one block per direction, looked up once
    (``src/schedule.jl:1742-1779``): ``(level or -1, [(leaf, offset, turns)])``,
    each finer neighbour's child offset taken into the virtual frame where
    this block sees it across a seam (``seam_offset``)."""

    def __init__(self, forest: Forest, j: int):
        self.forest = forest
        self.j = j
        self.level = forest.leaves[j].level
        self.entries = {}

    def remember(self, delta, nbrs, r: int = 0):
        if not nbrs:
            e = (-1, [])
        else:
            e = (nbrs[0].level, [(self.forest.find_leaf(n), seam_offset(self.forest, n, r), r)
                                 for n in nbrs])
        self.entries[tuple(delta)] = e
        return e

    def neighbours(self, delta):
        delta = tuple(delta)
        e = self.entries.get(delta)
        if e is None:
            r, nbrs = self.forest.turned_neighbors(self.forest.leaves[self.j], delta)
            e = self.remember(delta, nbrs, r)
        return e


def subpiece_position(forest: Forest, k: MortonKey, sub) -> Tuple[int, ...]:
    """The midpoint of sub-piece ``sub`` of leaf ``k`` at ``k``'s level, in
    units of a quarter of a block's edge (``src/schedule.jl:1856-1861``)."""
    rp = forest.root_position(k.root)
    return tuple(4 * ((rp[d] << k.level) + k.coords[d]) + sub[d] for d in range(forest.D))


def real_position(forest: Forest, p, r: int, lvl: int) -> Tuple[int, ...]:
    """A virtual position mapped back across the seam as a naive node is
    (``src/schedule.jl:1863-1879``); off the seam the position itself."""
    if r == 0:
        return tuple(p)
    d1, d2 = forest.seam_plane()
    a, b = p[d1], p[d2]
    if r == 1:
        a2, b2 = b, -a
    elif r == 3:
        a2, b2 = -b, a
    elif forest.ishalfturn():
        a2, b2 = -a, 4 * (forest.roots[d2] << lvl) - b
    else:
        a2, b2 = -a, -b
    out = list(p)
    out[d1], out[d2] = a2, b2
    return tuple(out)


def real_classes(forest: Forest, cls, r: int) -> Tuple[int, ...]:
    """A piece's classes seen in the virtual frame of orientation ``r``, in
    the real leaf's own frame (``src/schedule.jl:1900-1912``)."""
    if r == 0:
        return tuple(cls)
    d1, d2 = forest.seam_plane()
    a, b = cls[d1], cls[d2]
    a2, b2 = {1: (b, 2 - a), 3: (2 - b, a)}.get(r, (2 - a, 2 - b))
    out = list(cls)
    out[d1], out[d2] = a2, b2
    return tuple(out)


def piece_copies(t: NeighbourTable, sub, c):
    """Every copy of sub-piece ``sub`` of ``t``'s block on its level or a finer
    one, as ``(level, leaf, class, direction, offset, turns, position)``, its
    own first (``src/schedule.jl:1794-1854``): a copy across a seam has its
    classes and position in the real leaf's frame, so that the members of a
    seam point's orbit compare by position; off the seam every copy lies at
    the asking block's position."""
    D = len(c)
    zero = (0,) * D
    cls = piece_of(sub)
    forest = t.forest
    vpos = subpiece_position(forest, forest.leaves[t.j], sub)
    copies = [(t.level, t.j, cls, zero, zero, 0, vpos)]
    side = tuple((-1 if cls[d] == 0 else 1) if (c[d] == 1 and cls[d] != 1) else 0
                 for d in range(D))
    for m in range(1, 1 << D):
        if any((m >> d) & 1 and side[d] == 0 for d in range(D)):
            continue
        delta = tuple(side[d] if (m >> d) & 1 else 0 for d in range(D))
        lvl, nbrs = t.neighbours(delta)
        if lvl < 0 or lvl < t.level:
            continue
        across = tuple(cls[d] if delta[d] == 0 else 2 - cls[d] for d in range(D))
        if lvl == t.level:
            leaf, _, r = nbrs[0]
            copies.append((lvl, leaf, real_classes(forest, across, r), delta, zero, r,
                           real_position(forest, vpos, r, t.level)))
            continue
        for leaf, o, r in nbrs:
            holds = all(delta[d] != 0 or
                        (o[d] == (1 if sub[d] == 3 else 0) if c[d] == 0 else
                         (sub[d] == 2 or o[d] == (1 if sub[d] >= 3 else 0)))
                        for d in range(D))
            if not holds:
                continue
            fcls = []
            for d in range(D):
                if delta[d] != 0:
                    fcls.append(across[d])
                elif c[d] == 0:
                    fcls.append(1)
                elif sub[d] == 2:
                    fcls.append(2 if o[d] == 0 else 0)
                else:
                    fcls.append(cls[d] if sub[d] in (0, 4) else 1)
            copies.append((lvl, leaf, real_classes(forest, tuple(fcls), r), delta, o, r,
                           real_position(forest, vpos, r, t.level)))
    return copies


def piece_primary(copies):
    """The finest level, then the lexicographically greatest real position
    (which picks one member of a seam point's orbit, and is no choice off
    the seam), then the greatest class tuple; the first on a tie
    (``src/schedule.jl:1914-1921``)."""
    best, bkey = None, None
    for x in copies:
        key = (-x[0], tuple(-v for v in x[6]), tuple(-v for v in x[2]))
        if bkey is None or key < bkey:
            best, bkey = x, key
    return best


def box_spans(subs, allowed):
    D = len(allowed)
    lo = tuple(min(p[d] for p in subs) for d in range(D))
    hi = tuple(max(p[d] for p in subs) for d in range(D))
    box = 1
    for d in range(D):
        box *= sum(1 for x in allowed[d] if lo[d] <= x <= hi[d])
    return tuple(span_code(lo[d], hi[d]) for d in range(D)) if box == len(subs) else None


def merged_transfers(entries, allowed):
    """Stage 0's merging (``src/schedule.jl:2093-2125``): one transfer per
    source, direction, offset and orientation over the bounding box of its
    sub-pieces where they fill it; restrictions merged within one piece of
    the target only.  Entries ``(sub, kind, source, direction, offset[,
    turns])``; out ``(kind, source, direction, offset, spans, turns)``."""
    bysource = {}
    for e in entries:
        sub, kind, s, delta, o = e[:5]
        r = e[5] if len(e) > 5 else 0
        bysource.setdefault((KINDRANK[kind], s, delta, o, r), []).append(sub)
    out = []
    for key in sorted(bysource):
        rank, s, delta, o, r = key
        kind = COPY if rank == KINDRANK[COPY] else RESTRICT
        subs = list(dict.fromkeys(bysource[key]))
        spans = box_spans(subs, allowed) if kind == COPY else None
        if spans is None:
            for piece in sorted(set(piece_of(p) for p in subs)):
                part = [p for p in subs if piece_of(p) == piece]
                spans = box_spans(part, allowed)
                if spans is None:
                    for p in part:
                        out.append((kind, s, delta, o, tuple(span_code(x, x) for x in p), r))
                else:
                    out.append((kind, s, delta, o, spans, r))
        else:
            out.append((kind, s, delta, o, spans, r))
    return out


def unify_transfers(t: NeighbourTable, c):
    """Stage 0's transfers into ``t``'s block and its primary bits
    (``src/schedule.jl:1990-2040``)."""
    forest = t.forest
    b = t.j
    D = len(c)
    entries = []
    lvl = t.level
    npieces = 3 ** D
    shared = [0] * npieces
    primaries = [None] * npieces
    bits = 0
    for sub in subpiece_list(c, forest.N):
        cls = piece_of(sub)
        i = piece_index(cls)
        if shared[i] == 0:
            copies = piece_copies(t, piece_representative(cls, c), c)
            primaries[i] = piece_primary(copies)
            shared[i] = 1 if all(x[0] == lvl for x in copies) else 2
            s, scls = primaries[i][1], primaries[i][2]
            if s == b and scls == cls:
                bits |= 1 << i
        if all(x == 1 for x in cls):
            continue
        slvl, s, scls, delta, o, r = (primaries[i] if shared[i] == 1 else
                                      piece_primary(piece_copies(t, sub, c)))[:6]
        if s == b and scls == cls:
            continue
        entries.append((sub, COPY if slvl == lvl else RESTRICT, s, delta, o, r))
    return merged_transfers(entries, subpiece_values(c, forest.N)), bits


def unify_sources(pairs, forest: Forest, c, b: int, table: NeighbourTable) -> int:
    """Stage 0's transfers into block ``b`` (``src/schedule.jl:1948-1988``),
    a copy across a seam keyed by its orientation."""
    D = len(c)
    out, bits = unify_transfers(table, c)
    for kind, s, delta, o, spans, r in out:
        _record(pairs, GroupKey(kind, delta, o, 0, (0,) * D, spans, r), b, s)
    return bits


def ghost_plane_parts(forest: Forest, k: MortonKey, delta, dlook, c, coarse: int):
    """The ghosts of ``k`` in ``delta`` next to a coarser neighbour ``coarse``,
    split where a block of ``k``'s level holds a face-plane row along a
    tangential vertex-like dimension (``src/schedule.jl:1432-1507``).
    ``None`` where nothing splits; otherwise parts ``(kind, direction, span,
    source, turns)`` (0-based source; a copy across a seam keeps its
    orientation, a prolongation the one its caller has)."""
    D = forest.D
    tdims = [d for d in range(D) if delta[d] == 0 and c[d] == 1]
    if not tdims:
        return None
    l = k.level
    found = {}

    def holder(dirn):
        if dirn not in found:
            r, nbrs = forest.turned_neighbors(k, dirn)
            if not nbrs:
                found[dirn] = None
            else:
                lv = nbrs[0].level
                if lv > l:
                    raise RuntimeError(f"the ghost of {k} in direction {delta} has a face-plane "
                                       f"row held by a finer block across {dirn}; 2:1 balance "
                                       "forbids that, so this is a bug")
                found[dirn] = (lv, forest.find_leaf(nbrs[0]), r)
        return found[dirn]

    pieces = list(_product_dim1_fastest([(0, 1, 2)] * len(tdims)))
    sources = []
    for cls in pieces:
        plane = [(tdims[i], -1 if cls[i] == 0 else 1) for i in range(len(tdims)) if cls[i] != 1]
        best = None
        subsets = sorted(range(1, 2 ** len(plane)), key=lambda m: (bin(m).count("1"), m))
        for m in subsets:
            dirn = list(dlook)
            for i, (d, s) in enumerate(plane):
                if (m >> i) & 1:
                    dirn[d] = s
            h = holder(tuple(dirn))
            if h is None:
                continue
            lv, j, r = h
            if j == coarse:
                continue
            if lv == l and best is None:
                best = (m, j, r)
        if best is None:
            sources.append(None)
            continue
        m, j, r = best
        dirn = list(delta)
        for i, (d, s) in enumerate(plane):
            if (m >> i) & 1:
                dirn[d] = s
        sources.append((tuple(dirn), j, r))
    if all(s is None for s in sources):
        return None

    def code(x):
        return span_code(0, 0) if x == 0 else span_code(1, 3) if x == 1 else span_code(4, 4)

    def spanof(cls):
        return tuple(code(cls[tdims.index(d)]) if d in tdims else -1 for d in range(D))

    parts = []
    rest = [cls for cls, s in zip(pieces, sources) if s is None]
    if rest:
        n = len(tdims)
        lo = tuple(min(p[i] for p in rest) for i in range(n))
        hi = tuple(max(p[i] for p in rest) for i in range(n))
        vol = 1
        for i in range(n):
            vol *= hi[i] - lo[i] + 1
        if vol == len(rest):
            fs = {0: 0, 1: 1, 2: 4}
            ls = {0: 0, 1: 3, 2: 4}
            span = tuple(span_code(fs[lo[tdims.index(d)]], ls[hi[tdims.index(d)]])
                         if d in tdims else -1 for d in range(D))
            parts.append((PROLONG, tuple(delta), span, coarse, 0))
        else:
            for cls in rest:
                parts.append((PROLONG, tuple(delta), spanof(cls), coarse, 0))
    for cls, s in zip(pieces, sources):
        if s is None:
            continue
        parts.append((COPY, s[0], spanof(cls), s[1], s[2]))
    return parts


def axis_points(forest: Forest, G, c, bits):
    """A seam's axis points, ``([(block, 1-based stored index)], orbit)``
    (``axis_points``, ``src/schedule.jl:2653-2690``): the points of the
    blocks at the low corner of the seam's plane (a quarter turn), or at the
    low face of d1 meeting the centre plane of d2 (a half turn), on the
    pieces whose copy is the primary; the axis needs a vertex-like d1 and
    d2.  Each is its own image under the turn, so its variables become the
    mean of their images under the orbit's powers of the set's map, summed
    in pairs a half turn apart: orbit ``(0, 2, 1, 3)``, or ``(0, 2)``."""
    if not forest.hasrotating():
        return [], ()
    d1, d2 = forest.seam_plane()
    if not (c[d1] == 1 and c[d2] == 1):
        return [], ()
    half = forest.ishalfturn()
    D, N = forest.D, forest.N
    out = []
    for b, k in enumerate(forest.leaves):
        lvl = k.level
        rp = forest.root_position(k.root)
        g = [(rp[d] << lvl) + k.coords[d] for d in range(D)]
        if g[d1] != 0:
            continue
        n2 = forest.roots[d2] << lvl
        if half:
            cls2 = 0 if g[d2] == n2 // 2 else 2 if g[d2] + 1 == n2 // 2 else -1
        else:
            cls2 = 0 if g[d2] == 0 else -1
        if cls2 < 0:
            continue
        for cls in closed_pieces(c):
            if cls[d1] != 0 or cls[d2] != cls2 or not (bits[b] >> piece_index(cls)) & 1:
                continue
            rngs = [piece_range(N, G[d], c[d], piece_span(cls[d])) for d in range(D)]
            for I in _product_dim1_fastest([list(r) for r in rngs]):
                out.append((b, tuple(I)))
    return out, ((0, 2) if half else (0, 2, 1, 3))


def selfimage_sources(pairs, forest: Forest, c, b: int, parities, bits: int):
    """Stage P's transfers of block ``b``: every primary piece on a reflecting
    wall plane of a vertex-like dimension, keyed by mirror state 2 there
    (``src/schedule.jl:2605-2634``)."""
    D = forest.D
    if not any(cd == 1 for cd in c):
        return
    k = forest.leaves[b]

    def face(d, s):
        step = tuple(s if e == d else 0 for e in range(D))
        return forest.wall_direction(k, step)[1][d]

    refl = [((face(d, -1) == REFLECTING), (face(d, 1) == REFLECTING)) if c[d] == 1
            else (False, False) for d in range(D)]
    if not any(r[0] or r[1] for r in refl):
        return
    bystate = {}
    for cls in closed_pieces(c):
        if not (bits >> piece_index(cls)) & 1:
            continue
        state = tuple(2 if (cls[d] == 0 and refl[d][0]) or (cls[d] == 2 and refl[d][1]) else 0
                      for d in range(D))
        if not any(state):
            continue
        if parities and not any(any(state[d] == 2 and p[d] == "OddParity" for d in range(D))
                                for p in parities):
            continue
        bystate.setdefault(state, []).append(cls)
    zero = (0,) * D
    for state in sorted(bystate):
        for spans in piece_box_spans(bystate[state], c):
            _record(pairs, GroupKey(COPY, zero, zero, 0, state, spans), b, b)


def piece_box_spans(pieces, c):
    D = len(c)
    fs = {0: 0, 1: 1, 2: 4}
    ls = {0: 0, 1: 3, 2: 4}
    uniq = list(dict.fromkeys(pieces))
    lo = tuple(min(p[d] for p in uniq) for d in range(D))
    hi = tuple(max(p[d] for p in uniq) for d in range(D))
    vol = 1
    for d in range(D):
        vol *= hi[d] - lo[d] + 1
    if vol == len(uniq):
        return [tuple(span_code(fs[lo[d]], ls[hi[d]]) for d in range(D))]
    return [tuple(span_code(fs[p[d]], ls[p[d]]) for d in range(D)) for p in uniq]


def unify_stencil(T, N, G, c, key: GroupKey, d: int, p: int,
                  mode: int = UNBOUNDED) -> Stencil1D:
    """One dimension of a stage-0 (or stage-P) transfer (``src/schedule.jl:973-984``)."""
    dd, code = key.direction[d], key.span[d]
    if key.kind == COPY:
        return copy_stencil(T, N, G, c, dd, span=code)
    rng = piece_range(N, G, c, code)
    s = restrict_stencil_over(T, rng, N, G, c, dd, key.offset[d], p)
    if mode != BOUNDED_POINTVALUE:
        return s
    return stack_linear(s, restrict_stencil_over(T, rng, N, G, c, dd, key.offset[d], 2), T)


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
        closed = any(cd == 1 for cd in c)

        dirs = alldirections(D)
        pairs: Dict[GroupKey, Tuple[List[int], List[int]]] = {}
        ppairs: Dict[GroupKey, Tuple[List[int], List[int]]] = {}
        boundaries: List[BoundaryRegion] = []
        bits = [0] * forest.nleaves()
        for b in range(forest.nleaves()):
            bits[b] = block_sources(pairs, boundaries, forest, G, c, b, dirs)
        if closed:
            for b in range(forest.nleaves()):
                selfimage_sources(ppairs, forest, c, b, parity or [], bits[b])
        self.boundaries = boundaries
        self.primary_bits = bits
        # a seam's axis, its own image under the turn: projected after stage P
        self.axis, self.axis_orbit = axis_points(forest, G, c, bits)
        # stage W's regions, for a hook that prescribes the wall planes
        self.walls: List[BoundaryRegion] = []
        if closed:
            for b in range(forest.nleaves()):
                self.walls.extend(wall_regions(forest, G, c, b, bits[b]))

        built = {}

        def boundedof(key):
            return boundedmode(operators, key.kind, key.mirror, c)

        def build1(key: GroupKey, d: int) -> Stencil1D:
            mode = boundedof(key)
            if isunify(key):
                return unify_stencil(T, N, G[d], c[d], key, d, operators.restriction, mode)
            dd, od, state = key.direction[d], key.offset[d], key.mirror[d]
            ds = dd if state == 0 else 0
            if state != 0 and key.kind == RESTRICT and c[d] == 1:
                s = mirror_restriction(T, N, G[d], od, operators.restriction, mode)
            else:
                s = kind_stencil(T, N, G[d], c[d], key.kind, ds, od, operators, key.span[d],
                                 mode)
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
            # the mirror state and the orientation: mirror column + 3^D r
            # (src/schedule.jl:3218-3229)
            signs = tuple(0 if m == 3 else m for m in key.mirror)
            return mirrorcolumn(signs) + 3 ** D * key.orientation \
                if any(signs) or key.orientation else 0

        def axesof(key):
            if key.orientation:
                return axismap(key.orientation, *forest.seam_plane(), D)
            return None

        groups = []
        for key in sorted(pairs, key=GroupKey.order):
            tb, sb = pairs[key]
            groups.append(TransferGroup(key, build(key), tb, sb, factorcol(key),
                                        transfer_stage(key), axesof(key), boundedof(key)))
        for key in sorted(ppairs, key=GroupKey.order):
            tb, sb = ppairs[key]
            groups.append(TransferGroup(key, build(key), tb, sb, factorcol(key),
                                        SELFIMAGE_TAG, None, boundedof(key)))
        self.groups = groups
        self.turned = any(g.turned for g in groups)
        self.odd_turns = any(g.orientation % 2 for g in groups)
        self.selfimage = [g for g in groups if g.stage == SELFIMAGE_TAG]
        self.unify = [g for g in groups if g.stage == UNIFY_TAG]
        self.phase1 = [g for g in groups if g.stage == PHASE1_TAG]
        levels = sorted({g.key.level for g in groups if g.stage >= 2})
        self.levels = levels
        self.phase2 = [[g for g in groups if g.stage == prolongation_tag(l)] for l in levels]
        # the stage tags in the order the fill runs them: stage P, stage 0,
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
            if g.stage < PHASE1_TAG:        # stages P and 0 write owned points
                continue
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
