"""The tree: Morton keys and a brick forest of octrees.

Host-side restatement of the reference's tree, which the schedule build
walks once per regrid (never on the per-fill path):

* ``MortonKey`` and its curve order -- ``src/morton.jl:350-482``
  (root first, then Z-order with dimension 1 the most significant,
  an ancestor immediately before its descendants).
* ``Forest`` -- ``src/forest.jl:248-345`` (a brick of roots, periodic,
  reflecting and outflow faces, all-or-nothing refinement).
* ``alldirections`` -- ``src/forest.jl:1319-1323``.
* ``neighbor_anchor`` / ``oriented_neighbors`` -- ``src/forest.jl:1501-1520,
  1718-1740``; ``find_covering_leaf`` / ``collect_touching_leaves`` --
  ``src/forest.jl:1632-1675``.
* ``wall_direction`` -- ``src/forest.jl:1617-1630``.
* ``refine`` / ``coarsen`` / ``balance`` -- ``src/forest.jl:1761-1890``.
* Rotating seams (a quarter turn, ``rotating = (d1, d2)``) and half-turn
  seams (``halfturn = (d1, d2)``): the constructor's checks
  (``src/forest.jl:737-835``), the node a step lands on across the seam
  and its orientation (``seam_orientation``, ``unrotate_node``,
  ``stepped_node``, ``src/forest.jl:1406-1501``), the direction and child
  offset maps (``real_direction``, ``virtual_offset``, :1428-1464) and
  conformity at the seam in ``balance`` (:1837-1890).

Glued patches are not implemented here.
"""
from __future__ import annotations

import itertools
from fractions import Fraction
from typing import Dict, Iterable, List, NamedTuple, Optional, Sequence, Tuple

MAX_LEVEL = 32

OUTER, REFLECTING, OUTFLOW = 0, 1, 2          # FaceKind (src/forest.jl:60-70)


class MortonKey(NamedTuple):
    """A node of the forest: root index, level and per-dimension coordinates
    (each in ``0:2^level-1``) -- ``src/morton.jl:350``."""
    root: int
    level: int
    coords: Tuple[int, ...]


def level(k: MortonKey) -> int:
    return k.level


def parentkey(k: MortonKey) -> MortonKey:
    if k.level == 0:
        raise ValueError(f"a root-level key ({k}) has no parent")
    return MortonKey(k.root, k.level - 1, tuple(c >> 1 for c in k.coords))


def sortedchildkeys(k: MortonKey) -> List[MortonKey]:
    """The ``2^D`` children in curve order.  Dimension 1 is the most
    significant bit of the interleaving (``src/morton.jl:454-482``), so the
    children sort lexicographically by their offsets with dimension 1 first."""
    if k.level >= MAX_LEVEL:
        raise ValueError(f"a key at MAX_LEVEL ({k}) cannot be refined")
    D = len(k.coords)
    out = []
    for off in itertools.product((0, 1), repeat=D):      # last dimension fastest
        out.append(MortonKey(k.root, k.level + 1,
                             tuple(2 * c + o for c, o in zip(k.coords, off))))
    return out


def curve_key(k: MortonKey) -> Tuple[int, int, int]:
    """A sort key equal to the reference's ``isless`` order (``src/morton.jl:454-482``):
    root, then the bit-interleaved padded coordinates with dimension 1 most
    significant, then level (the ancestor first)."""
    D = len(k.coords)
    pad = [c << (MAX_LEVEL - k.level) for c in k.coords]
    code = 0
    for bit in range(MAX_LEVEL - 1, -1, -1):
        for d in range(D):
            code = (code << 1) | ((pad[d] >> bit) & 1)
    return (k.root, code, k.level)


def childoffset(k: MortonKey) -> Tuple[int, ...]:
    """A block's offset within its parent (``src/schedule.jl:1403``)."""
    return tuple(c & 1 for c in k.coords)


def real_direction(delta, r: int, d1: int, d2: int) -> Tuple[int, ...]:
    """``R^{-r} delta`` (``src/forest.jl:1428-1438``): a ghost direction as
    seen from the real leaves across a seam in orientation ``r``; ``d1`` and
    ``d2`` are 0-based."""
    a, b = delta[d1], delta[d2]
    r1, r2 = {1: (b, -a), 3: (-b, a), 2: (-a, -b)}.get(r, (a, b))
    out = list(delta)
    out[d1], out[d2] = r1, r2
    return tuple(out)


def virtual_offset(o, r: int, d1: int, d2: int) -> Tuple[int, ...]:
    """A real leaf's child offset taken into the virtual frame, where the
    asking block sees it across the seam (``src/forest.jl:1450-1464``)."""
    a, b = o[d1], o[d2]
    v1, v2 = {1: (1 - b, a), 3: (b, 1 - a), 2: (1 - a, 1 - b)}.get(r, (a, b))
    out = list(o)
    out[d1], out[d2] = v1, v2
    return tuple(out)


def axismap(r: int, d1: int, d2: int, D: int):
    """The axis map of orientation ``r`` across the seam of the plane
    ``(d1, d2)`` (0-based), in gather form (``src/ghosts.jl:221-234``):
    virtual stored index ``k`` reads the real point whose index along ``e``
    is ``k[perm[e]]``, or ``S + 1 - k[perm[e]]`` where ``flip[e]``."""
    swapped = r % 2 == 1
    perm = tuple(d2 if swapped and e == d1 else d1 if swapped and e == d2 else e
                 for e in range(D))
    flip = tuple((r >= 2) if e == d1 else (r in (1, 2)) if e == d2 else False
                 for e in range(D))
    return perm, flip


def alldirections(D: int) -> List[Tuple[int, ...]]:
    """All ``3^D - 1`` directions, dimension 1 fastest, as Julia's
    ``Iterators.product`` gives them (``src/forest.jl:1319-1323``)."""
    out = []
    for rev in itertools.product((-1, 0, 1), repeat=D):
        d = tuple(reversed(rev))
        if any(d):
            out.append(d)
    return out


class Forest:
    """A ``D``-dimensional brick of ``roots`` octree roots refined into a
    leaf-only linear octree (``src/forest.jl:248``).

    ``faces[d] = (lo, hi)`` is the kind of each non-periodic face:
    ``OUTER`` (the boundary hook's), ``REFLECTING`` or ``OUTFLOW``.
    """

    def __init__(self, roots: Sequence[int], *, N: int,
                 periodic: Optional[Sequence[bool]] = None,
                 reflecting: Optional[Sequence[Tuple[bool, bool]]] = None,
                 outflow: Optional[Sequence[Tuple[bool, bool]]] = None,
                 extents: Optional[Sequence[Tuple[float, float]]] = None,
                 leaves: Optional[Iterable[MortonKey]] = None,
                 rotating: Optional[Tuple[int, int]] = None,
                 halfturn: Optional[Tuple[int, int]] = None):
        D = len(roots)
        if not all(r > 0 for r in roots):
            raise ValueError(f"roots must all be positive, got {tuple(roots)}")
        if N <= 0:
            raise ValueError(f"N must be positive, got {N}")
        if N % 2:
            raise ValueError(f"N must be even, got {N}")
        periodic = tuple(bool(p) for p in (periodic or (False,) * D))
        reflecting = tuple(tuple(bool(x) for x in r) for r in (reflecting or ((False, False),) * D))
        outflow = tuple(tuple(bool(x) for x in r) for r in (outflow or ((False, False),) * D))
        faces = []
        for d in range(D):                                  # src/forest.jl:349-375
            if periodic[d] and any(reflecting[d]):
                raise ValueError(f"dimension {d + 1} is both periodic and reflecting")
            if periodic[d] and any(outflow[d]):
                raise ValueError(f"dimension {d + 1} is both periodic and outflow")
            fk = []
            for s in range(2):
                if reflecting[d][s] and outflow[d][s]:
                    raise ValueError(f"face {s} of dimension {d + 1} is both reflecting and outflow")
                fk.append(REFLECTING if reflecting[d][s] else OUTFLOW if outflow[d][s] else OUTER)
            faces.append(tuple(fk))
        if extents is None:
            extents = tuple((0.0, float(r)) for r in roots)
        if halfturn is not None:
            self.rotating = _check_halfturn(halfturn, rotating, tuple(roots), periodic,
                                            reflecting, outflow)
        else:
            self.rotating = _check_rotating(rotating, tuple(roots), periodic, reflecting,
                                            outflow)
        self.D = D
        self.roots = tuple(int(r) for r in roots)
        self.periodic = periodic
        self.faces = tuple(faces)
        self.extents = tuple((float(a), float(b)) for a, b in extents)
        self.N = int(N)
        self.generation = 0
        if leaves is None:
            nroots = 1
            for r in self.roots:
                nroots *= r
            self.leaves = [MortonKey(r, 0, (0,) * D) for r in range(nroots)]
        else:
            self.leaves = sorted(leaves, key=curve_key)
        self._reindex()

    # -- bookkeeping ---------------------------------------------------------
    def _reindex(self):
        self._index: Dict[MortonKey, int] = {k: i for i, k in enumerate(self.leaves)}

    def nleaves(self) -> int:
        return len(self.leaves)

    def maxlevel(self) -> int:
        return max(k.level for k in self.leaves)

    def find_leaf(self, key: MortonKey) -> Optional[int]:
        """0-based index of ``key`` in ``leaves``, or ``None`` (``src/forest.jl:1332``)."""
        return self._index.get(key)

    def isleaf(self, key: MortonKey) -> bool:
        return key in self._index

    # -- roots ---------------------------------------------------------------
    def root_position(self, root: int) -> Tuple[int, ...]:
        """0-based brick position of a root, dimension 1 fastest (``src/forest.jl:1266``)."""
        pos = []
        for r in self.roots:
            pos.append(root % r)
            root //= r
        return tuple(pos)

    def root_index(self, pos: Sequence[int]) -> int:
        idx, stride = 0, 1
        for p, r in zip(pos, self.roots):
            idx += p * stride
            stride *= r
        return idx

    # -- the seam (quarter or half turn) ---------------------------------------
    def hasrotating(self) -> bool:
        return self.rotating[0] != 0

    def ishalfturn(self) -> bool:
        return self.rotating[1] < 0

    def seam_plane(self) -> Tuple[int, int]:
        """The seam's plane ``(d1, d2)`` as 0-based dimensions."""
        return self.rotating[0] - 1, abs(self.rotating[1]) - 1

    def rotating_dims(self):
        """The ``rotating`` keyword's pair (1-based), or ``None``."""
        return (self.rotating[0], self.rotating[1]) if self.hasrotating() and \
            not self.ishalfturn() else None

    def halfturn_dims(self):
        return (self.rotating[0], -self.rotating[1]) if self.ishalfturn() else None

    def seam_orientation(self, g: Sequence[int]) -> int:
        """The orientation of the naive node at global level coordinates
        ``g`` (``src/forest.jl:1406-1413``)."""
        if not self.hasrotating():
            return 0
        d1, d2 = self.seam_plane()
        if self.ishalfturn():
            return 2 if g[d1] < 0 else 0
        a, b = g[d1] < 0, g[d2] < 0
        return (2 if b else 1) if a else (3 if b else 0)

    def stepped_node(self, k: MortonKey, delta: Sequence[int]):
        """The real node one step from ``k`` in ``delta`` in global level
        coordinates, and its orientation: the naive step mapped back across
        the seam it crosses (``unrotate_node``, ``stepped_node``,
        ``src/forest.jl:1415-1499``).  Periodic wraps and high faces are
        left to ``neighbor_anchor``."""
        lvl = k.level
        rp = self.root_position(k.root)
        g = [(rp[d] << lvl) + k.coords[d] + delta[d] for d in range(self.D)]
        r = self.seam_orientation(g)
        if r == 0:
            return g, 0
        d1, d2 = self.seam_plane()
        n2 = self.roots[d2] << lvl if self.ishalfturn() else 0
        g1, g2 = g[d1], g[d2]
        if r == 1:
            g[d1], g[d2] = g2, -1 - g1
        elif r == 3:
            g[d1], g[d2] = -1 - g2, g1
        else:
            g[d1], g[d2] = -1 - g1, n2 - 1 - g2
        return g, r

    def turns(self, k: MortonKey, delta: Sequence[int]) -> int:
        """The orientation of the region of ``k`` in ``delta``: 0 off the
        seam, else the quarter turns that carry the real leaves there to
        where ``k`` sees them (``Crossing.turns``)."""
        return self.stepped_node(k, delta)[1] if self.hasrotating() else 0

    # -- neighbours ----------------------------------------------------------
    def neighbor_anchor(self, k: MortonKey, delta: Sequence[int]):
        """The same-level node one step from ``k`` in ``delta`` as
        ``(root, coords)``, wrapping periodic dimensions and crossing a seam
        into the real node; ``None`` beyond a non-periodic face that is not
        the seam (``src/forest.jl:1501-1520``)."""
        lvl = k.level
        g, _ = self.stepped_node(k, delta)
        for d in range(self.D):
            n = self.roots[d] << lvl
            if (g[d] < 0 or g[d] >= n) and not self.periodic[d]:
                return None
        wrapped = [g[d] % (self.roots[d] << lvl) for d in range(self.D)]
        mask = (1 << lvl) - 1
        rootpos = [w >> lvl for w in wrapped]
        return self.root_index(rootpos), tuple(w & mask for w in wrapped)

    def find_covering_leaf(self, root: int, lvl: int, coords: Tuple[int, ...]) -> Optional[int]:
        """The leaf that is the node or its nearest coarser ancestor
        (``src/forest.jl:1632-1642``)."""
        c = coords
        for l in range(lvl, -1, -1):
            i = self._index.get(MortonKey(root, l, c))
            if i is not None:
                return i
            c = tuple(x >> 1 for x in c)
        return None

    def _collect_touching(self, out: List[MortonKey], root: int, lvl: int,
                          coords: Tuple[int, ...], delta: Sequence[int]):
        """Children of a refined node touching its boundary in ``delta``,
        recursively (``src/forest.jl:1650-1670``)."""
        D = self.D
        cl = lvl + 1
        base = [2 * coords[d] + (1 if delta[d] == -1 else 0) for d in range(D)]
        spans = [(0, 1) if delta[d] == 0 else (0,) for d in range(D)]
        # Julia's Iterators.product iterates the first dimension fastest.
        for rev in itertools.product(*reversed(spans)):
            off = tuple(reversed(rev))
            cc = tuple(base[d] + off[d] for d in range(D))
            key = MortonKey(root, cl, cc)
            if key in self._index:
                out.append(key)
            else:
                self._collect_touching(out, root, cl, cc, delta)
        return out

    def turned_neighbors(self, k: MortonKey, delta: Sequence[int]):
        """``(turns, keys)``: the real leaves abutting ``k`` across the face,
        edge or corner ``delta`` and the orientation that carries them to
        where ``k`` sees them (``oriented_neighbors``,
        ``src/forest.jl:1718-1740``).  Across a seam ``turns`` is the
        region's orientation even when there is no leaf; the search for
        finer leaves runs in the real frame, in the direction from them back
        to ``k``'s image."""
        anchor = self.neighbor_anchor(k, delta)
        r = self.turns(k, delta)
        if anchor is None:
            return r, []
        root, coords = anchor
        i = self.find_covering_leaf(root, k.level, coords)
        if i is not None:
            return r, [self.leaves[i]]
        dreal = real_direction(delta, r, *self.seam_plane()) if r else delta
        return r, self._collect_touching([], root, k.level, coords, dreal)

    def oriented_neighbors(self, k: MortonKey, delta: Sequence[int]) -> List[MortonKey]:
        """The leaves abutting ``k`` across the face, edge or corner
        ``delta`` (``neighbor_keys``): the keys of ``turned_neighbors``."""
        return self.turned_neighbors(k, delta)[1]

    neighbor_keys = oriented_neighbors

    def wall_direction(self, k: MortonKey, delta: Sequence[int]):
        """``(delta', walls)``: ``walls[d]`` is the reflecting or outflow face
        that stepping by ``delta[d]`` leaves through (``OUTER`` otherwise) and
        ``delta'`` zeroes those components (``src/forest.jl:1617-1630``)."""
        n = 1 << k.level
        rp = self.root_position(k.root)
        walls = []
        for d in range(self.D):
            if delta[d] == 0 or self.periodic[d]:
                walls.append(OUTER)
                continue
            stepped = k.coords[d] + delta[d]
            exits = (stepped < 0 and rp[d] == 0) if delta[d] < 0 else \
                    (stepped >= n and rp[d] == self.roots[d] - 1)
            walls.append(self.faces[d][0 if delta[d] < 0 else 1] if exits else OUTER)
        dprime = tuple(delta[d] if walls[d] == OUTER else 0 for d in range(self.D))
        return dprime, tuple(walls)

    # -- mutation ------------------------------------------------------------
    def refine(self, keys):
        """Replace each leaf in ``keys`` by its children (``src/forest.jl:1761``)."""
        if isinstance(keys, MortonKey):
            keys = (keys,)
        targets = set()
        for k in keys:
            if k not in self._index:
                raise ValueError(f"cannot refine {k}: not a leaf of the forest")
            if k.level >= MAX_LEVEL:
                raise ValueError(f"cannot refine {k}: already at MAX_LEVEL")
            targets.add(k)
        if not targets:
            return self
        new = []
        for k in self.leaves:
            if k in targets:
                new.extend(sortedchildkeys(k))
            else:
                new.append(k)
        self.leaves = new
        self.generation += 1
        self._reindex()
        return self

    def coarsen(self, keys):
        """Replace the children of each key by the key (``src/forest.jl:1792``)."""
        if isinstance(keys, MortonKey):
            keys = (keys,)
        parentof = {}
        for p in keys:
            for c in sortedchildkeys(p):
                if c not in self._index:
                    raise ValueError(f"cannot coarsen {p}: child {c} is not a leaf")
                parentof[c] = p
        if not parentof:
            return self
        new, emitted = [], set()
        for k in self.leaves:
            p = parentof.get(k)
            if p is None:
                new.append(k)
            elif p not in emitted:
                new.append(p)
                emitted.add(p)
        self.leaves = new
        self.generation += 1
        self._reindex()
        return self

    def balance_slack(self, k: MortonKey, delta: Sequence[int]) -> int:
        """How many levels two adjacent leaves may differ by: one, but none
        across a seam's face, where the leaves conform
        (``src/forest.jl:1882-1883``)."""
        if self.hasrotating() and sum(1 for x in delta if x) == 1 and self.turns(k, delta):
            return 0
        return 1

    def balance(self):
        """2:1 balance across faces, edges and corners, and conformity at a
        seam's face (``src/forest.jl:1837-1868``)."""
        dirs = alldirections(self.D)
        seam = self.hasrotating()
        while True:
            found = []
            seen = set()
            for k in self.leaves:
                if k.level < 2 and not (k.level == 1 and seam):
                    continue
                for delta in dirs:
                    anchor = self.neighbor_anchor(k, delta)
                    if anchor is None:
                        continue
                    i = self.find_covering_leaf(anchor[0], k.level, anchor[1])
                    if i is None:
                        continue
                    nb = self.leaves[i]
                    if nb.level < k.level - self.balance_slack(k, delta) and nb not in seen:
                        seen.add(nb)
                        found.append(nb)
            if not found:
                break
            self.refine(found)
        return self

    def isbalanced(self) -> bool:
        dirs = alldirections(self.D)
        for k in self.leaves:
            for delta in dirs:
                for nb in self.oriented_neighbors(k, delta):
                    if abs(nb.level - k.level) > self.balance_slack(k, delta):
                        return False
        return True

    # -- geometry (src/geometry.jl) -----------------------------------------
    def _anchors(self):
        """Per dimension the integer anchor ``m``: zero is a node of the
        level-0 grid at index ``m`` (``src/geometry.jl:position_anchors``)."""
        out = []
        for d in range(self.D):
            lo, hi = Fraction(self.extents[d][0]), Fraction(self.extents[d][1])
            n = self.roots[d] * self.N
            m = -lo * n / (hi - lo)
            out.append(int(m) if m.denominator == 1 and 0 <= m <= n else 0)
        return out

    def block_low(self, k: MortonKey) -> Tuple[float, ...]:
        m = self._anchors()
        return tuple(0.0 if m[d] > 0 else self.extents[d][0] for d in range(self.D))

    def block_base(self, k: MortonKey) -> Tuple[int, ...]:
        rp = self.root_position(k.root)
        m = self._anchors()
        lvl = k.level
        return tuple(((rp[d] << lvl) + k.coords[d]) * self.N - (m[d] << lvl)
                     for d in range(self.D))

    def spacing(self, lvl: int, dtype=float) -> float:
        """``(hi - lo) / roots / N / 2^lvl`` rounded step by step in ``dtype``
        (``src/geometry.jl:root_spacing``, ``spacing``)."""
        import numpy as np
        T = np.dtype(dtype).type
        h = (T(self.extents[0][1]) - T(self.extents[0][0])) / T(self.roots[0]) / T(self.N)
        return h / T(1 << lvl)

    def block_extent(self, k: MortonKey) -> Tuple[Tuple[float, float], ...]:
        lo, B = self.block_low(k), self.block_base(k)
        h = float(self.spacing(k.level))
        return tuple((nodeposition(lo[d], h, B[d], 1, 1), nodeposition(lo[d], h, B[d], self.N + 1, 1))
                     for d in range(self.D))


def _check_rotating(rotating, roots, periodic, reflecting, outflow):
    """The ``rotating`` keyword as the forest stores it, ``(0, 0)`` for none
    (``check_rotating``, ``src/forest.jl:740-784``)."""
    if rotating is None:
        return (0, 0)
    D = len(roots)
    d1, d2 = int(rotating[0]), int(rotating[1])
    rot = (d1, d2)
    if D < 2:
        raise ValueError(f"rotating = {rot} needs at least two dimensions, and this forest "
                         f"has {D}: the rotation turns the plane of two dimensions about the "
                         "line where their low faces meet")
    if not (1 <= d1 <= D and 1 <= d2 <= D):
        raise ValueError(f"rotating = {rot} names a dimension outside 1:{D}: the pair "
                         "(d1, d2) is the plane of the rotation, two of the forest's own "
                         "dimensions")
    if d1 == d2:
        raise ValueError(f"rotating = {rot} names dimension {d1} twice: the rotation turns "
                         "the plane of two different dimensions")
    if roots[d1 - 1] != roots[d2 - 1]:
        raise ValueError(f"rotating = {rot} needs as many roots along dimension {d1} as "
                         f"along {d2}, got {roots[d1 - 1]} and {roots[d2 - 1]}: the seam "
                         f"glues the low face of {d1} onto the low face of {d2}, root for "
                         "root")
    for d in (d1, d2):
        if periodic[d - 1]:
            raise ValueError(f"rotating = {rot}, but dimension {d} is periodic: its low "
                             "face is the rotating seam, and a periodic dimension has no "
                             "faces")
        if any(reflecting[d - 1]):
            raise ValueError(f"rotating = {rot}, but dimension {d} has a reflecting face: "
                             "its low face is the rotating seam and its high face stays "
                             "outer; a reflecting high wall with the rotation is an open "
                             "question, not implemented")
        if any(outflow[d - 1]):
            raise ValueError(f"rotating = {rot}, but dimension {d} has an outflow face: "
                             "its low face is the rotating seam and its high face stays "
                             "outer; an outflow high face with the rotation is an open "
                             "question, not implemented")
    return (d1, d2)


def _check_halfturn(halfturn, rotating, roots, periodic, reflecting, outflow):
    """The ``halfturn`` keyword as the forest stores it, ``(d1, -d2)``
    (``check_halfturn``, ``src/forest.jl:788-834``)."""
    if rotating is not None:
        raise ValueError(f"rotating = {tuple(rotating)} and halfturn = {tuple(halfturn)} are "
                         "both given: a forest has one seam at most. Declare one.")
    D = len(roots)
    d1, d2 = int(halfturn[0]), int(halfturn[1])
    ht = (d1, d2)
    if D < 2:
        raise ValueError(f"halfturn = {ht} needs at least two dimensions, and this forest "
                         f"has {D}")
    if not (1 <= d1 <= D and 1 <= d2 <= D):
        raise ValueError(f"halfturn = {ht} names a dimension outside 1:{D}: the pair "
                         "(d1, d2) is the plane of the rotation")
    if d1 == d2:
        raise ValueError(f"halfturn = {ht} names dimension {d1} twice: the half turn glues "
                         "the low face of the first dimension to itself, reversed along "
                         "the second, a different one")
    if roots[d2 - 1] % 2:
        raise ValueError(f"halfturn = {ht} needs an even number of roots along dimension "
                         f"{d2}, got {roots[d2 - 1]}: the axis of the turn lies on the "
                         "centre plane, and it must lie on a root boundary")
    for d in (d1, d2):
        if periodic[d - 1]:
            raise ValueError(f"halfturn = {ht}, but dimension {d} is periodic: a periodic "
                             "dimension with a half turn is an open question, not "
                             "implemented")
        if any(reflecting[d - 1]):
            raise ValueError(f"halfturn = {ht}, but dimension {d} has a reflecting face: "
                             "a reflecting face with the half turn is an open question, not "
                             "implemented")
        if any(outflow[d - 1]):
            raise ValueError(f"halfturn = {ht}, but dimension {d} has an outflow face: "
                             "an outflow face with the half turn is an open question, not "
                             "implemented")
    return (d1, -d2)


def nodeposition(lo, h, B: int, I: int, c: int, dtype=float):
    """Position of stored index ``I`` (1-based) of a block with integer base
    ``B``: ``fma(m, s, lo)`` with ``m = B + I - 1, s = h`` along a vertex-like
    dimension and ``m = 2(B + I - 1) + 1, s = h/2`` along a cell-like one,
    rounded once (``src/storage.jl:1008-1017``)."""
    import numpy as np
    T = np.dtype(dtype).type
    k = B + I - 1
    if c == 1:
        m, s = k, T(h)
    else:
        m, s = 2 * k + 1, T(h) / T(2)
    exact = Fraction(float(T(m))) * Fraction(float(s)) + Fraction(float(T(lo)))
    return _round_fraction(exact, np.dtype(dtype))


def _round_fraction(q: Fraction, dtype) -> float:
    """Round an exact rational once, to nearest-even, into ``dtype``."""
    import numpy as np
    if np.dtype(dtype) == np.float64:
        return float(q)                       # int/int true division rounds once
    return float(round_rational_f32(q.numerator, q.denominator))


def round_rational_f32(num: int, den: int):
    """``num/den`` rounded once to the nearest ``float32``, ties to even.

    The float64 quotient may sit a double rounding away from the answer, so
    the three ``float32`` values around it are compared exactly."""
    import numpy as np
    q = Fraction(num, den)
    a = np.float32(float(q))
    cands = [a, np.nextafter(a, np.float32(np.inf)), np.nextafter(a, np.float32(-np.inf))]

    def rank(c):
        odd = int(np.array(c, dtype=np.float32).view(np.uint32)) & 1
        return (abs(Fraction(float(c)) - q), odd)
    return min(cands, key=rank)
