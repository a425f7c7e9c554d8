"""Field storage: one array holding every leaf block with its ghosts.

Restates ``src/storage.jl``:

* ``FieldSet`` -- ``src/storage.jl:364-472``: ``work`` is
  ``(S_1, ..., S_D, nvars, nblocks)`` column-major with ``S_d = N + 2G_d + c_d``
  (``storedsize``, ``src/storage.jl:865-872``).  Here it is a torch tensor of
  shape ``(nblocks, nvars, S_D, ..., S_1)`` in C order, which is the same
  bytes: index 1 fastest, then the variable, then the block.
* ``staggers`` -- ``src/storage.jl:165``.
* ``Parity`` and ``parityfactors`` / ``mirrorcolumn`` -- ``src/storage.jl:171-555``.
* ``coordinates`` through ``nodeposition`` -- ``src/storage.jl:1008-1017``.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple

import numpy as np
import torch

from .forest import Forest, REFLECTING, nodeposition

EvenParity, OddParity, NoParity = "EvenParity", "OddParity", "NoParity"

_TORCH = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}


def cellcentered(D: int) -> Tuple[str, ...]:
    return ("cell",) * D


def vertexcentered(D: int) -> Tuple[str, ...]:
    return ("vertex",) * D


def facecentered(D: int, d: int) -> Tuple[str, ...]:
    """Vertex-like along dimension ``d`` (1-based), cell-like along the others:
    a flux through the faces normal to ``d``."""
    return tuple("vertex" if e == d - 1 else "cell" for e in range(D))


def edgecentered(D: int, d: int) -> Tuple[str, ...]:
    """Cell-like along dimension ``d`` (1-based), vertex-like along the others:
    a quantity on the edges that run along ``d``."""
    return tuple("cell" if e == d - 1 else "vertex" for e in range(D))


def staggers(centering: Sequence[str]) -> Tuple[int, ...]:
    """``c_d = 1`` along a vertex-like dimension, 0 along a cell-like one."""
    for c in centering:
        if c not in ("cell", "vertex"):
            raise ValueError(f"centering must be 'cell' or 'vertex' per dimension, got {c!r}")
    return tuple(1 if c == "vertex" else 0 for c in centering)


def ghostwidths(G, D: int) -> Tuple[int, ...]:
    if isinstance(G, int):
        G = (G,) * D
    G = tuple(int(g) for g in G)
    if len(G) != D:
        raise ValueError(f"G must have one width per dimension: got {len(G)} for D={D}")
    if any(g < 0 for g in G):
        raise ValueError(f"G must be nonnegative, got {G}")
    return G


def storedsize(N: int, G: Sequence[int], c: Sequence[int]) -> Tuple[int, ...]:
    """``N + 2G_d + c_d``, refusing ``N < 2G_d`` (``src/storage.jl:865-872``)."""
    if not all(N >= 2 * g for g in G):
        raise ValueError(f"N must be >= 2G in every dimension, got N={N}, G={tuple(G)}")
    return tuple(N + 2 * g + cd for g, cd in zip(G, c))


def parityfactors(dtype, parities, D: int) -> np.ndarray:
    """The factor table, ``nvars x 3^D`` column-major: column
    ``1 + sum_d s_d 3^(d-1)`` for mirror state ``s``; entry the product over
    ``d`` of 1, the parity sign, or ``(1+sigma)/2`` (``src/storage.jl:536-551``)."""
    nstates = 3 ** D
    f = np.empty((len(parities), nstates), dtype=dtype)
    for v, p in enumerate(parities):
        for col in range(nstates):
            x = 1
            for d in range(D):
                state = (col // 3 ** d) % 3
                sigma = -1 if p[d] == OddParity else 1
                x *= 1 if state == 0 else sigma if state == 1 else (1 + sigma) // 2
            f[v, col] = x
    return f


def mirrorcolumn(state: Sequence[int]) -> int:
    """1-based factor column of a mirror state (``src/storage.jl:553-555``)."""
    return 1 + sum(int(s) * 3 ** d for d, s in enumerate(state))


# --- seams: the rotation tables (src/storage.jl:557-760) -----------------------

def signed_map(m, nvars: int, name: str, turn: str) -> List[int]:
    """A signed variable map checked for its shape: one nonzero integer per
    variable, naming every variable once (``src/storage.jl:632-652``)."""
    if not isinstance(m, (list, tuple)):
        raise ValueError(f"{name} must be a vector or tuple with one signed variable index per "
                         f"variable, got a {type(m).__name__}")
    if len(m) != nvars:
        raise ValueError(f"{name} must have one entry per variable: got {len(m)} for "
                         f"nvars = {nvars}")
    q = []
    for x in m:
        if isinstance(x, bool) or not isinstance(x, (int, np.integer)):
            raise ValueError(f"each {name} entry must be a nonzero integer, a signed variable "
                             f"index; got {x!r}")
        q.append(int(x))
    if sorted(abs(x) for x in q) != list(range(1, nvars + 1)):
        raise ValueError(f"{name} = {tuple(q)} is not a signed permutation of 1:{nvars}: {turn} "
                         "sends each variable to plus or minus exactly one variable")
    return q


def composed_rotation(steps, nvars: int):
    """After the steps, target variable ``v`` reads variable ``sigma[v]`` of
    the set the last step reads from, times ``sign[v]`` (1-based variables;
    ``src/storage.jl:684-694``)."""
    sigma = list(range(1, nvars + 1))
    sign = [1] * nvars
    for q in steps:
        for v in range(nvars):
            x = q[sigma[v] - 1]
            sign[v] *= 1 if x > 0 else -1
            sigma[v] = abs(x)
    return sigma, sign


def symmetric_layout(forest: Forest, G, c) -> bool:
    """Whether the layout turns into itself: always under a half turn, and
    under a quarter turn with equal ghost widths and staggers in the seam's
    plane (``src/storage.jl:571-575``)."""
    if forest.ishalfturn():
        return True
    d1, d2 = forest.seam_plane()
    return G[d1] == G[d2] and c[d1] == c[d2]


def _check_rotation_parity(forest: Forest, parities, q, what: str):
    if parities is None:
        return
    for v in range(len(q)):
        w = abs(q[v]) - 1
        for d in range(forest.D):
            if REFLECTING not in forest.faces[d]:
                continue
            if parities[v][d] != parities[w][d]:
                raise ValueError(f"{what} sends variable {v + 1} to variable {w + 1}, but in "
                                 f"dimension {d + 1}, which has a reflecting face, the first has "
                                 f"{parities[v][d]} and the second {parities[w][d]}: a variable "
                                 "and its image under the turn must have the same parity there")


def rotations_of(rotation, forest: Forest, nvars: int, G, c, parities):
    """``src/storage.jl:592-628``."""
    quarter = forest.rotating_dims() is not None
    if rotation is None:
        if quarter:
            raise ValueError(f"this forest has a rotating seam, rotating = "
                             f"{forest.rotating_dims()}, so the field set needs `rotation`: one "
                             "signed variable index per variable, saying which variable, and "
                             "with which sign, each one equals a quarter turn away")
        return None
    q = signed_map(rotation, nvars, "rotation", "a quarter turn")
    if not quarter:
        return q
    if symmetric_layout(forest, G, c):
        sigma, sign = composed_rotation((q, q, q, q), nvars)
        if sigma != list(range(1, nvars + 1)) or any(x != 1 for x in sign):
            raise ValueError(f"rotation = {tuple(q)} turned four times is not the identity: "
                             "four quarter turns are no turn at all")
        _check_rotation_parity(forest, parities, q, "rotation")
    return q


def halfturns_of(halfturn, forest: Forest, nvars: int, parities):
    """``src/storage.jl:658-677``."""
    if halfturn is None:
        if forest.ishalfturn():
            raise ValueError(f"this forest has a half-turn seam, halfturn = "
                             f"{forest.halfturn_dims()}, so the field set needs `halfturn`: one "
                             "signed variable index per variable")
        return None
    q = signed_map(halfturn, nvars, "halfturn", "a half turn")
    if not forest.ishalfturn():
        return q
    sigma, sign = composed_rotation((q, q), nvars)
    if sigma != list(range(1, nvars + 1)) or any(x != 1 for x in sign):
        raise ValueError(f"halfturn = {tuple(q)} applied twice is not the identity: two half "
                         "turns are no turn at all")
    _check_rotation_parity(forest, parities, q, "halfturn")
    return q


def seamtables(dtype, parities, steps, nvars: int, D: int, half=None):
    """``(factors, rotvars)`` of the turned transfers (``src/storage.jl:
    717-740``): ``rotvars[v, r]`` (1-based variables) is the variable
    ``Q^r`` reads for target ``v``, and the factor at column ``mirror column
    + 3^D r`` the target variable's parity factor for that mirror state
    times the sign of ``Q^r``.  ``steps`` is the set's own map three times
    for a symmetric layout, ``None`` for an asymmetric one (zero factors
    and the identity for ``r >= 1``); ``half`` the half turn's own map,
    orientation 2."""
    nstates = 3 ** D
    factors = np.empty((nvars, 4 * nstates), dtype=dtype)
    rotvars = np.empty((nvars, 4), dtype=np.int32)
    for r in range(4):
        if r == 0:
            sigma, sign = list(range(1, nvars + 1)), [1] * nvars
        elif half is not None and r == 2:
            sigma, sign = composed_rotation((half,), nvars)
        elif steps is None or half is not None:
            sigma, sign = list(range(1, nvars + 1)), [0] * nvars
        else:
            sigma, sign = composed_rotation(steps[:r], nvars)
        rotvars[:, r] = sigma
        par = parityfactors(dtype, parities, D)
        for v in range(nvars):
            for col in range(nstates):
                factors[v, col + nstates * r] = dtype.type(int(par[v, col]) * sign[v])
    return factors, rotvars


def check_parity(forest: Forest, nvars: int, parity):
    D = forest.D
    anyreflect = any(REFLECTING in forest.faces[d] for d in range(D))
    if parity is None:
        if anyreflect:
            raise ValueError("the forest has a reflecting face, so the field set needs a "
                             "parity per variable")
        return None
    if len(parity) != nvars:
        raise ValueError(f"parity must have one entry per variable: got {len(parity)} for nvars = {nvars}")
    out = []
    for v, p in enumerate(parity):
        if isinstance(p, str):
            p = (p,) * D
        p = tuple(p)
        if len(p) != D or not all(q in (EvenParity, OddParity, NoParity) for q in p):
            raise ValueError(f"each parity entry must be a Parity or one per dimension, got {p!r}")
        for d in range(D):
            if REFLECTING in forest.faces[d] and p[d] == NoParity:
                raise ValueError(f"variable {v + 1} has NoParity in dimension {d + 1}, which has "
                                 "a reflecting face")
        out.append(p)
    return out


class FieldSet:
    """Block storage for ``nvars`` variables over every leaf of ``forest``."""

    def __init__(self, forest: Forest, nvars: int, *, G, centering=None, T=np.float64,
                 parity=None, rotation=None, halfturn=None, device="cpu"):
        D = forest.D
        if nvars < 1:
            raise ValueError(f"nvars must be positive, got {nvars}")
        self.forest = forest
        self.nvars = int(nvars)
        self.G = ghostwidths(G, D)
        self.centering = tuple(centering) if centering is not None else cellcentered(D)
        self.c = staggers(self.centering)
        self.stored = storedsize(forest.N, self.G, self.c)
        self.T = np.dtype(T)
        if self.T not in _TORCH:
            raise TypeError(f"element type must be float32 or float64, got {self.T}")
        self.generation = forest.generation
        self.parities = check_parity(forest, self.nvars, parity)
        table = self.parities if self.parities is not None else \
            [("EvenParity",) * D] * self.nvars
        self.rotation = rotations_of(rotation, forest, self.nvars, self.G, self.c,
                                     self.parities)
        self.halfturn = halfturns_of(halfturn, forest, self.nvars, self.parities)
        # the variable table of turned transfers, nvars x 4 (None off a seam)
        self.rotvars_host = None
        if forest.ishalfturn():
            self.factors_host, self.rotvars_host = seamtables(self.T, table, None, self.nvars,
                                                              D, half=self.halfturn)
        elif forest.hasrotating():
            q = self.rotation
            steps = (q, q, q) if symmetric_layout(forest, self.G, self.c) else None
            self.factors_host, self.rotvars_host = seamtables(self.T, table, steps,
                                                              self.nvars, D)
        else:
            self.factors_host = parityfactors(self.T, table, D)
        self.device = torch.device(device)
        shape = (forest.nleaves(), self.nvars) + tuple(reversed(self.stored))
        # zero-filled, as the reference's first touch (src/storage.jl:1433-1446)
        self.work = torch.zeros(shape, dtype=_TORCH[self.T], device=self.device)
        # the factor table column-major (nvars fastest), as the kernel reads it
        self.factors = torch.from_numpy(np.asfortranarray(self.factors_host).ravel(order="F").copy()).to(self.device)
        # column-major too: rotvars[v + nvars * r]
        self.rotvars = None if self.rotvars_host is None else torch.from_numpy(
            np.asfortranarray(self.rotvars_host).ravel(order="F").copy()).to(self.device)

    @property
    def D(self) -> int:
        return self.forest.D

    def nblocks(self) -> int:
        return self.work.shape[0]

    def blockkey(self, b: int):
        return self.forest.leaves[b]

    def blockview(self, b: int, v: int) -> torch.Tensor:
        """Block ``b``'s variable ``v`` (0-based) indexed ``[i_D, ..., i_1]``."""
        return self.work[b, v]

    def interior(self) -> Tuple[slice, ...]:
        """Owned range ``G+1 : G+N+c`` per dimension, as slices in the
        tensor's reversed index order."""
        N = self.forest.N
        return tuple(slice(g, g + N + cd) for g, cd in reversed(list(zip(self.G, self.c))))

    def positions(self, b: int) -> Sequence[np.ndarray]:
        """Per dimension ``d`` the positions of stored indices ``1:S_d`` of
        block ``b``, each rounded once (``src/storage.jl:1008-1017``)."""
        f = self.forest
        k = f.leaves[b]
        lo, B = f.block_low(k), f.block_base(k)
        h = f.spacing(k.level, self.T)
        out = []
        for d in range(self.D):
            G = self.G[d]
            pos = [nodeposition(lo[d], h, B[d], i - G, self.c[d], self.T)
                   for i in range(1, self.stored[d] + 1)]
            out.append(np.array(pos, dtype=self.T))
        return out

    def fill_by_coordinates(self, fn: Callable, *, ghosts=True) -> "FieldSet":
        """Set every stored point to ``fn(x, v)`` with ``x`` a tuple of
        per-dimension coordinate arrays broadcast over the block
        (``src/storage.jl:1245-1310``).  ``v`` is 0-based."""
        host = np.zeros(tuple(self.work.shape), dtype=self.T)
        for b in range(self.nblocks()):
            pos = self.positions(b)
            grids = np.meshgrid(*pos, indexing="ij")           # each [i_1, ..., i_D]
            for v in range(self.nvars):
                vals = np.asarray(fn(tuple(grids), v), dtype=np.float64)
                host[b, v] = np.broadcast_to(vals, grids[0].shape).astype(self.T).transpose()
        self.work.copy_(torch.from_numpy(host))
        return self

    def zero(self):
        self.work.zero_()
        return self


def coordinates(fs: FieldSet, b: int, idx: Sequence[int]):
    """Position of the 1-based stored index ``idx`` of block ``b``."""
    pos = fs.positions(b)
    return tuple(pos[d][idx[d] - 1] for d in range(fs.D))


class RotationPair:
    """Two field sets over one forest with a quarter-turn seam, each of which
    turns into the other (``RotationPair``, ``src/storage.jl:742-857``): a set
    whose layout is not symmetric in the seam's plane takes its ghosts across
    the seam from the set of the swapped layout.  Holds the tables of each
    set's targets: for ``a`` the maps ``Q_a``, ``Q_a Q_b`` and ``Q_a Q_b Q_a``
    for one, two and three quarter turns, the odd ones reading ``b``; and
    symmetrically for ``b``.  Fill it with ``fill_ghosts(pair, (sa, sb))``."""

    def __init__(self, a: FieldSet, b: FieldSet):
        if a.forest is not b.forest:
            raise ValueError("the two sets of a RotationPair must be over one forest: each "
                             "fills its ghosts across the seam from the other's blocks")
        forest = a.forest
        if not forest.hasrotating():
            raise ValueError("a RotationPair needs a forest with a rotating seam: without one "
                             "no set turns into another")
        if forest.ishalfturn():
            raise ValueError("a RotationPair needs a quarter-turn seam, and this forest's is a "
                             "half turn: every set turns into itself")
        d1, d2 = forest.seam_plane()

        def swap(t):
            t = list(t)
            t[d1], t[d2] = t[d2], t[d1]
            return tuple(t)
        if a.G != swap(b.G) or a.centering != swap(b.centering):
            raise ValueError("the two sets of a RotationPair must have each other's layout "
                             f"with the seam's dimensions {d1 + 1} and {d2 + 1} exchanged: got "
                             f"G = {a.G} and {b.G}, centering {a.centering} and {b.centering}")
        if symmetric_layout(forest, a.G, a.c):
            raise ValueError("these sets have a layout symmetric in the seam's dimensions, so "
                             "each turns into itself and fills its ghosts alone")
        if a.nvars != b.nvars:
            raise ValueError("the two sets of a RotationPair must have the same number of "
                             f"variables: got {a.nvars} and {b.nvars}")
        if a.T != b.T:
            raise ValueError("the two sets of a RotationPair must store one element type: got "
                             f"{a.T} and {b.T}")
        if a.work.device != b.work.device:
            raise ValueError("the two sets of a RotationPair must live on one device")
        qa, qb = a.rotation, b.rotation
        sigma, sign = composed_rotation((qa, qb, qa, qb), a.nvars)
        if sigma != list(range(1, a.nvars + 1)) or any(x != 1 for x in sign):
            raise ValueError(f"the rotations of the pair, {tuple(qa)} and {tuple(qb)}, composed "
                             "four times as Q_a Q_b Q_a Q_b are not the identity")
        for x, y, q, what in ((a, b, qa, "the first set"), (b, a, qb, "the second set")):
            if x.parities is not None and y.parities is not None:
                for v in range(len(q)):
                    w = abs(q[v]) - 1
                    for d in range(forest.D):
                        if REFLECTING in forest.faces[d] and x.parities[v][d] != y.parities[w][d]:
                            raise ValueError(f"the rotation of {what} sends variable {v + 1} to "
                                             f"variable {w + 1} of the other, which must have "
                                             f"the same parity in dimension {d + 1}")
        self.a, self.b = a, b

        def table(fs):
            return fs.parities if fs.parities is not None else \
                [("EvenParity",) * forest.D] * fs.nvars
        self.afactors_host, self.arotvars_host = seamtables(a.T, table(a), (qa, qb, qa),
                                                            a.nvars, forest.D)
        self.bfactors_host, self.brotvars_host = seamtables(b.T, table(b), (qb, qa, qb),
                                                            b.nvars, forest.D)
        dev = a.work.device

        def col(x):
            return torch.from_numpy(np.asfortranarray(x).ravel(order="F").copy()).to(dev)
        self.afactors, self.bfactors = col(self.afactors_host), col(self.bfactors_host)
        self.arotvars, self.brotvars = col(self.arotvars_host), col(self.brotvars_host)

    def to(self, device):
        """The tables on ``device`` (the sets' arrays move with the sets)."""
        for name in ("afactors", "bfactors", "arotvars", "brotvars"):
            setattr(self, name, getattr(self, name).to(device))
        return self

