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

from typing import Callable, Optional, Sequence, Tuple

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
                 parity=None, device="cpu"):
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
        self.factors_host = parityfactors(self.T, table, D)
        self.device = torch.device(device)
        shape = (forest.nleaves(), self.nvars) + tuple(reversed(self.stored))
        # zero-filled, as the reference's first touch (src/storage.jl:1433-1446)
        self.work = torch.zeros(shape, dtype=_TORCH[self.T], device=self.device)
        # the factor table column-major (nvars fastest), as the kernel reads it
        self.factors = torch.from_numpy(np.asfortranarray(self.factors_host).ravel(order="F").copy()).to(self.device)

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
