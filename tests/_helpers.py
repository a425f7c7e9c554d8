"""Shared helpers of the tests: the reference's test meshes and oracles.

Restated from the reference's ``test/ghost_oracles.jl`` (``nested_forest``
:275-291, ``refine_where!`` :332-343, ``periodic_vs_tiled`` :358-401,
``exchange_error`` :111-118, ``scalarpoly`` :87) and ``test/helpers/ghost.jl``
(awkward data, NaN compared as one pattern, :191-219).
"""
from __future__ import annotations

import math

import numpy as np
import torch

import oracle
from treeamr import FieldSet, Forest, GhostSchedule, Operators


def nested_forest(D, N=4, roots=4, periodic=None):
    """Three levels meeting: two nested refinement regions around 1.5."""
    f = Forest((roots,) * D, N=N, periodic=periodic or (False,) * D,
               extents=[(0.0, float(roots))] * D)
    center = (1.5,) * D

    def near(c, r):
        return all(abs(c[d] - center[d]) <= r for d in range(D))

    for _ in range(2):
        targets = []
        for k in f.leaves:
            c = tuple((a + b) / 2 for a, b in f.block_extent(k))
            if (k.level == 0 and near(c, 1.0)) or (k.level == 1 and near(c, 0.3)):
                targets.append(k)
        if not targets:
            break
        f.refine(targets)
        f.balance()
    return f


def makepoly(D, deg):
    """A polynomial of total degree ``deg`` per variable (``scalarpoly``)."""
    def f(x, v):
        return sum(0.7 * (d + 1) + 0.31 * (d + 2) * x[d] ** e
                   for d in range(D) for e in range(deg + 1)) + 0.5 * v
    return f


def exact_values(fs, fn):
    fs.fill_by_coordinates(fn)
    return fs.work.detach().cpu().numpy().copy()


def ghost_mask(fs):
    m = np.ones(tuple(reversed(fs.stored)), bool)
    m[fs.interior()] = False
    return m


def boundary_from(exact):
    """The hook of ``boundary_by_coordinates``, from precomputed exact values."""
    def bv(host, fs, regions):
        for r in regions:
            sl = tuple(slice(a - 1, z) for a, z in reversed(r.region))
            host[(r.block, slice(None)) + sl] = exact[(r.block, slice(None)) + sl]
    return bv


def exchange_error(forest, ops, fn, *, nvars=2, G=1, T=np.float64):
    """Fill with ``fn``, poison the ghosts, run the oracle fill with the exact
    boundary, report the worst deviation anywhere."""
    fs = FieldSet(forest, nvars, G=G, T=T)
    exact = exact_values(fs, fn)
    host = exact.copy()
    host[:, :, ghost_mask(fs)] = np.nan
    fs.work.copy_(torch.from_numpy(host))
    sched = GhostSchedule(fs, ops)
    out = oracle.fill_fieldset(fs, sched, boundary_values=boundary_from(exact))
    if np.isnan(out).any():
        return math.inf
    return float(np.max(np.abs(out - exact)))


def periodic_vs_tiled(D, M, *, N=4, G=1, nvars=2, ops=None, passes=2):
    """An ``M``-root periodic domain against the middle tile of an explicit
    ``3M``-root tiling; returns ``(maxdiff, ncells)`` or ``None``."""
    ops = ops or Operators(prolongation=2, restriction=2)
    L = float(M)

    def seam(ext, lvl):
        c = [(a + b) / 2 for a, b in ext]
        return lvl < passes and all(min(c[d] % L, L - c[d] % L) < 0.55 for d in range(D))

    def refine(f):
        for _ in range(passes):
            targets = [k for k in f.leaves if seam(f.block_extent(k), k.level)]
            if not targets:
                break
            f.refine(targets)
            f.balance()
        return f

    periodic = refine(Forest((M,) * D, N=N, periodic=(True,) * D, extents=[(0.0, L)] * D))
    tiled = refine(Forest((3 * M,) * D, N=N, extents=[(-L, 2 * L)] * D))

    def data(x, v):
        return sum(np.sin(3.1 * np.mod(x[d], L) + 0.7 * (v + 1)) * (1 + 0.3 * (d + 1))
                   for d in range(D))

    fsp = FieldSet(periodic, nvars, G=G)
    fsp.fill_by_coordinates(data)
    outp = oracle.fill_fieldset(fsp, GhostSchedule(fsp, ops))
    fst = FieldSet(tiled, nvars, G=G)
    exact = exact_values(fst, data)
    outt = oracle.fill_fieldset(fst, GhostSchedule(fst, ops), boundary_values=boundary_from(exact))

    def lower(f, k):
        return tuple(e[0] for e in f.block_extent(k))
    index = {(k.level, lower(tiled, k)): b for b, k in enumerate(tiled.leaves)}
    worst, ncells = 0.0, 0
    for b, k in enumerate(periodic.leaves):
        tb = index.get((k.level, lower(periodic, k)))
        if tb is None:
            return None
        worst = max(worst, float(np.max(np.abs(outp[b] - outt[tb]))))
        ncells += outp[b].size
    return worst, ncells


def awkward_fill(shape, dtype, seed=0):
    """Data with +-0, NaN, +-Inf and subnormals among uniform values
    (``test/helpers/ghost.jl:191-219``)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1, 1, size=shape).astype(dtype)
    flat = a.reshape(-1)
    n = flat.size
    tiny = np.finfo(dtype).tiny
    specials = np.array([0.0, -0.0, np.nan, np.inf, -np.inf, tiny / 4, -tiny / 8, tiny],
                        dtype=dtype)
    idx = rng.choice(n, size=max(1, n // 50), replace=False)
    flat[idx] = specials[rng.integers(0, len(specials), size=len(idx))]
    return a


def nanbits(a: np.ndarray) -> np.ndarray:
    """Bits of every value, every NaN mapped to one pattern."""
    a = a.copy()
    a[np.isnan(a)] = np.nan
    return a.view(np.uint64 if a.dtype == np.float64 else np.uint32)


class Geometry:
    """Exact positions as integers: root units times ``scale = 2 N 2^L``, L
    the finest level, so cell centres and half fine spacings are whole
    (the oracle's ``exact_point`` and ``leafbox``, wrapped where periodic)."""

    def __init__(self, forest):
        self.f = forest
        self.L = max(k.level for k in forest.leaves)
        self.scale = 2 * forest.N * (1 << self.L)

    def low(self, k):
        rp = self.f.root_position(k.root)
        return [((rp[d] << k.level) + k.coords[d]) * (self.scale >> k.level)
                for d in range(self.f.D)]

    def wrap(self, d, x):
        f = self.f
        return x % (f.roots[d] * self.scale) if f.periodic[d] else x

    def points(self, k, G, c, N):
        """Per dimension the positions of own indices 1..N+c (stored G+1..)."""
        unit = 1 << (self.L - k.level)        # half a cell of this level
        lo = self.low(k)
        out = []
        for d in range(self.f.D):
            i = np.arange(N + c[d])           # own index 0.. (stored G+1+i)
            x = lo[d] + (2 * i + (0 if c[d] == 1 else 1)) * unit
            out.append(self.wrap(d, x))
        return out
