"""Seeded synthetic meshes and data of the ghost-fill workloads.

The reference measures on synthetic meshes only (``bench/*.jl``); these are
the meshes the engine is tested and benchmarked on, each built the way the
reference's tests build theirs (``refine!`` then ``balance!``,
``test/ghost_oracles.jl:275-343``).
"""
from __future__ import annotations

import math
import numpy as np

from .forest import Forest
from .operators import Operators
from .storage import FieldSet


def _box_meets_sphere(ext, center, r) -> bool:
    lo2 = hi2 = 0.0
    for (a, b), c in zip(ext, center):
        near = min(max(c, a), b)
        lo2 += (near - c) ** 2
        hi2 += max((a - c) ** 2, (b - c) ** 2)
    return lo2 <= r * r <= hi2


def refine_where(forest: Forest, pred, levels):
    """For each level in ``levels``: refine every leaf of that level where
    ``pred(extent)`` holds, then balance."""
    for lvl in levels:
        targets = [k for k in forest.leaves if k.level == lvl and pred(forest.block_extent(k))]
        if not targets:
            continue
        forest.refine(targets)
        forest.balance()
    return forest


def quadrant_forest(seed: int = 0) -> Forest:
    """2-D, 4x4 periodic roots, N = 8; a seeded quarter of the roots refined
    once, then balanced (the CPU-sized correctness mesh)."""
    rng = np.random.default_rng(seed)
    f = Forest((4, 4), N=8, periodic=(True, True), extents=((0.0, 4.0), (0.0, 4.0)))
    roots = list(f.leaves)
    pick = rng.choice(len(roots), size=len(roots) // 4, replace=False)
    f.refine([roots[i] for i in sorted(pick)])
    f.balance()
    return f


def sphere_forest(roots: int = 8, N: int = 16, levels: int = 3, radius: float = 0.25,
                  periodic: bool = True) -> Forest:
    """3-D, ``roots^3`` roots over the unit cube, periodic unless asked not to
    be (then every face is an outer face, filled by the boundary hook);
    ``levels`` nested refinements of every leaf whose box meets the sphere
    ``|x - 1/2| = radius``, each followed by balance."""
    f = Forest((roots,) * 3, N=N, periodic=(periodic,) * 3, extents=((0.0, 1.0),) * 3)
    c = (0.5, 0.5, 0.5)
    return refine_where(f, lambda ext: _box_meets_sphere(ext, c, radius), range(levels))


def sphere_data(seed: int = 1, noise: float = 1e-3):
    """``sin(2 pi x) sin(2 pi y) sin(2 pi z)`` plus seeded uniform noise."""
    rng = np.random.default_rng(seed)

    def fn(x, v):
        base = np.sin(2 * math.pi * x[0]) * np.sin(2 * math.pi * x[1]) * np.sin(2 * math.pi * x[2])
        return base + noise * rng.uniform(-1.0, 1.0, size=np.shape(x[0]))
    return fn


def _stored_positions(fs: FieldSet, device):
    """Per dimension a float64 tensor (nblocks, S_d) of every block's stored
    positions: ``lo + (B + I - 1) h`` along a vertex-like dimension and
    ``lo + (B + I - 1/2) h`` along a cell-like one.  On the dyadic extents of
    the synthetic meshes both are exact, so they equal the single-rounding
    positions of ``FieldSet.positions``."""
    import torch
    f = fs.forest
    nb = f.nleaves()
    B = torch.tensor([f.block_base(k) for k in f.leaves], dtype=torch.float64, device=device)
    h = torch.tensor([float(f.spacing(k.level)) for k in f.leaves], dtype=torch.float64,
                     device=device)
    lo = f.block_low(f.leaves[0]) if nb else (0.0,) * f.D
    out = []
    for d in range(f.D):
        i = torch.arange(fs.stored[d], dtype=torch.float64, device=device) - fs.G[d]
        off = 0.0 if fs.c[d] == 1 else 0.5
        out.append(lo[d] + (B[:, d:d + 1] + i[None, :] + off) * h[:, None])
    return out


def config_fill(fs: FieldSet, workload: str, seed: int = 1) -> FieldSet:
    """Every stored point of a 3-D field set set to a workload's stated data,
    computed on the field set's device: ``"sphere"`` is ``sin(2 pi x)
    sin(2 pi y) sin(2 pi z)`` plus seeded uniform noise of 1e-3 (every
    variable), ``"walls"`` Gaussian bumps of width 0.05 at the two seeded
    refinement centres plus seeded uniform noise in [-1, 1]."""
    import torch
    dev = fs.work.device
    X = _stored_positions(fs, dev)
    g = torch.Generator(device=dev).manual_seed(seed)
    nb = fs.nblocks()
    shape = (nb,) + tuple(reversed(fs.stored))
    if workload == "sphere":
        s = [torch.sin(2 * math.pi * x) for x in X]
        base = (s[2][:, :, None, None] * s[1][:, None, :, None] * s[0][:, None, None, :])
        for v in range(fs.nvars):
            noise = torch.empty(shape, dtype=torch.float64, device=dev).uniform_(
                -1e-3, 1e-3, generator=g)
            fs.work[:, v].copy_(base + noise)
    elif workload == "walls":
        bump = torch.zeros(shape, dtype=torch.float64, device=dev)
        w2 = 2 * 0.05 ** 2
        for p in walls_points():
            e = [torch.exp(-(x - c) ** 2 / w2) for x, c in zip(X, p)]
            bump += e[2][:, :, None, None] * e[1][:, None, :, None] * e[0][:, None, None, :]
        for v in range(fs.nvars):
            noise = torch.empty(shape, dtype=torch.float64, device=dev).uniform_(
                -1.0, 1.0, generator=g)
            fs.work[:, v].copy_(bump + noise)
    else:
        raise ValueError(f"no stated data for workload {workload!r}")
    return fs


def uniform_data(seed: int = 1):
    rng = np.random.default_rng(seed)

    def fn(x, v):
        return rng.uniform(-1.0, 1.0, size=np.shape(x[0]))
    return fn


def random_fill(fs: FieldSet, seed: int = 1, lo=-1.0, hi=1.0) -> FieldSet:
    """Every stored point of ``fs`` seeded uniform in ``[lo, hi]`` (fast: no
    positions)."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    host = torch.empty(tuple(fs.work.shape), dtype=fs.work.dtype).uniform_(lo, hi, generator=g)
    fs.work.copy_(host)
    return fs


def walls_points(seed: int = 2, n: int = 2):
    """The seeded refinement centres of the walls mesh, inside (0.1, 0.9)^3."""
    rng = np.random.default_rng(seed)
    return [tuple(float(x) for x in rng.uniform(0.1, 0.9, size=3)) for _ in range(n)]


def walls_forest(roots: int = 8, N: int = 32, levels: int = 5, seed: int = 2) -> Forest:
    """3-D over the unit cube, ``roots^3`` roots, low faces reflecting and high
    faces outflow; ``levels`` passes that refine every leaf of the pass's
    level containing or adjacent to one of two seeded points, each followed by
    balance."""
    f = Forest((roots,) * 3, N=N, reflecting=((True, False),) * 3,
               outflow=((False, True),) * 3, extents=((0.0, 1.0),) * 3)
    pts = walls_points(seed)

    def near(ext):
        w = ext[0][1] - ext[0][0]
        return any(all(a - w <= p[d] <= b + w for d, (a, b) in enumerate(ext)) for p in pts)
    return refine_where(f, near, range(levels))


def walls_data(seed: int = 3, width: float = 0.05):
    """Gaussian bumps of width ``width`` at the two refinement centres plus
    seeded uniform noise in [-1, 1]."""
    rng = np.random.default_rng(seed)
    pts = walls_points()

    def fn(x, v):
        bump = sum(np.exp(-sum((x[d] - p[d]) ** 2 for d in range(3)) / (2 * width ** 2))
                   for p in pts)
        return bump + rng.uniform(-1.0, 1.0, size=np.shape(x[0]))
    return fn


def walls_parities():
    """Five even variables and a vector's three components, each odd in its
    own dimension."""
    from .storage import EvenParity, OddParity
    even = (EvenParity,) * 3
    vec = [tuple(OddParity if e == d else EvenParity for e in range(3)) for d in range(3)]
    return [even] * 5 + vec


def walls_setup(device="cpu", T=np.float64, roots=8, N=32, levels=5, G=2):
    from .storage import vertexcentered
    f = walls_forest(roots=roots, N=N, levels=levels)
    fs = FieldSet(f, 8, G=G, centering=vertexcentered(3), parity=walls_parities(), T=T,
                  device=device)
    ops = Operators(prolongation=4, restriction=4)
    return f, fs, ops


def forest_batch_specs(n: int = 64, seed: int = 4, max_roots: int = 6, max_levels: int = 4):
    """The uneven batch: ``n`` forests with roots per side drawn from
    {2,...,6}^3, N from {8, 16} and 1-4 refinement levels around two seeded
    points each (cell-centred, periodic)."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        roots = tuple(int(x) for x in rng.integers(2, max_roots + 1, size=3))
        N = int(rng.choice([8, 16]))
        levels = int(rng.integers(1, max_levels + 1))
        pts = [tuple(float(rng.uniform(0, r)) for r in roots) for _ in range(2)]
        specs.append((roots, N, levels, pts))
    return specs


def batch_forest(roots, N, levels, pts) -> Forest:
    f = Forest(roots, N=N, periodic=(True,) * 3, extents=tuple((0.0, float(r)) for r in roots))

    def near(ext):
        w = ext[0][1] - ext[0][0]
        return any(all(a - w <= p[d] <= b + w for d, (a, b) in enumerate(ext)) for p in pts)
    return refine_where(f, near, range(levels))


def forest_batch_setup(n: int = 64, seed: int = 4, T=np.float32, device="cuda", G: int = 2,
                       max_roots: int = 6, max_levels: int = 4):
    """The fields sets, schedules and batch of the uneven multi-forest
    workload: 2 variables (u, v), G = 2, PV(4,4)."""
    from .batch import ForestBatch
    from .schedule import GhostSchedule
    ops = Operators(prolongation=4, restriction=4)
    fss, scheds = [], []
    for roots, N, levels, pts in forest_batch_specs(n, seed, max_roots, max_levels):
        f = batch_forest(roots, N, levels, pts)
        fs = FieldSet(f, 2, G=G, T=T)
        fss.append(fs)
        scheds.append(GhostSchedule(fs, ops))
    return fss, scheds, ForestBatch(fss, scheds, device=device)


def wave_initial(batch, seed: int = 5):
    """A smooth pulse in u and zero v, per forest, plus small seeded noise."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    for fs in batch.fieldsets:
        f = fs.forest
        ext = f.extents
        centre = [(a + b) / 2 for a, b in ext]
        host = np.zeros(tuple(fs.work.shape), dtype=fs.T)
        for b in range(fs.nblocks()):
            pos = fs.positions(b)
            X = np.meshgrid(*pos, indexing="ij")
            r2 = sum((X[d] - centre[d]) ** 2 for d in range(3))
            host[b, 0] = np.exp(-r2 / 0.5).astype(fs.T).transpose()
        noise = torch.empty(host.shape, dtype=torch.float64).uniform_(-1e-3, 1e-3, generator=g)
        fs.work.copy_(torch.from_numpy(host) + noise.to(fs.work.dtype))
    return batch


WORKLOADS = {
    "quadrant": dict(desc="2-D 4x4 periodic roots, N=8, G=2, cell, 1 var F64, 25% of roots "
                          "refined once, PV(4,4)"),
    "sphere": dict(desc="3-D 8^3 periodic roots, N=16, G=3, cell, 4 vars F64, 3 levels nested "
                        "around the sphere |x-1/2|=0.25, PV(4,4)"),
}


def quadrant_setup(device="cpu", seed=0):
    f = quadrant_forest(seed)
    fs = FieldSet(f, 1, G=2, T=np.float64, device=device)
    ops = Operators(prolongation=4, restriction=4)
    return f, fs, ops


def sphere_setup(device="cpu", nvars=4, T=np.float64, roots=8, N=16, G=3, levels=3, p=4):
    f = sphere_forest(roots=roots, N=N, levels=levels)
    fs = FieldSet(f, nvars, G=G, T=T, device=device)
    ops = Operators(prolongation=p, restriction=p)
    return f, fs, ops
