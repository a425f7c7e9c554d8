"""Property checks of a filled field set, shared by the full-size GPU tests
and their small CPU counterparts (which run the oracle's fill): polynomial
exactness on the sphere and walls meshes (``test/ghost_tests.jl:247-281``),
parity across reflecting faces (``test/reflect_tests.jl:98-131``) and an
outflow ghost equal to the nearest own point (``test/outflow_tests.jl:123-151``)."""
import math
import os

import torch

import oracle
from treeamr import fill_ghosts, meshes

NTHREADS = os.cpu_count() or 1


def _q3(X, v):
    """A polynomial of degree 3 in each coordinate (tensor-product order 4
    reproduces it), different per variable."""
    x, y, z = X
    a = 0.3 + 0.1 * v
    return (1.0 + a * x - 0.7 * x ** 3 + 0.25 * y ** 2 * z - 0.4 * x * y * z ** 3
            + 0.9 * z ** 2 - 0.15 * y ** 3 * x ** 2 + 0.05 * v)


def _grid(X, b0, b1):
    x = X[0][b0:b1][:, None, None, :]
    y = X[1][b0:b1][:, None, :, None]
    z = X[2][b0:b1][:, :, None, None]
    return x, y, z


def _fill(fs, sched, where):
    """The fill on the GPU, or the oracle's on the host (the small CPU cases)."""
    if where == "gpu":
        fill_ghosts(fs, sched)
        torch.cuda.synchronize()
    else:
        host = fs.work.numpy()
        oracle.fill(sched, host, fs.nvars, fs.factors_host, nthreads=NTHREADS)


def sphere_polynomial_error(fs, sched, where):
    """Largest deviation from the polynomial at any point, and its scale.
    A ghost past a periodic face holds the polynomial at its wrapped
    position.  Every level jump lies inside the unit cube (the sphere's
    refinement stays clear of the domain's faces), so no stencil mixes
    wrapped and unwrapped data."""
    X = meshes._stored_positions(fs, fs.work.device)
    W = [torch.remainder(x, 1.0) for x in X]
    ghost = torch.ones(tuple(reversed(fs.stored)), dtype=torch.bool, device=fs.work.device)
    ghost[fs.interior()] = False
    nb, step = fs.nblocks(), 1024
    for v in range(fs.nvars):
        for b0 in range(0, nb, step):
            b1 = min(nb, b0 + step)
            val = _q3(_grid(W, b0, b1), v)
            fs.work[b0:b1, v].copy_(torch.where(ghost, torch.nan, val))
    _fill(fs, sched, where)
    worst, scale = 0.0, 0.0
    for v in range(fs.nvars):
        for b0 in range(0, nb, step):
            b1 = min(nb, b0 + step)
            exact = _q3(_grid(W, b0, b1), v)
            got = fs.work[b0:b1, v]
            assert not torch.isnan(got).any()
            worst = max(worst, float((got - exact).abs().max()))
            scale = max(scale, float(exact.abs().max()))
    return worst, scale


def _parity_poly(X, v):
    """Degree 3 in each coordinate, even in every coordinate for variables
    0-4 and odd in coordinate ``v - 5`` (even in the others) for 5-7: the
    parities of the walls mesh's variables about the reflecting planes
    x = 0, y = 0, z = 0."""
    x, y, z = X
    even = (1.0 + 0.5 * x ** 2) * (2.0 - 0.3 * y ** 2) * (1.0 + 0.2 * z ** 2) + 0.1 * v
    if v < 5:
        return even
    s = X[v - 5]
    return s * (1.0 - 0.6 * s ** 2) * (1.0 + 0.4 * (x * x + y * y + z * z - s * s))


def walls_properties(fs, sched, where, margin):
    """Fills the parity polynomial (ghosts poisoned) and returns the largest
    deviation from it and its scale over every point farther than
    ``margin`` from the outflow faces x, y, z = 1 (a ghost past a reflecting
    face holds the polynomial at its own position, by its parity), and the
    number of points past an outflow face that differ in their bits from
    the block's point on the face (``test/outflow_tests.jl:123-151``: an
    outflow ghost takes the nearest own point's value).  Near an outflow
    face a prolongation reads coarse ghosts that are clamped, not
    polynomial, so exactness is checked away from it."""
    X = meshes._stored_positions(fs, fs.work.device)
    dev = fs.work.device
    ghost = torch.ones(tuple(reversed(fs.stored)), dtype=torch.bool, device=dev)
    ghost[fs.interior()] = False
    nb, step = fs.nblocks(), 256
    for v in range(fs.nvars):
        for b0 in range(0, nb, step):
            b1 = min(nb, b0 + step)
            val = _parity_poly(_grid(X, b0, b1), v)
            fs.work[b0:b1, v].copy_(torch.where(ghost, torch.nan, val))
    _fill(fs, sched, where)
    worst, scale = 0.0, 0.0
    for v in range(fs.nvars):
        for b0 in range(0, nb, step):
            b1 = min(nb, b0 + step)
            x, y, z = _grid(X, b0, b1)
            exact = _parity_poly((x, y, z), v)
            got = fs.work[b0:b1, v]
            assert not torch.isnan(got).any()
            far = (x < 1.0 - margin) & (y < 1.0 - margin) & (z < 1.0 - margin)
            dev_ = torch.where(far, (got - exact).abs(), torch.zeros_like(got))
            worst = max(worst, float(dev_.max()))
            scale = max(scale, float(exact.abs().max()))
    # outflow: rows past a high face equal the face row, whole slab
    N, G = fs.forest.N, fs.G[0]
    face = G + N                     # 0-based stored index of the high face plane
    bad = 0
    wk = fs.work
    for d in range(3):
        ax = 4 - d                   # the array's axis of dimension d
        touch = [b for b, k in enumerate(fs.forest.leaves)
                 if fs.forest.block_extent(k)[d][1] >= 1.0]
        if not touch:
            continue
        idx = torch.tensor(touch, device=dev)
        sub = wk.index_select(0, idx)
        ref = sub.narrow(ax, face, 1)
        past = sub.narrow(ax, face + 1, G)
        bad += int((past.view(torch.int64 if wk.dtype == torch.float64 else torch.int32) !=
                    ref.expand_as(past).contiguous().view(
                        torch.int64 if wk.dtype == torch.float64 else torch.int32)).sum())
    return worst, scale, bad


def _dot(a: torch.Tensor, b: torch.Tensor) -> float:
    """Float64 dot product in chunks summed exactly on the host."""
    a, b = a.reshape(-1), b.reshape(-1)
    step = 1 << 22
    return math.fsum(float(torch.dot(a[i:i + step], b[i:i + step]))
                     for i in range(0, a.numel(), step))
