"""The adjoint fill: dot-product tests, dense transpose, finite differences.

The reference has no adjoint; its oracle is the linear algebra of the
forward fill (the oracle's forward fill applied to unit vectors, and its
scatter-form transpose).  Tolerances: the dot-product test to 1e-13 relative
in Float64 (the target the engine is built to), gradients against central
differences to 1e-6 relative."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import nested_forest
from treeamr import FieldSet, Forest, GhostSchedule, Operators, EvenParity, OddParity
from treeamr import meshes


def _dot(a, b):
    return float(np.dot(a.ravel().astype(np.float64), b.ravel().astype(np.float64)))


def _forward(s, fs, x):
    out = x.copy()
    return oracle.fill(s, out, fs.nvars, fs.factors_host)


def _adjoint(s, fs, y):
    out = y.copy()
    return oracle.fill_adjoint(s, out, fs.nvars, fs.factors_host)


def _cases():
    out = []
    f = nested_forest(3, N=8)
    out.append(("nested3d", FieldSet(f, 2, G=2), Operators(prolongation=4, restriction=4)))
    f2 = nested_forest(2, N=8, periodic=(True, True))
    out.append(("nested2d-periodic", FieldSet(f2, 1, G=3),
                Operators(prolongation=6, restriction=6)))
    D = 3
    fr = Forest((2,) * D, N=8, reflecting=tuple((True, False) for _ in range(D)),
                outflow=tuple((False, True) for _ in range(D)), extents=[(0.0, 2.0)] * D)
    fr.refine(fr.leaves[0])
    fr.balance()
    par = [(EvenParity,) * D, (OddParity, EvenParity, EvenParity)]
    out.append(("walls3d", FieldSet(fr, 2, G=2, parity=par), Operators(prolongation=4, restriction=4)))
    return out


@pytest.mark.parametrize("case", range(3))
def test_oracle_dot_product(case):
    name, fs, ops = _cases()[case]
    s = GhostSchedule(fs, ops)
    rng = np.random.default_rng(case)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    lhs = _dot(_forward(s, fs, x), y)
    rhs = _dot(x, _adjoint(s, fs, y))
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))


@pytest.mark.parametrize("seed", range(40))
def test_oracle_dot_product_random_layouts(seed):
    """The oracle's scatter-form transpose against its forward fill on the
    seeded random layouts of the point-by-point tests (1-D to 3-D, cell and
    vertex, periodic or walled, orders 2 to 6), in Float64."""
    from test_pointwise import _random_layout
    fs, p, _, _ = _random_layout(np.random.default_rng(1000 + seed), dtype=np.float64)
    s = GhostSchedule(fs, Operators(prolongation=p, restriction=p))
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    lhs = _dot(_forward(s, fs, x), y)
    rhs = _dot(x, _adjoint(s, fs, y))
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))


@pytest.mark.parametrize("seed", range(16))
def test_oracle_dot_product_random_conservative_layouts(seed):
    """The conservative family (odd prolongation orders, the exact volume
    average as restriction) on seeded random cell-centred layouts: periodic
    or walled dimensions, random parities.  The tolerance is relative to the
    sum of the products' magnitudes, which the rounding of a dot product
    scales with."""
    from test_pointwise import _near
    from treeamr.operators import Conservative
    rng = np.random.default_rng(9000 + seed)
    D, N, p = int(rng.integers(1, 4)), int(rng.choice([8, 16])), int(rng.choice([1, 3, 5]))
    periodic = tuple(bool(rng.integers(2)) for _ in range(D))
    kinds = [tuple(int(rng.integers(2)) for _ in range(2)) for _ in range(D)]
    refl = tuple((k[0] == 0 and not periodic[d], k[1] == 0 and not periodic[d])
                 for d, k in enumerate(kinds))
    outf = tuple((k[0] == 1 and not periodic[d], k[1] == 1 and not periodic[d])
                 for d, k in enumerate(kinds))
    G = (p - 1) // 2 + int(rng.integers(1, 3))
    levels = int(rng.integers(1, 4 if D < 3 else 3))
    pts = [tuple(float(x) for x in rng.uniform(0.05, 0.95, size=D)) for _ in range(2)]
    f = Forest((4,) * D, N=N, periodic=periodic, reflecting=refl, outflow=outf,
               extents=((0.0, 1.0),) * D)
    meshes.refine_where(f, _near(pts), range(levels))
    par = [tuple(OddParity if rng.integers(2) else EvenParity for _ in range(D))
           for _ in range(2)]
    fs = FieldSet(f, 2, G=G, parity=par, T=np.float64)
    s = GhostSchedule(fs, Operators(prolongation=p, restriction=2, family=Conservative))
    r = np.random.default_rng(seed)
    x = r.uniform(-1, 1, size=tuple(fs.work.shape))
    y = r.uniform(-1, 1, size=tuple(fs.work.shape))
    ax = _forward(s, fs, x)
    lhs, rhs = _dot(ax, y), _dot(x, _adjoint(s, fs, y))
    assert abs(lhs - rhs) <= 1e-15 * _dot(np.abs(ax), np.abs(y))


def test_oracle_dense_transpose_2d():
    """Every entry of A^T from the scatter-form transpose equals the entry of
    A from the forward fill on unit vectors (a tiny 2-D mesh, all columns)."""
    f = Forest((2, 2), N=4, periodic=(True, True))
    f.refine(f.leaves[0])
    f.balance()
    fs = FieldSet(f, 1, G=2)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=2))
    n = fs.work.numel()
    shape = tuple(fs.work.shape)
    A = np.zeros((n, n))
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        A[:, i] = _forward(s, fs, e.reshape(shape)).ravel()
    AT = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        AT[:, j] = _adjoint(s, fs, e.reshape(shape)).ravel()
    assert np.max(np.abs(AT - A.T)) <= 1e-15


# --- the GPU kernel ----------------------------------------------------------

def _gpu_setup(fs):
    fs.work = fs.work.cuda()
    fs.factors = fs.factors.cuda()
    return fs


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(3))
def test_gpu_dot_product_and_oracle(cuda_lib, case):
    from treeamr import fill_ghosts
    from treeamr.adjoint import fill_ghosts_adjoint
    name, fs, ops = _cases()[case]
    s = GhostSchedule(fs, ops)
    rng = np.random.default_rng(10 + case)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    _gpu_setup(fs)
    fs.work.copy_(torch.from_numpy(x))
    fill_ghosts(fs, s)
    ax = fs.work.cpu().numpy()
    yt = torch.from_numpy(y).cuda()
    fill_ghosts_adjoint(fs, s, yt)
    aty = yt.cpu().numpy()
    lhs, rhs = _dot(ax, y), _dot(x, aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))
    expect = _adjoint(s, fs, y)
    scale = np.max(np.abs(expect))
    assert np.max(np.abs(aty - expect)) <= 1e-13 * scale


@pytest.mark.gpu
def test_gpu_adjoint_deterministic_and_scratch(cuda_lib):
    from treeamr.adjoint import fill_ghosts_adjoint
    from treeamr.ghosts import device_schedule
    f, fs, ops = meshes.sphere_setup(nvars=2, roots=4, levels=2)
    s = GhostSchedule(fs, ops)
    _gpu_setup(fs)
    g = torch.Generator(device="cuda").manual_seed(3)
    y0 = torch.rand(fs.work.shape, dtype=fs.work.dtype, device="cuda", generator=g)
    a = y0.clone()
    fill_ghosts_adjoint(fs, s, a)
    b = y0.clone()
    fill_ghosts_adjoint(fs, s, b)
    assert torch.equal(a.view(torch.int64), b.view(torch.int64))
    nbytes = device_schedule(s, 0).adjoint_scratch_bytes(fs.nvars)
    scratch = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device="cuda")
    c = y0.clone()
    fill_ghosts_adjoint(fs, s, c, scratch=scratch)
    assert torch.equal(a.view(torch.int64), c.view(torch.int64))
    with pytest.raises(Exception):
        fill_ghosts_adjoint(fs, s, y0.clone(), scratch=scratch[:8])


@pytest.mark.gpu
def test_gpu_dense_transpose_sample(cuda_lib):
    """Sampled entries of A^T from the GPU adjoint against A from the oracle on
    the 2x2x2-root periodic mesh (N = 16, G = 3), one block refined."""
    from treeamr.adjoint import fill_ghosts_adjoint
    f = Forest((2, 2, 2), N=16, periodic=(True,) * 3)
    f.refine(f.leaves[0])
    f.balance()
    fs = FieldSet(f, 1, G=3)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    shape = tuple(fs.work.shape)
    n = int(np.prod(shape))
    rng = np.random.default_rng(4)
    # rows j of A among ghost points, columns i among all points
    J = rng.choice(n, size=24, replace=False)
    cols = {}
    _gpu_setup(fs)
    for j in J:
        e = torch.zeros(n, dtype=torch.float64, device="cuda")
        e[j] = 1.0
        e = e.view(shape).contiguous()
        fill_ghosts_adjoint(fs, s, e)
        cols[j] = e.view(-1).cpu().numpy()                 # = A[j, :]
    I = set()
    for j in J:
        I.update(np.nonzero(cols[j])[0][:6].tolist())
    I.update(rng.choice(n, size=40, replace=False).tolist())
    for i in sorted(I):
        e = np.zeros(n)
        e[i] = 1.0
        Ai = _forward(s, fs, e.reshape(shape)).ravel()      # = A[:, i]
        for j in J:
            assert abs(cols[j][i] - Ai[j]) <= 1e-15


@pytest.mark.gpu
def test_gpu_gradient_vs_finite_differences(cuda_lib):
    """L = sum(w * lap7(A u)) over owned points: autograd through GhostFill
    against central differences (h = 1e-6) on a sample of entries."""
    from treeamr.adjoint import ghost_fill
    f = Forest((2, 2, 2), N=8, periodic=(True,) * 3)
    f.refine(f.leaves[0])
    f.balance()
    fs = FieldSet(f, 2, G=2)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    _gpu_setup(fs)
    g = torch.Generator(device="cuda").manual_seed(8)
    u = torch.rand(fs.work.shape, dtype=torch.float64, device="cuda", generator=g)
    w = torch.rand(fs.work.shape, dtype=torch.float64, device="cuda", generator=g)
    G, N = 2, 8
    own = slice(G, G + N)

    def loss(x):
        a = ghost_fill(x, fs, s)
        c = a[:, :, own, own, own]
        lap = (a[:, :, G + 1:G + N + 1, own, own] + a[:, :, G - 1:G + N - 1, own, own] +
               a[:, :, own, G + 1:G + N + 1, own] + a[:, :, own, G - 1:G + N - 1, own] +
               a[:, :, own, own, G + 1:G + N + 1] + a[:, :, own, own, G - 1:G + N - 1] - 6 * c)
        return (w[:, :, own, own, own] * lap).sum()

    x = u.clone().requires_grad_(True)
    L = loss(x)
    L.backward()
    grad = x.grad.detach()
    rng = np.random.default_rng(1)
    flat = u.view(-1)
    h = 1e-6
    idx = rng.choice(flat.numel(), size=30, replace=False)
    # entries that matter: owned points next to a block face feed ghosts
    for k in idx:
        up = u.clone().view(-1)
        dn = u.clone().view(-1)
        up[k] += h
        dn[k] -= h
        with torch.no_grad():
            fd = (loss(up.view(u.shape)) - loss(dn.view(u.shape))).item() / (2 * h)
        gk = grad.view(-1)[k].item()
        assert abs(fd - gk) <= 1e-6 * max(1.0, abs(gk))
