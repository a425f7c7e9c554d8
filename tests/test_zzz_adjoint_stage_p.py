"""The adjoint of stage P, the wall-plane projection of vertex-centred sets.

Stage P scales each point of a reflecting wall plane in place by its
variable's factor, (1 + sigma)/2: one for a variable even across the wall,
zero for an odd one.  Its transfers read their own targets, and its transpose
is itself.  A transpose that adds a stage's targets onto their sources and
then zeroes the targets loses the even variables there; these layouts hold
even and odd variables across reflecting walls, as the walls mesh does.

The oracle's transpose is checked against the dense forward map and by the
dot-product test; the GPU's against the oracle's and by the dot-product test,
for one schedule and for a batch of walls forests.  (The file is named to run
after the other GPU test files.)"""
import numpy as np
import pytest
import torch

import oracle
from treeamr import (EvenParity, FieldSet, Forest, GhostSchedule, Operators, OddParity,
                     fill_ghosts, meshes)
from treeamr.storage import vertexcentered


def _dot(a, b):
    return float(np.dot(a.ravel().astype(np.float64), b.ravel().astype(np.float64)))


def _plane_case(G=1):
    """2-D, 2 x 2 roots, N = 4: periodic along x, a reflecting low and an
    outflow high face along y; a variable odd in both dimensions and one even
    in both."""
    f = Forest((2, 2), N=4, periodic=(True, False), reflecting=((False, False), (True, False)),
               outflow=((False, False), (False, True)), extents=((0.0, 1.0),) * 2)
    fs = FieldSet(f, 2, G=G, centering=vertexcentered(2),
                  parity=[(OddParity, OddParity), (EvenParity, EvenParity)], T=np.float64)
    return fs, GhostSchedule(fs, Operators(prolongation=2, restriction=2))


def _walls_case(roots=2, levels=2):
    """The walls mesh's layout, small: reflecting low and outflow high faces,
    8 variables (5 even, a vector's 3 components odd in their own dimension)."""
    f = meshes.walls_forest(roots=roots, N=8, levels=levels)
    fs = FieldSet(f, 8, G=2, centering=vertexcentered(3), parity=meshes.walls_parities(),
                  T=np.float64)
    return fs, GhostSchedule(fs, Operators(prolongation=4, restriction=4))


def _dense(fs, s, first=oracle.ALL_FIRST, last=oracle.ALL_LAST):
    n = fs.work.numel()
    shape = tuple(fs.work.shape)
    A, AT = np.zeros((n, n)), np.zeros((n, n))
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        A[:, i] = oracle.fill(s, e.reshape(shape).copy(), fs.nvars, fs.factors_host,
                              first=first, last=last).ravel()
        AT[:, i] = oracle.fill_adjoint(s, e.reshape(shape).copy(), fs.nvars, fs.factors_host,
                                       first=first, last=last).ravel()
    return A, AT


def test_stage_p_is_there_with_even_and_odd_variables():
    for fs, s in (_plane_case(), _plane_case(G=2), _walls_case()):
        assert any(g.stage == -1 for g in s.groups)


def test_oracle_dense_transpose_with_stage_p():
    """Every entry of the oracle's A^T equals A's, for the whole fill and for
    stage P alone, which is diagonal and its own transpose."""
    fs, s = _plane_case()
    A, AT = _dense(fs, s)
    assert np.max(np.abs(AT - A.T)) <= 1e-15
    P, PT = _dense(fs, s, first=-1, last=-1)
    assert np.array_equal(P, np.diag(np.diag(P)))
    assert np.array_equal(PT, P)
    assert set(np.unique(np.diag(P))) == {0.0, 1.0}


def test_oracle_dot_product_walls_layout():
    fs, s = _walls_case()
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    ax = oracle.fill(s, x.copy(), fs.nvars, fs.factors_host)
    aty = oracle.fill_adjoint(s, y.copy(), fs.nvars, fs.factors_host)
    lhs, rhs = _dot(ax, y), _dot(x, aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["plane", "walls"])
def test_gpu_adjoint_with_stage_p(cuda_lib, case):
    from treeamr.adjoint import fill_ghosts_adjoint
    fs, s = _plane_case(G=2) if case == "plane" else _walls_case()
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    y = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    fs.work = fs.work.cuda()
    fs.factors = fs.factors.cuda()
    fs.work.copy_(torch.from_numpy(x))
    fill_ghosts(fs, s)
    ax = fs.work.cpu().numpy()
    yt = torch.from_numpy(y).cuda()
    fill_ghosts_adjoint(fs, s, yt)
    aty = yt.cpu().numpy()
    lhs, rhs = _dot(ax, y), _dot(x, aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))
    expect = oracle.fill_adjoint(s, y.copy(), fs.nvars, fs.factors_host)
    assert np.max(np.abs(aty - expect)) <= 1e-13 * np.max(np.abs(expect))


@pytest.mark.gpu
def test_gpu_batch_adjoint_with_stage_p(cuda_lib):
    """A batch of two walls forests: its adjoint against each member's oracle
    adjoint, and the dot-product test over the whole arena."""
    from treeamr.batch import ForestBatch
    fss, scheds = [], []
    for roots, levels in ((2, 2), (3, 2)):
        fs, s = _walls_case(roots, levels)
        fss.append(fs)
        scheds.append(s)
    batch = ForestBatch(fss, scheds, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(6)
    batch.arena.uniform_(-1, 1, generator=g)
    x = batch.arena.clone()
    y = torch.empty_like(x).uniform_(-1, 1, generator=g)
    batch.fill()
    ax = batch.arena.clone()
    aty = y.clone()
    batch.fill_adjoint(aty)
    torch.cuda.synchronize()
    lhs = float(torch.dot(ax.double().ravel(), y.double().ravel()))
    rhs = float(torch.dot(x.double().ravel(), aty.double().ravel()))
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))
    for m, (fs, s) in enumerate(zip(fss, scheds)):
        ym = batch.member_view(y, m).cpu().numpy().copy()
        expect = oracle.fill_adjoint(s, ym, fs.nvars, fs.factors_host)
        got = batch.member_view(aty, m).cpu().numpy()
        assert np.max(np.abs(got - expect)) <= 1e-13 * np.max(np.abs(expect)), m
