"""The device boundary hook (``CellBoundary``, ``src/ghosts.jl:1166-1318``)
with built-in functions of position: the GPU's values equal the oracle's
host evaluation bit for bit at every outer-face ghost, a full fill with the
hook equals the oracle's fill with the same boundary values, and a
polynomial boundary keeps an order-p fill exact for degree p-1 data up to
the outer faces (``test/ghost_tests.jl:247-281`` with boundaries)."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import ghost_mask, nanbits, nested_forest
from treeamr import FieldSet, GhostSchedule, Operators, fill_ghosts
from treeamr.boundary import CellBoundary, Constant, Polynomial
from treeamr.storage import vertexcentered


def _poly(D, nvars):
    terms = {(0,) * D: [0.5 + v for v in range(nvars)]}
    for d in range(D):
        e = [0] * D
        e[d] = 1
        terms[tuple(e)] = [0.25 * (d + 1) - v for v in range(nvars)]
    e = [0] * D
    e[0] = 2
    terms[tuple(e)] = [0.125 * (v + 1) for v in range(nvars)]
    return Polynomial(terms)


def test_hook_refuses_what_is_not_built():
    with pytest.raises(TypeError):
        CellBoundary(lambda x, v, d: 0.0)
    with pytest.raises(ValueError):
        CellBoundary(Constant([1.0]), wall="prescribed")
    with pytest.raises(ValueError):
        Polynomial({(i, 0, 0): [1.0] for i in range(21)})


def test_oracle_polynomial_boundary_is_the_polynomial():
    D = 2
    f = nested_forest(D, N=8)
    fs = FieldSet(f, 2, G=2)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    assert s.boundaries
    g = _poly(D, 2)
    host = np.zeros(tuple(fs.work.shape))
    oracle.cell_boundary(fs, host, s.boundaries, g)
    r = s.boundaries[0]
    pos = fs.positions(r.block)
    idx = tuple(a for a, _ in r.region)
    x = [pos[d][idx[d] - 1] for d in range(D)]
    want = 0.5 + 0.25 * x[0] + 0.5 * x[1] + 0.125 * x[0] ** 2
    got = host[(r.block, 0) + tuple(i - 1 for i in reversed(idx))]
    assert abs(got - want) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
@pytest.mark.parametrize("centering", ["cell", "vertex"])
def test_gpu_hook_bit_exact(cuda_lib, D, T, centering):
    f = nested_forest(D, N=8)
    C = vertexcentered(D) if centering == "vertex" else None
    fs = FieldSet(f, 2, G=2, centering=C, T=T)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    for g in (Constant([1.5, -2.25]), _poly(D, 2)):
        rng = np.random.default_rng(D)
        host = rng.uniform(-1, 1, size=tuple(fs.work.shape)).astype(T)
        fs.work = torch.from_numpy(host.copy())
        fs.factors = fs.factors.cpu()
        bv = lambda h, fs_, regions: oracle.cell_boundary(fs_, h, regions, g)  # noqa: E731
        expect = oracle.fill_fieldset(fs, s, boundary_values=bv)
        fs.work = torch.from_numpy(host.copy()).cuda()
        fs.factors = fs.factors.cuda()
        fill_ghosts(fs, s, boundary=CellBoundary(g))
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect))


@pytest.mark.gpu
def test_gpu_polynomial_hook_keeps_the_fill_exact(cuda_lib):
    """Degree-2 data with a degree-2 polynomial boundary: an order-4 fill is
    exact in every ghost, the outer faces' included."""
    D = 3
    f = nested_forest(D, N=8)
    fs = FieldSet(f, 1, G=2, device="cuda")
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    g = _poly(D, 1)

    def exact(x):
        return 0.5 + sum(0.25 * (d + 1) * x[d] for d in range(D)) + 0.125 * x[0] ** 2
    host = np.zeros(tuple(fs.work.shape))
    for b in range(fs.nblocks()):
        pos = fs.positions(b)
        grids = np.meshgrid(*pos, indexing="ij")
        host[b, 0] = np.transpose(exact(grids))
    filled = host.copy()
    filled[:, :, ghost_mask(fs)] = np.nan
    fs.work.copy_(torch.from_numpy(filled))
    fill_ghosts(fs, s, boundary=CellBoundary(g))
    got = fs.work.cpu().numpy()
    assert not np.isnan(got).any()
    assert np.max(np.abs(got - host)) < 1e-10


# --- the relative form ---------------------------------------------------------

def _oracle_relative_fill(fs, s, g, host):
    """The fill with the relative hook in parts: phase 1, the slot-1
    regions, then each later stage followed by its slot's regions."""
    from treeamr.schedule import PHASE1_TAG
    out = oracle.fill(s, host, fs.nvars, fs.factors_host, last=PHASE1_TAG)
    by = {}
    for r in s.boundaries:
        by.setdefault(r.slot, []).append(r)
    oracle.cell_boundary(fs, out, by.get(PHASE1_TAG, []), g)
    for tag in [t for t in s.stage_tags if t > PHASE1_TAG]:
        oracle.fill(s, out, fs.nvars, fs.factors_host, first=tag, last=tag)
        oracle.cell_boundary(fs, out, by.get(tag, []), g)
    return out


def test_relative_zero_is_a_zero_gradient_outflow():
    """``Relative(0)``: every outer ghost equals the nearest evolved point
    (``src/ghosts.jl:1445``), and a later slot exists on this mesh."""
    from treeamr.boundary import Relative
    D = 2
    f = nested_forest(D, N=8)
    fs = FieldSet(f, 2, G=2)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    rng = np.random.default_rng(2)
    host = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    out = _oracle_relative_fill(fs, s, Relative(Constant([0.0, 0.0])), host.copy())
    for r in s.boundaries:
        idxs = [range(a, z + 1) for a, z in r.region]
        for I in np.ndindex(*[len(i) for i in idxs]):
            idx = tuple(idxs[d][I[d]] for d in range(D))
            rr = tuple(r.clamps[d] or idx[d] for d in range(D))
            for v in range(2):
                assert out[(r.block, v) + tuple(i - 1 for i in reversed(idx))] == \
                    out[(r.block, v) + tuple(i - 1 for i in reversed(rr))]


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_relative_hook_bit_exact(cuda_lib, D, T):
    from treeamr.boundary import Relative
    f = nested_forest(D, N=8)
    fs = FieldSet(f, 2, G=2, T=T)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    g = Relative(_poly(D, 2))
    rng = np.random.default_rng(7 + D)
    host = rng.uniform(-1, 1, size=tuple(fs.work.shape)).astype(T)
    expect = _oracle_relative_fill(fs, s, g, host.copy())
    fs.work = torch.from_numpy(host.copy()).cuda()
    fs.factors = fs.factors.cuda()
    fill_ghosts(fs, s, boundary=CellBoundary(g))
    torch.cuda.synchronize()
    assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect))
