"""The device boundary hook (``CellBoundary``, ``src/ghosts.jl:1166-1318``)
with built-in functions of position: the GPU's values equal the oracle's
host evaluation bit for bit at every outer-face ghost, a full fill with the
hook equals the oracle's fill with the same boundary values, and a
polynomial boundary keeps an order-p fill exact for degree p-1 data up to
the outer faces (``test/ghost_tests.jl:247-281`` with boundaries).

A hook that prescribes the wall planes (``wall = "prescribed"``, stage W,
``src/ghosts.jl:1378-1412, 1639-1652``) writes the primaries of every wall
point of a vertex-like dimension first; after the fill every own copy of
a wall point is one number, the hook's at the primary."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import Geometry, ghost_mask, nanbits, nested_forest
from treeamr import FieldSet, GhostSchedule, Operators, fill_ghosts
from treeamr.boundary import CellBoundary, Constant, Polynomial, Relative
from treeamr.schedule import PHASE1_TAG, UNIFY_TAG
from treeamr.storage import edgecentered, facecentered, vertexcentered


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
        CellBoundary(Constant([1.0]), wall="dirichlet")
    assert CellBoundary(Constant([1.0]), wall="prescribed").prescribes_wall
    assert not CellBoundary(Constant([1.0])).prescribes_wall
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


# --- stage W: a prescribed wall ---------------------------------------------------

def _oracle_prescribed_fill(fs, s, g, host):
    """Stage W on the host, then the fill with the hook as usual."""
    oracle.cell_boundary(fs, host, s.walls, g)
    if isinstance(g, Relative):
        return _oracle_relative_fill(fs, s, g, host)
    oracle.fill(s, host, fs.nvars, fs.factors_host, last=PHASE1_TAG)
    oracle.cell_boundary(fs, host, s.boundaries, g)
    return oracle.fill(s, host, fs.nvars, fs.factors_host, first=PHASE1_TAG + 1)


def _wall_copies(fs):
    """Per point on an outer face of a vertex-like dimension, every own copy
    as ``(block, 1-based stored index)``."""
    f = fs.forest
    geo = Geometry(f)
    D, N = f.D, f.N
    top = [f.roots[d] * geo.scale for d in range(D)]
    out = {}
    for b, k in enumerate(f.leaves):
        pts = geo.points(k, fs.G, fs.c, N)
        for I in np.ndindex(*[len(p) for p in pts]):
            x = tuple(int(pts[d][I[d]]) for d in range(D))
            if any(fs.c[d] == 1 and x[d] in (0, top[d]) for d in range(D)):
                out.setdefault(x, []).append((b, tuple(fs.G[d] + 1 + I[d] for d in range(D))))
    return out


def _val(host, b, v, idx):
    return host[(b, v) + tuple(i - 1 for i in reversed(idx))]


def _wall_cases(D):
    out = [vertexcentered(D)]
    if D >= 2:
        out.append(facecentered(D, 2))
    if D == 3:
        out.append(edgecentered(3, 1))
    return out


@pytest.mark.parametrize("D", [1, 2, 3])
def test_wall_regions(D):
    """Stage W's regions (``src/schedule.jl:2134-2170``): primaries on the
    outer wall planes of vertex-like dimensions only, one plane in as the
    relative form's point, none for a cell-centred set."""
    f = nested_forest(D, N=8)
    ops = Operators(prolongation=4, restriction=4)
    assert GhostSchedule(FieldSet(f, 1, G=2), ops).walls == []
    for C in _wall_cases(D):
        fs = FieldSet(f, 1, G=2, centering=C)
        s = GhostSchedule(fs, ops)
        assert s.walls, C
        N, G, c = f.N, fs.G, fs.c
        for r in s.walls:
            assert r.slot == UNIFY_TAG and any(r.direction)
            for d in range(D):
                a, z = r.region[d]
                if r.direction[d] < 0:
                    assert c[d] == 1 and a == z == G[d] + 1 and r.clamps[d] == G[d] + 2
                elif r.direction[d] > 0:
                    assert c[d] == 1 and a == z == G[d] + N + 1 and r.clamps[d] == G[d] + N
                else:
                    assert r.clamps[d] == 0
            assert (s.primary_bits[r.block] >> sum(
                (0 if a == G[d] + 1 and c[d] == 1 else 2 if a == G[d] + N + 1 and c[d] == 1
                 else 1) * 3 ** d for d, (a, z) in enumerate(r.region))) & 1


@pytest.mark.parametrize("D", [2, 3])
def test_oracle_prescribed_wall_is_one_number(D):
    """After a fill with a prescribed wall every own copy of a wall point is
    one number: the constant, the polynomial at the point, or for the
    relative form the primary's value one plane in shifted by f."""
    f = nested_forest(D, N=8)
    ops = Operators(prolongation=4, restriction=4)
    for C in _wall_cases(D):
        fs = FieldSet(f, 2, G=2, centering=C)
        s = GhostSchedule(fs, ops)
        copies = _wall_copies(fs)
        assert copies
        rng = np.random.default_rng(3 + D)
        host = rng.uniform(-1, 1, size=tuple(fs.work.shape))
        for g in (Constant([1.5, -2.25]), _poly(D, 2), Relative(Constant([0.0, 0.0]))):
            out = _oracle_prescribed_fill(fs, s, g, host.copy())
            shared = 0
            for x, cp in copies.items():
                for v in range(2):
                    vals = {_val(out, b, v, idx) for b, idx in cp}
                    assert len(vals) == 1, (C, x, vals)
                    if isinstance(g, Constant):
                        assert vals == {g.values[v]}
                shared += len(cp) > 1
            # a wall point of a set vertex-like along one dimension alone
            # lies in one block; along two it is shared across their edges
            assert (shared > 0) == (sum(fs.c) >= 2), C
            if isinstance(g, Polynomial):
                r = s.walls[0]
                pos = fs.positions(r.block)
                idx = tuple(a for a, _ in r.region)
                xw = [pos[d][idx[d] - 1] for d in range(D)]
                want = 0.5 + sum(0.25 * (d + 1) * xw[d] for d in range(D)) + 0.125 * xw[0] ** 2
                assert abs(_val(out, r.block, 0, idx) - want) < 1e-12
            if isinstance(g, Relative):
                for r in s.walls:
                    idxs = [range(a, z + 1) for a, z in r.region]
                    for I in np.ndindex(*[len(i) for i in idxs]):
                        idx = tuple(idxs[d][I[d]] for d in range(D))
                        rr = tuple(r.clamps[d] or idx[d] for d in range(D))
                        assert _val(out, r.block, 1, idx) == _val(out, r.block, 1, rr)
        # the evolved default leaves the wall planes to the state
        out = oracle.fill(s, host.copy(), fs.nvars, fs.factors_host)
        r = s.walls[0]
        idx = tuple(a for a, _ in r.region)
        assert _val(out, r.block, 0, idx) == _val(host, r.block, 0, idx)


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_prescribed_wall_bit_exact(cuda_lib, D, T):
    f = nested_forest(D, N=8)
    ops = Operators(prolongation=4, restriction=4)
    for C in _wall_cases(D):
        fs = FieldSet(f, 2, G=2, centering=C, T=T)
        s = GhostSchedule(fs, ops)
        rng = np.random.default_rng(11 + D)
        host = rng.uniform(-1, 1, size=tuple(fs.work.shape)).astype(T)
        for g in (Constant([1.5, -2.25]), _poly(D, 2), Relative(_poly(D, 2))):
            expect = _oracle_prescribed_fill(fs, s, g, host.copy())
            fs.work = torch.from_numpy(host.copy()).cuda()
            fs.factors = fs.factors.cuda()
            fill_ghosts(fs, s, boundary=CellBoundary(g, wall="prescribed"))
            torch.cuda.synchronize()
            assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), (C, g)
            fs.factors = fs.factors.cpu()


@pytest.mark.parametrize("seed", range(12))
def test_oracle_polynomial_hook_keeps_random_fills_exact(seed):
    """Seeded random layouts with outer faces everywhere (1-D to 3-D, cell or
    vertex sets, orders 2 and 4, one or two levels around two random
    points): with polynomial data of degree p-1 (at most 2) and the same
    polynomial as the hook, between phase 1 and the prolongations, the
    oracle's fill is exact at every point, ghosts past the outer faces
    included."""
    from test_pointwise import _near
    from treeamr import Forest, meshes
    rng = np.random.default_rng(6100 + seed)
    D, vertex, p = int(rng.integers(1, 4)), bool(rng.integers(2)), int(rng.choice([2, 4]))
    f = Forest((3,) * D, N=8, periodic=(False,) * D, extents=((0.0, 1.0),) * D)
    pts = [tuple(float(x) for x in rng.uniform(0.05, 0.95, size=D)) for _ in range(2)]
    meshes.refine_where(f, _near(pts), range(int(rng.integers(1, 3))))
    fs = FieldSet(f, 1, G=2, centering=vertexcentered(D) if vertex else None)
    s = GhostSchedule(fs, Operators(prolongation=p, restriction=p))
    assert s.boundaries
    terms = {(0,) * D: [0.5]}
    for d in range(D):
        e = [0] * D
        e[d] = 1
        terms[tuple(e)] = [0.25 * (d + 1)]
    quad = 0.125 if p == 4 else 0.0
    if quad:
        e = [0] * D
        e[0] = 2
        terms[tuple(e)] = [quad]

    def exact(x):
        return 0.5 + sum(0.25 * (d + 1) * x[d] for d in range(D)) + quad * x[0] ** 2
    host = np.zeros(tuple(fs.work.shape))
    for b in range(fs.nblocks()):
        grids = np.meshgrid(*fs.positions(b), indexing="ij")
        host[b, 0] = np.transpose(exact(grids))
    filled = host.copy()
    filled[:, :, ghost_mask(fs)] = np.nan
    out = oracle.fill(s, filled, fs.nvars, fs.factors_host, last=PHASE1_TAG)
    oracle.cell_boundary(fs, out, s.boundaries, Polynomial(terms))
    out = oracle.fill(s, out, fs.nvars, fs.factors_host, first=PHASE1_TAG + 1)
    assert not np.isnan(out).any()
    assert np.max(np.abs(out - host)) < 1e-10
