"""Bounded operators (``Operators(...; bounded=True)``, ``src/operators.jl:194-250,
417-441``, kernels ``bounded_sum`` and ``bracket_clamp_sum``,
``src/ghosts.jl:286-361``), restated from the reference's ``test/bounded_tests.jl``:
every claim is checked against an oracle that knows only the formula and
the geometry (the coarse cell a fine point lies in, which side of its
centre, the Lagrange window and its bracket), never the schedule's stencils.
On the GPU the bounded groups' launch is the oracle's bit for bit."""
import itertools
from fractions import Fraction

import numpy as np
import pytest
import torch

import oracle
from _helpers import boundary_from, nanbits, nested_forest
from treeamr import FieldSet, Forest, GhostSchedule, Operators
from treeamr.operators import BOUNDED_CONSERVATIVE, BOUNDED_POINTVALUE, UNBOUNDED, \
    Conservative, lagrange_weights
from treeamr.regrid import RegridTransfer
from treeamr.storage import vertexcentered

BOUNDED = Operators(prolongation=3, restriction=2, family=Conservative, bounded=True)
BOUNDED_PV = Operators(prolongation=4, restriction=4, bounded=True)
PLAIN_PV = Operators(prolongation=4, restriction=4)


def oracle_mc(a, b):
    """The monotonized central slope written as the smallest of three
    candidates that agree in sign (``test/bounded_tests.jl:15-16``)."""
    if np.sign(a) != np.sign(b):
        return 0.0
    return np.sign(a) * min(abs(2 * a), abs(2 * b), abs((a + b) / 2))


def bounded_child(U, I, sigma):
    """``test/bounded_tests.jl:18-30``: the bounded child of coarse cell ``I``
    of the periodic coarse grid ``U`` on sides ``sigma``."""
    D = U.ndim
    n = U.shape

    def at(J):
        return U[tuple(J[d] % n[d] for d in range(D))]
    u = at(I)
    lo = [at(tuple(I[k] - (k == d) for k in range(D))) for d in range(D)]
    hi = [at(tuple(I[k] + (k == d) for k in range(D))) for d in range(D)]
    s = [oracle_mc(hi[d] - u, u - lo[d]) for d in range(D)]
    M, m = max([u] + lo + hi), min([u] + lo + hi)
    S = sum(abs(x) for x in s) / 4
    phi = min(1.0, (M - u) / S, (u - m) / S) if S > 0 else 1.0
    return u + phi * sum(sigma[d] * s[d] for d in range(D)) / 4


def coarse_cell(x, h, n):
    """The coarse cell of spacing ``h`` a point lies in, wrapped onto a
    periodic grid of ``n`` cells, and the side of its centre it is on."""
    I = tuple(int(np.floor(xd / h)) % n for xd in x)
    sigma = tuple(1 if xd - (np.floor(xd / h) + 0.5) * h > 0 else -1 for xd in x)
    return I, sigma


def _points(fs, b, rng_per_dim):
    pos = fs.positions(b)
    for idx in np.ndindex(*[len(r) for r in rng_per_dim]):
        I = tuple(rng_per_dim[d][idx[d]] for d in range(fs.D))
        yield I, tuple(float(pos[d][I[d] - 1]) for d in range(fs.D))


def _at(host, b, I, v=0):
    return host[(b, v) + tuple(i - 1 for i in reversed(I))]


def _fill_fn(fs, fn):
    """Every stored point of every block to ``fn(x)`` (a point's coordinates)."""
    host = np.zeros(tuple(fs.work.shape), dtype=fs.T)
    for b in range(fs.nblocks()):
        pos = fs.positions(b)
        for I in np.ndindex(*[len(p) for p in pos]):
            x = tuple(float(pos[d][I[d]]) for d in range(fs.D))
            host[(b, 0) + tuple(reversed(I))] = fn(x)
    fs.work = torch.from_numpy(host)
    return host


def _regrid_all(fs, ops):
    """Refine every leaf and move the data with the oracle's replay of the
    regrid transfer (the ghosts filled first, as ``regrid!`` does)."""
    from test_regrid import oracle_regrid
    f = fs.forest
    s = GhostSchedule(fs, ops)
    host = oracle.fill(s, fs.work.numpy().copy(), fs.nvars, fs.factors_host)
    old = list(f.leaves)
    f.refine(old)
    f.balance()
    t = RegridTransfer(f, old, fs.G, fs.centering, fs.T, ops)
    new = np.zeros((f.nleaves(),) + tuple(fs.work.shape[1:]), fs.T)
    out = FieldSet(f, fs.nvars, G=fs.G, centering=fs.centering, T=fs.T)
    out.work = torch.from_numpy(oracle_regrid(t, host, new, fs.nvars))
    return out, t


def test_a_bound_is_refused_where_it_means_nothing():
    """``test/bounded_tests.jl:44-60``."""
    assert BOUNDED.bounded
    assert not Operators(prolongation=3, restriction=2, family=Conservative).bounded
    with pytest.raises(ValueError, match="prolongation = 3 or 1"):
        Operators(prolongation=5, restriction=2, family=Conservative, bounded=True)
    assert Operators(prolongation=6, restriction=4, bounded=True).bounded
    assert repr(Operators(prolongation=4, restriction=4, bounded=True)) == \
        "Operators(prolongation=4, restriction=4, family=PointValue, bounded=true)"
    assert repr(BOUNDED) == \
        "Operators(prolongation=3, restriction=2, family=Conservative, bounded=true)"
    assert repr(Operators(prolongation=3, restriction=2, family=Conservative)) == \
        "Operators(prolongation=3, restriction=2, family=Conservative)"
    with pytest.raises(ValueError, match="vertex_prolongation"):
        Operators(prolongation=3, restriction=2, family=Conservative, bounded=True,
                  vertex_prolongation=2)


@pytest.mark.parametrize("D", [1, 2, 3])
def test_bounded_orders_that_are_bounded_already_change_nothing(D):
    """``test/bounded_tests.jl:62-87, 314-339``: conservative order 1 copies
    the parent and point-value width 2 is linear interpolation: every group
    stays unbounded and the fill is the plain one bit for bit."""
    pairs = [(Operators(prolongation=1, restriction=2, family=Conservative),
              Operators(prolongation=1, restriction=2, family=Conservative, bounded=True),
              None),
             (Operators(prolongation=2, restriction=2),
              Operators(prolongation=2, restriction=2, bounded=True), None),
             (Operators(prolongation=2, restriction=2),
              Operators(prolongation=2, restriction=2, bounded=True), vertexcentered(D))]
    for plain, ops, C in pairs:
        outs = []
        for o in (plain, ops):
            f = nested_forest(D, N=8, periodic=(True,) * D)
            fs = FieldSet(f, 1, G=1, centering=C)
            _fill_fn(fs, lambda x: (sum(97.13 * (d + 1.37) * x[d] for d in range(D))) % 1)
            s = GhostSchedule(fs, o)
            assert all(g.bounded == UNBOUNDED for g in s.groups)
            outs.append(oracle.fill(s, fs.work.numpy().copy(), 1, fs.factors_host))
        assert np.array_equal(nanbits(outs[0]), nanbits(outs[1]))


@pytest.mark.parametrize("D", [1, 2, 3])
def test_a_refined_child_is_the_bounded_reconstruction(D):
    """``test/bounded_tests.jl:89-113``: a periodic brick refined everywhere
    at once; every child is the formula applied to the coarse grid."""
    N = 4 if D == 3 else 8
    f = Forest((2,) * D, N=N, periodic=(True,) * D, extents=((0.0, 2.0),) * D)
    n, h = 2 * N, 2 / (2 * N)
    U = np.random.default_rng(40 + D).uniform(size=(n,) * D)
    fs = FieldSet(f, 1, G=1)
    _fill_fn(fs, lambda x: U[coarse_cell(x, h, n)[0]])
    out, t = _regrid_all(fs, BOUNDED)
    assert any(g.bounded == BOUNDED_CONSERVATIVE for g in t.groups)
    host = out.work.numpy()
    worst = 0.0
    for b in range(out.nblocks()):
        for I, x in _points(out, b, [range(2, N + 2)] * D):
            Ic, sig = coarse_cell(x, h, n)
            worst = max(worst, abs(_at(host, b, I) - bounded_child(U, Ic, sig)))
    assert worst < 1e-14


@pytest.mark.parametrize("D", [1, 2, 3])
def test_a_ghost_across_a_coarse_fine_face_is_the_bounded_reconstruction(D):
    """``test/bounded_tests.jl:115-158``: every fine ghost lying in a coarse
    leaf is the formula applied to the coarse picture of the mesh."""
    N, roots = 4, 4
    f = Forest((roots,) * D, N=N, periodic=(True,) * D, extents=((0.0, float(roots)),) * D)

    def refined(x):
        return all((xd % roots) < 2 for xd in x)
    f.refine([k for k in f.leaves if refined(tuple(lo for lo, _ in f.block_extent(k)))])
    n, h = roots * N, 1 / N
    rng = np.random.default_rng(50 + D)
    U = rng.uniform(size=(n,) * D)
    Fg = rng.uniform(size=(2 * n,) * D)
    for I in np.ndindex(*U.shape):
        x = tuple((I[d] + 0.5) * h for d in range(D))
        if refined(x):
            kids = [tuple(2 * I[d] + o[d] for d in range(D))
                    for o in np.ndindex(*(2,) * D)]
            U[I] = sum(Fg[J] for J in kids) / 2 ** D
    fs = FieldSet(f, 1, G=1)
    _fill_fn(fs, lambda x: Fg[coarse_cell(x, h / 2, 2 * n)[0]] if refined(x)
             else U[coarse_cell(x, h, n)[0]])
    s = GhostSchedule(fs, BOUNDED)
    host = oracle.fill(s, fs.work.numpy().copy(), 1, fs.factors_host)
    worst, checked = 0.0, 0
    for b, k in enumerate(f.leaves):
        if k.level != 1:
            continue
        for I, x in _points(fs, b, [range(1, N + 3)] * D):
            if refined(x):
                continue                                  # a copy or a restriction
            Ic, sig = coarse_cell(x, h, n)
            worst = max(worst, abs(_at(host, b, I) - bounded_child(U, Ic, sig)))
            checked += 1
    assert checked > 0 and worst < 1e-14


def bounded_point(U, x, h, cen, p, raw=False):
    """``test/bounded_tests.jl:283-306``: the clamped width-p interpolant of
    the periodic coarse grid ``U`` at ``x``."""
    D = U.ndim
    n = U.shape
    axes = []
    for d in range(D):
        xi = Fraction(round(4 * x[d] / h), 4) + (Fraction(1, 2) if cen == "cell" else 1)
        if xi.denominator == 1:
            axes.append((int(xi), [1.0], [int(xi)]))
            continue
        fl = xi.numerator // xi.denominator
        lo = fl - p // 2 + 1
        w = lagrange_weights([Fraction(j) for j in range(lo, lo + p)], xi)
        axes.append((lo, [float(v) for v in w], [fl, fl + 1]))
    acc = 0.0
    for m in np.ndindex(*[len(a[1]) for a in axes]):
        wt = 1.0
        for d in range(D):
            wt *= axes[d][1][m[d]]
        acc += wt * U[tuple((axes[d][0] + m[d] - 1) % n[d] for d in range(D))]
    if raw:
        return acc
    corners = [U[tuple((c[d] - 1) % n[d] for d in range(D))]
               for c in itertools.product(*[a[2] for a in axes])]
    return min(max(acc, min(corners)), max(corners))


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("cen", ["cell", "vertex"])
def test_a_refined_point_is_the_bounded_interpolant(D, cen):
    """``test/bounded_tests.jl:341-372``: every new point of a brick refined
    everywhere at once is the clamped interpolant; random data clamp often."""
    N = 6 if D == 3 else 8
    f = Forest((2,) * D, N=N, periodic=(True,) * D, extents=((0.0, 2.0),) * D)
    n, h = 2 * N, 2 / (2 * N)
    U = np.random.default_rng(80 + D).uniform(size=(n,) * D)
    C = (cen,) * D
    fs = FieldSet(f, 1, G=2, centering=C)

    def at(x):
        return tuple(int(round(xd / h + (0.5 if cen == "cell" else 1))) % n - 1 for xd in x)
    _fill_fn(fs, lambda x: U[at(x)])
    out, t = _regrid_all(fs, BOUNDED_PV)
    assert any(g.bounded == BOUNDED_POINTVALUE for g in t.groups)
    host = out.work.numpy()
    worst, clamped = 0.0, 0
    c = 1 if cen == "vertex" else 0
    for b in range(out.nblocks()):
        for I, x in _points(out, b, [range(3, N + 3 + c)] * D):
            want = bounded_point(U, x, h, cen, 4)
            worst = max(worst, abs(_at(host, b, I) - want))
            clamped += want != bounded_point(U, x, h, cen, 4, raw=True)
    assert worst < 1e-14 and clamped > 0


@pytest.mark.parametrize("D", [1, 2, 3])
def test_bounded_point_values_reproduce_a_monotone_cubic_bit_for_bit(D):
    """``test/bounded_tests.jl:374-393``: where no clamp acts the bounded
    value is the order-p interpolant itself, bit for bit."""
    f = nested_forest(D, N=8)

    def cubic(x, v):
        return v + sum(0.4 * (d + 1) * x[d] + 0.05 * x[d] ** 3 for d in range(D))
    for C in (None, vertexcentered(D)):
        works = []
        for ops in (PLAIN_PV, BOUNDED_PV):
            fs = FieldSet(f, 2, G=2, centering=C)
            fs.fill_by_coordinates(cubic)
            exact = fs.work.numpy().copy()
            s = GhostSchedule(fs, ops)
            works.append(oracle.fill_fieldset(fs, s, boundary_values=boundary_from(exact)))
            own = (slice(None), slice(None)) + fs.interior()
            assert np.max(np.abs(works[-1] - exact)) < 1e-11
        assert np.array_equal(nanbits(works[0]), nanbits(works[1]))


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("cen", ["cell", "vertex"])
def test_bounded_point_values_create_no_new_extrema(D, cen):
    """``test/bounded_tests.jl:395-431``: through the fill, random, step and
    surface data stay within their range; the unbounded control overshoots
    a step."""
    C = (cen,) * D
    N = 6 if D == 3 else 8
    for data in ("random", "step", "surface"):
        f = nested_forest(D, N=N, periodic=(True,) * D)
        fs = FieldSet(f, 1, G=2, centering=C)
        rng = np.random.default_rng(90 + D)
        fn = {"random": lambda x: rng.uniform(),
              "step": lambda x: 0.0 if x[0] < 1.3 else 1.0,
              "surface": lambda x: 1.0 if x[0] < 1.3 else 1.0e-13}[data]
        _fill_fn(fs, fn)
        out = oracle.fill(GhostSchedule(fs, BOUNDED_PV), fs.work.numpy().copy(), 1,
                          fs.factors_host)
        lower = 1.0e-13 if data == "surface" else 0.0
        assert lower <= out.min() and out.max() <= 1
    # the unbounded control, refined everywhere at once, overshoots
    f = nested_forest(D, N=N, periodic=(True,) * D)
    fs = FieldSet(f, 1, G=2, centering=C)
    _fill_fn(fs, lambda x: 1.0 if x[0] < 1.3 else 1.0e-13)
    plain, _ = _regrid_all(fs, PLAIN_PV)
    own = (slice(None), slice(None)) + plain.interior()     # the regrid moves own points
    assert plain.work.numpy()[own].min() < 0
    fs = FieldSet(nested_forest(D, N=N, periodic=(True,) * D), 1, G=2, centering=C)
    _fill_fn(fs, lambda x: 1.0 if x[0] < 1.3 else 1.0e-13)
    bounded, _ = _regrid_all(fs, BOUNDED_PV)
    assert bounded.work.numpy()[own].min() >= 1.0e-13


# --- the device -------------------------------------------------------------------------

def _gpu_cases(D):
    return [("conservative", None, BOUNDED, 1), ("pv-cell", None, BOUNDED_PV, 2),
            ("pv-vertex", vertexcentered(D), BOUNDED_PV, 2)]


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_bounded_fill_bit_exact(cuda_lib, D, T):
    """The device fill with bounded operators, fused (CPU form) and plain
    (device form), is the oracle's bit for bit, on random data that clamp."""
    from treeamr import fill_ghosts
    for name, C, ops, G in _gpu_cases(D):
        f = nested_forest(D, N=8, periodic=(True,) * D)
        fs = FieldSet(f, 2, G=G, centering=C, T=T)
        s = GhostSchedule(fs, ops)
        assert any(g.bounded for g in s.groups), name
        host = np.random.default_rng(D).uniform(-1, 1, size=tuple(fs.work.shape)).astype(T)
        fs.factors = fs.factors.cuda()
        for method, one_tap in (("fused", True), ("plain", False)):
            expect = oracle.fill(s, host.copy(), 2, fs.factors_host, one_tap=one_tap)
            fs.work = torch.from_numpy(host.copy()).cuda()
            fill_ghosts(fs, s, method=method)
            torch.cuda.synchronize()
            assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), \
                (name, method)


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
def test_gpu_bounded_awkward_data_bit_exact(cuda_lib, D):
    """+-0, NaN, +-Inf and subnormals through both bounds (the extrema and
    the clamp with Julia's NaN-propagating min and max): the device fill,
    fused and plain, is the oracle's bit for bit."""
    from _helpers import awkward_fill
    from treeamr import fill_ghosts
    for name, C, ops, G in _gpu_cases(D):
        f = nested_forest(D, N=8, periodic=(True,) * D)
        fs = FieldSet(f, 2, G=G, centering=C)
        s = GhostSchedule(fs, ops)
        host = awkward_fill(tuple(fs.work.shape), np.float64, seed=D + 3)
        fs.factors = fs.factors.cuda()
        for method, one_tap in (("fused", True), ("plain", False)):
            expect = oracle.fill(s, host.copy(), 2, fs.factors_host, one_tap=one_tap)
            fs.work = torch.from_numpy(host.copy()).cuda()
            fill_ghosts(fs, s, method=method)
            torch.cuda.synchronize()
            assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), \
                (name, method)


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
def test_gpu_bounded_regrid_bit_exact(cuda_lib, D):
    """A bounded regrid on the device (the children bounded) is the
    oracle's replay bit for bit; the adjoint of a bounded schedule is
    refused."""
    from test_regrid import oracle_regrid
    from treeamr.adjoint import fill_ghosts_adjoint
    for name, C, ops, G in _gpu_cases(D):
        f = nested_forest(D, N=8, periodic=(True,) * D)
        fs = FieldSet(f, 1, G=G, centering=C)
        host = np.random.default_rng(7).uniform(size=tuple(fs.work.shape))
        old = list(f.leaves)
        f.refine([k for k in old if k.level == 0][:3])
        f.balance()
        t = RegridTransfer(f, old, fs.G, fs.centering, fs.T, ops)
        assert any(g.bounded for g in t.groups), name
        new0 = np.full((f.nleaves(),) + tuple(fs.work.shape[1:]), np.nan)
        expect = oracle_regrid(t, host, new0.copy(), 1)
        dev = torch.from_numpy(new0.copy()).cuda()
        t.run(torch.from_numpy(host).cuda(), dev, 1)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(dev.cpu().numpy()), nanbits(expect)), name
    g = nested_forest(D, N=8, periodic=(True,) * D)
    gs = FieldSet(g, 1, G=1, device="cuda")
    with pytest.raises(Exception, match="no adjoint"):
        fill_ghosts_adjoint(gs, GhostSchedule(gs, BOUNDED))
