"""The schedule and the oracle fill, against the reference's property tests
(``test/ghost_tests.jl:214-300, 455-483``, ``test/reflect_tests.jl``,
``test/outflow_tests.jl``).  CPU only."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import (exchange_error, exact_values, ghost_mask, makepoly, nested_forest,
                      periodic_vs_tiled)
from treeamr import (EvenParity, FieldSet, Forest, GhostSchedule, OddParity, Operators)
from treeamr.schedule import COPY, PROLONG, RESTRICT


@pytest.mark.parametrize("D", [1, 2, 3])
def test_schedule_partitions_the_ghost_cells(D):
    rng = np.random.default_rng(500 + D)
    for trial in range(3):
        f = Forest((2,) * D, N=4, periodic=tuple((d + 1 + trial) % 2 == 1 for d in range(D)))
        for _ in range(4):
            k = f.leaves[rng.integers(f.nleaves())]
            if k.level < 2:
                f.refine(k)
        f.balance()
        fs = FieldSet(f, 1, G=1)
        s = GhostSchedule(fs, Operators(prolongation=2, restriction=2))
        counts = s.write_counts()
        m = ghost_mask(fs)
        for b in range(f.nleaves()):
            assert (counts[b][m] == 1).all()
            assert (counts[b][~m] == 0).all()
        assert counts.sum() == f.nleaves() * (6 ** D - 4 ** D)


@pytest.mark.parametrize("D", [1, 2, 3])
def test_exchange_exact_for_polynomials(D):
    f = nested_forest(D)
    assert f.isbalanced()
    assert len({k.level for k in f.leaves}) >= 3
    ops = Operators(prolongation=2, restriction=2)
    counts = GhostSchedule(FieldSet(f, 1, G=1), ops).transfer_counts()
    assert counts[COPY] > 0 and counts[RESTRICT] > 0 and counts[PROLONG] > 0
    assert exchange_error(f, ops, makepoly(D, 1)) < 1e-12
    assert exchange_error(f, ops, makepoly(D, 2)) > 1e-6
    wide = nested_forest(D, N=8)
    ops4 = Operators(prolongation=4, restriction=4)
    assert exchange_error(wide, ops4, makepoly(D, 3), G=2) < 1e-10
    assert exchange_error(wide, ops4, makepoly(D, 4), G=2) > 1e-8


@pytest.mark.parametrize("D", [1, 2])
def test_order6_exchange(D):
    f = nested_forest(D, N=8)
    ops = Operators(prolongation=6, restriction=6)
    assert exchange_error(f, ops, makepoly(D, 5), G=3) < 1e-9
    assert exchange_error(f, ops, makepoly(D, 6), G=3) > 1e-9


@pytest.mark.parametrize("D", [1, 2, 3])
def test_three_level_corners(D):
    f = nested_forest(D)
    s = GhostSchedule(FieldSet(f, 1, G=1), Operators(prolongation=2, restriction=2))
    assert len(s.levels) >= 2 and s.levels == sorted(s.levels)
    assert len(s.phase2) == len(s.levels)


@pytest.mark.parametrize("D,M", [(1, 1), (1, 2), (2, 1), (2, 2), (3, 1)])
def test_periodic_equals_tiling_bit_for_bit(D, M):
    r = periodic_vs_tiled(D, M)
    assert r is not None
    diff, ncells = r
    assert diff == 0.0
    assert ncells > 0


@pytest.mark.parametrize("D", [1, 2, 3])
def test_interiors_untouched(D):
    f = Forest((2,) * D, N=4, periodic=(True,) * D)
    f.refine(f.leaves[0])
    f.balance()
    fs = FieldSet(f, 2, G=1)
    exact_values(fs, makepoly(D, 1))
    before = fs.work.numpy().copy()
    out = oracle.fill_fieldset(fs, GhostSchedule(fs, Operators(prolongation=2, restriction=2)))
    inter = (slice(None), slice(None)) + fs.interior()
    assert np.array_equal(out[inter], before[inter])
    assert not np.array_equal(out, before)


def test_conservative_exchange_cell_averages():
    # The conservative family reproduces cell averages of degree p-1:
    # checked through the weights' moments on the 1-D mesh.
    from fractions import Fraction as F
    from treeamr.operators import conservative_prolong_weights
    for p in (1, 3, 5):
        low, high = conservative_prolong_weights(p)
        r = (p - 1) // 2
        for deg in range(p):
            # averages of x^deg over unit cells centred at t - r
            def avg(c0, c1):
                return (F(c1) ** (deg + 1) - F(c0) ** (deg + 1)) / (deg + 1) / (c1 - c0)
            coarse = [avg(F(t - r) - F(1, 2), F(t - r) + F(1, 2)) for t in range(p)]
            assert sum(w * u for w, u in zip(low, coarse)) == avg(F(-1, 2), F(0))
            assert sum(w * u for w, u in zip(high, coarse)) == avg(F(0), F(1, 2))


def _faces_forest(D, lo_kind, hi_kind, N=8):
    refl = tuple((lo_kind == "reflect", hi_kind == "reflect") for _ in range(D))
    outf = tuple((lo_kind == "outflow", hi_kind == "outflow") for _ in range(D))
    f = Forest((2,) * D, N=N, reflecting=refl, outflow=outf, extents=[(0.0, 2.0)] * D)
    f.refine(f.leaves[0])
    f.balance()
    return f


@pytest.mark.parametrize("D", [1, 2, 3])
def test_reflecting_parity_polynomials(D):
    """Even data mirror to themselves, odd data change sign: a field even (or
    odd) about the low walls is exact across them (``test/reflect_tests.jl:98-131``)."""
    f = _faces_forest(D, "reflect", "none")
    ops = Operators(prolongation=4, restriction=4)
    parity = [(EvenParity,) * D, tuple(OddParity if d == 0 else EvenParity for d in range(D))]
    fs = FieldSet(f, 2, G=2, parity=parity)

    def fn(x, v):
        even = sum((x[d] ** 2) * (0.5 + d) for d in range(D)) + 1.0
        return even if v == 0 else x[0] * (1.0 + sum(x[d] ** 2 for d in range(1, D)))

    exact = exact_values(fs, fn)
    host = exact.copy()
    host[:, :, ghost_mask(fs)] = np.nan
    fs.work.copy_(torch.from_numpy(host))
    s = GhostSchedule(fs, ops)

    def bv(h, fs_, regions):
        for r in regions:
            sl = tuple(slice(a - 1, z) for a, z in reversed(r.region))
            h[(r.block, slice(None)) + sl] = exact[(r.block, slice(None)) + sl]
    out = oracle.fill_fieldset(fs, s, boundary_values=bv)
    assert not np.isnan(out).any()
    assert np.max(np.abs(out - exact)) < 1e-10
    # the wrong parity fails
    fs_bad = FieldSet(f, 2, G=2, parity=[parity[1], parity[0]])
    fs_bad.work.copy_(torch.from_numpy(host))
    out_bad = oracle.fill_fieldset(fs_bad, GhostSchedule(fs_bad, ops), boundary_values=bv)
    assert np.nanmax(np.abs(out_bad - exact)) > 1e-3


@pytest.mark.parametrize("D", [1, 2, 3])
def test_outflow_ghost_is_nearest_owned_point(D):
    """Across an outflow face every ghost holds the nearest owned row's value
    (``test/outflow_tests.jl:123-151``)."""
    f = Forest((1,) * D, N=8, outflow=tuple((True, True) for _ in range(D)))
    fs = FieldSet(f, 1, G=2)
    rng = np.random.default_rng(7)
    host = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    fs.work.copy_(torch.from_numpy(host))
    out = oracle.fill_fieldset(fs, GhostSchedule(fs, Operators(prolongation=2, restriction=2)))
    G, N = 2, 8
    idx = np.indices(tuple(reversed(fs.stored)))
    near = [np.clip(idx[k], G, G + N - 1) for k in range(D)]
    expect = out[0, 0][tuple(near)]
    assert np.array_equal(out[0, 0], expect)


def test_grouped_fill_leaves_no_nan_from_prefill():
    f = nested_forest(3, N=8)
    fs = FieldSet(f, 1, G=2)
    exact = exact_values(fs, makepoly(3, 1))
    host = exact.copy()
    host[:, :, ghost_mask(fs)] = np.nan
    fs.work.copy_(torch.from_numpy(host))
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))

    def bv(h, fs_, regions):
        for r in regions:
            sl = tuple(slice(a - 1, z) for a, z in reversed(r.region))
            h[(r.block, slice(None)) + sl] = exact[(r.block, slice(None)) + sl]
    out = oracle.fill_fieldset(fs, s, boundary_values=bv, nthreads=4)
    assert not np.isnan(out).any()
    # threaded and serial oracle agree bit for bit
    out1 = oracle.fill_fieldset(fs, s, boundary_values=bv, nthreads=1)
    assert np.array_equal(out.view(np.uint64), out1.view(np.uint64))


def test_stale_schedule_refused():
    f = Forest((2, 2), N=4, periodic=(True, True))
    fs = FieldSet(f, 1, G=1)
    s = GhostSchedule(fs, Operators(prolongation=2, restriction=2))
    assert not s.isstale()
    f.refine(f.leaves[0])
    assert s.isstale()
    from treeamr.ghosts import check_fill
    with pytest.raises(ValueError, match="stale"):
        check_fill(fs, s)


def test_layout_checks():
    f = Forest((2,), N=4)
    with pytest.raises(ValueError):
        GhostSchedule(FieldSet(f, 1, G=2), Operators(prolongation=6, restriction=2))
    with pytest.raises(ValueError):
        FieldSet(f, 1, G=3)
