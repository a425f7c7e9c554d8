"""The regrid transfer (``src/regrid.jl:585-756, 942-955``): classification
of new leaves (copy, prolongation from the parent, restriction from the
children), exactness on polynomial data of degree p-1 for created and
coarsened blocks with kept blocks copied bit for bit (the properties of
``test/regrid_tests.jl``), and on the GPU the device transfer equal to the
oracle's replay of the same groups bit for bit.

The kept-over-created pass (``src/regrid.jl:788-881``) is restated from
``test/closed_tests.jl:1129-1236``: a periodic brick refined over its high
half along dimension 1, whose low half the regrid refines, so that created
fine blocks meet kept fine blocks on the planes x1 = 0 and 1.  After the
regrid and before any fill every created copy of a point a kept block holds
at the finest level is the kept block's old value bit for bit, and the
next fill leaves the kept values there unchanged."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import Geometry, exact_values, makepoly, nanbits, nested_forest
from treeamr import FieldSet, Forest, GhostSchedule, Operators
from treeamr.forest import parentkey
from treeamr.regrid import (REGRID_KEPT_TAG, REGRID_TAG, RegridTransfer, regrid,
                            regrid_kept_pairs, regrid_sources)
from treeamr.schedule import COPY, PROLONG, RESTRICT, TransferGroup
from treeamr.storage import edgecentered, facecentered


def _move(D, N=8):
    """A nested forest, then one leaf refined and one family coarsened."""
    f = nested_forest(D, N=N)
    old = list(f.leaves)
    fine = [k for k in old if k.level == max(x.level for x in old)]
    fam = parentkey(fine[0])
    level0 = [k for k in old if k.level == 0]
    f.coarsen([fam])
    f.refine([level0[-1]])
    f.balance()
    return f, old


class _Concat:
    """The transfer over one array: new blocks first, then the old ones, so
    the oracle's fill replays it (sources moved past the new blocks)."""

    def __init__(self, t):
        self.T, self.stored = t.T, t.stored

        class F:
            D = t.forest.D

            @staticmethod
            def nleaves():
                return t.nnew + t.nold
        self.forest = F
        self.groups = [TransferGroup(g.key, g.stencils, g.targetblocks,
                                     np.asarray(g.sourceblocks) + t.nnew, 0, REGRID_TAG, None,
                                     g.bounded)
                       for g in t.groups]

    def all_groups(self):
        return self.groups


class _Kept:
    """The kept-over-created pass as a schedule over the new array."""

    def __init__(self, t):
        self.T, self.stored, self.forest = t.T, t.stored, t.forest
        self.groups = t.kept_groups

    def all_groups(self):
        return self.groups


def oracle_regrid(t, old_host, new_host, nvars, kept=True):
    """The oracle's replay of both stages: the transfer, then the
    kept-over-created pass within the new array."""
    both = np.concatenate([new_host, old_host], axis=0)
    ones = np.ones((nvars, 3 ** t.forest.D), t.T)
    oracle.fill(_Concat(t), both, nvars, ones)
    new = np.ascontiguousarray(both[:t.nnew])
    if kept and t.kept_groups:
        oracle.fill(_Kept(t), new, nvars, ones)
    return new


def half_refined(D, N=8):
    """``test/closed_tests.jl:1134-1140``: 2^D periodic roots on (0, 2)^D,
    those with x1 >= 1 refined once."""
    f = Forest((2,) * D, N=N, periodic=(True,) * D, extents=((0.0, 2.0),) * D)
    f.refine([k for k in f.leaves if f.root_position(k.root)[0] >= 1])
    f.balance()
    return f


def kept_created(forest, oldleaves, G, c):
    """Per point that kept and created new leaves both hold at the finest
    level holding it: ``([(new block, old block, own index)], [(new block,
    own index)])`` (``test/closed_tests.jl:1145-1157``)."""
    geo = Geometry(forest)
    N, D = forest.N, forest.D
    old = {k: i for i, k in enumerate(oldleaves)}
    byposition = {}
    for b, k in enumerate(forest.leaves):
        pts = geo.points(k, G, c, N)
        for I in np.ndindex(*[len(p) for p in pts]):
            x = tuple(int(pts[d][I[d]]) for d in range(D))
            byposition.setdefault(x, []).append((k.level, b, I))
    out = []
    for copies in byposition.values():
        finest = max(x[0] for x in copies)
        atf = [x for x in copies if x[0] == finest]
        kept = [(b, old[forest.leaves[b]], I) for _, b, I in atf if forest.leaves[b] in old]
        created = [(b, I) for _, b, I in atf if forest.leaves[b] not in old]
        if kept and created:
            out.append((kept, created))
    return out


def _at(arr, b, I, G):
    return arr[(b, slice(None)) + tuple(reversed([g + i for g, i in zip(G, I)]))]


def kept_cases(D):
    out = [("vertex",) * D, ("cell",) * D]
    if D >= 2:
        out += [facecentered(D, 1), facecentered(D, 2)]
    if D == 3:
        out += [edgecentered(3, 1)]
    return out


def _kept_run(D, C, T=np.float64, nvars=2, seed=0):
    """Fill (unify) the old storage with the oracle, regrid on the host
    with and without the kept pass; returns everything the checks need."""
    ops = Operators(prolongation=4, restriction=4)
    f = half_refined(D)
    fs = FieldSet(f, nvars, G=2, centering=C, T=T)
    rng = np.random.default_rng(60 + D + seed)
    fs.work.copy_(torch.from_numpy(rng.standard_normal(tuple(fs.work.shape)).astype(T)))
    old_host = oracle.fill_fieldset(fs, GhostSchedule(fs, ops))
    oldleaves = list(f.leaves)
    f.refine([k for k in oldleaves if k.level == 0])
    f.balance()
    t = RegridTransfer(f, oldleaves, fs.G, C, T, ops)
    new0 = np.zeros((f.nleaves(),) + tuple(fs.work.shape[1:]), T)
    moved = oracle_regrid(t, old_host, new0.copy(), nvars)
    unkept = oracle_regrid(t, old_host, new0.copy(), nvars, kept=False)
    return f, fs, t, oldleaves, old_host, moved, unkept, ops


@pytest.mark.parametrize("D", [2, 3])
def test_classification(D):
    f, old = _move(D)
    pairs = regrid_sources(old, f.leaves)
    kinds = {}
    for key, (tb, sb) in pairs.items():
        kinds[key.kind] = kinds.get(key.kind, 0) + len(tb)
        assert all(np.diff(tb) >= 0)
    assert kinds[COPY] == sum(1 for k in f.leaves if k in set(old))
    assert kinds[RESTRICT] % (2 ** D) == 0 and kinds[RESTRICT] >= 2 ** D
    assert kinds[PROLONG] % (2 ** D) == 0 and kinds[PROLONG] >= 2 ** D


@pytest.mark.parametrize("D", [2, 3])
def test_oracle_regrid_exact_for_polynomials(D):
    p = 4
    f, old = _move(D)
    new_leaves = list(f.leaves)
    # the old layout's exact data, ghosts included
    f_old = nested_forest(D, N=8)
    fs_old = FieldSet(f_old, 2, G=2)
    old_host = exact_values(fs_old, makepoly(D, p - 1))
    fs_new = FieldSet(f, 2, G=2)
    want = exact_values(fs_new, makepoly(D, p - 1))
    t = RegridTransfer(f, old, (2,) * D, ("cell",) * D, np.float64,
                       Operators(prolongation=p, restriction=p))
    new_host = np.full(tuple(fs_new.work.shape), np.nan)
    got = oracle_regrid(t, old_host, new_host, 2)
    own = (slice(None), slice(None)) + tuple(slice(2, 10) for _ in range(D))
    assert not np.isnan(got[own]).any()
    assert np.max(np.abs(got[own] - want[own])) < 1e-10
    # kept blocks: bit for bit
    index = {k: i for i, k in enumerate(old)}
    for b, k in enumerate(new_leaves):
        if k in index:
            assert np.array_equal(got[(b,) + own[1:]], old_host[(index[k],) + own[1:]])


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
@pytest.mark.parametrize("centering", ["cell", "vertex"])
def test_gpu_regrid_bit_exact(cuda_lib, D, T, centering):
    f, old = _move(D)
    C = ("vertex",) * D if centering == "vertex" else ("cell",) * D
    t = RegridTransfer(f, old, (2,) * D, C, T, Operators(prolongation=4, restriction=4))
    S = t.stored
    rng = np.random.default_rng(D)
    old_host = rng.uniform(-1, 1, size=(len(old), 3) + tuple(reversed(S))).astype(T)
    new_host = np.full((f.nleaves(), 3) + tuple(reversed(S)), np.nan, dtype=T)
    expect = oracle_regrid(t, old_host, new_host.copy(), 3)
    new_dev = torch.from_numpy(new_host).cuda()
    t.run(torch.from_numpy(old_host).cuda(), new_dev, 3)
    torch.cuda.synchronize()
    assert np.array_equal(nanbits(new_dev.cpu().numpy()), nanbits(expect))
    with pytest.raises(ValueError):
        t.run(torch.from_numpy(old_host).cuda(), new_dev[:-1], 3)


@pytest.mark.gpu
def test_gpu_regrid_of_a_field_set(cuda_lib):
    """``regrid`` moves a field set's own points through a refinement and a
    coarsening; degree-3 data stay exact under order-4 operators."""
    D, p = 3, 4
    f = nested_forest(D, N=8)
    fs = FieldSet(f, 1, G=2, device="cuda")
    fs.work.copy_(torch.from_numpy(exact_values(fs, makepoly(D, p - 1))))
    fine = [k for k in f.leaves if k.level == max(x.level for x in f.leaves)]
    level0 = [k for k in f.leaves if k.level == 0]
    regrid(fs, Operators(prolongation=p, restriction=p), refine=[level0[-1]],
           coarsen=[parentkey(fine[0])])
    assert fs.work.shape[0] == f.nleaves()
    want = exact_values(FieldSet(f, 1, G=2), makepoly(D, p - 1))
    own = (slice(None), slice(None)) + tuple(slice(2, 10) for _ in range(D))
    got = fs.work.cpu().numpy()
    assert np.max(np.abs(got[own] - want[own])) < 1e-10


@pytest.mark.parametrize("D", [1, 2, 3])
def test_kept_over_created_oracle(D):
    """Only a set vertex-like along dimension 1 shares the planes x1 = 0 and
    1 between kept and created fine blocks; there every created copy is the
    kept block's old value bit for bit (without the pass the interpolated
    hanging points of a plane are not), and the next fill keeps the kept
    values."""
    for C in kept_cases(D):
        f, fs, t, oldleaves, old_host, moved, unkept, ops = _kept_run(D, C)
        c = t.c
        pairs = kept_created(f, oldleaves, t.G, c)
        if c[0] == 1:
            assert pairs and t.kept_groups, C
            assert all(g.stage == REGRID_KEPT_TAG and g.kind == COPY for g in t.kept_groups)
        else:
            assert not pairs and not t.kept_groups, C
            continue
        differs = False
        for kept, created in pairs:
            b0, o0, I0 = kept[0]
            want = _at(old_host, o0, I0, t.G).view(np.uint64)
            for b, o, I in kept:
                assert np.array_equal(_at(old_host, o, I, t.G).view(np.uint64), want)
            for b, I in created:
                assert np.array_equal(_at(moved, b, I, t.G).view(np.uint64), want), (C, b, I)
                differs |= not np.array_equal(_at(unkept, b, I, t.G).view(np.uint64), want)
        # in 1-D the shared points are coarse vertices, which a prolongation
        # injects; on a plane the hanging points are interpolated
        assert differs == (D >= 2), C
        # the kept-over-created targets are disjoint: each point written once
        seen = set()
        for g in t.kept_groups:
            box = [range(s.targetfirst, s.targetfirst + s.ntarget) for s in g.stencils]
            for tb in g.targetblocks:
                for I in np.ndindex(*[len(r) for r in box]):
                    p = (int(tb),) + tuple(box[d][I[d]] for d in range(D))
                    assert p not in seen
                    seen.add(p)
        # the next fill keeps every kept value at those points
        fs2 = FieldSet(f, fs.nvars, G=2, centering=C, T=fs.T)
        fs2.work.copy_(torch.from_numpy(moved))
        filled = oracle.fill_fieldset(fs2, GhostSchedule(fs2, ops))
        for kept, _ in pairs:
            for b, o, I in kept:
                assert np.array_equal(_at(filled, b, I, t.G).view(np.uint64),
                                      _at(old_host, o, I, t.G).view(np.uint64))


def test_kept_pairs_need_a_vertex_like_dimension():
    f = half_refined(2)
    old = list(f.leaves)
    f.refine([k for k in old if k.level == 0])
    f.balance()
    assert regrid_kept_pairs(f, old, (0, 0)) == {}
    assert regrid_kept_pairs(f, old, (1, 1))
    # nothing created: nothing to copy
    assert regrid_kept_pairs(f, list(f.leaves), (1, 1)) == {}


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_kept_over_created_bit_exact(cuda_lib, D, T):
    """The device transfer with its kept-over-created pass equals the
    oracle's replay of both stages bit for bit."""
    for C in (("vertex",) * D, facecentered(D, 1)):
        f, fs, t, oldleaves, old_host, moved, unkept, ops = _kept_run(D, C, T=T, nvars=3)
        assert t.kept_groups
        new_dev = torch.zeros((f.nleaves(),) + tuple(fs.work.shape[1:]), dtype=fs.work.dtype,
                              device="cuda")
        t.run(torch.from_numpy(old_host).cuda(), new_dev, 3)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(new_dev.cpu().numpy()), nanbits(moved)), C


@pytest.mark.gpu
def test_gpu_regrid_keeps_evolved_values(cuda_lib):
    """``regrid`` of a vertex-centred set on the device: fill, transfer,
    kept-over-created pass, bit for bit the oracle's."""
    D, C = 3, ("vertex",) * 3
    f, fs, t, oldleaves, old_host, moved, unkept, ops = _kept_run(D, C)
    g = half_refined(D)
    gs = FieldSet(g, fs.nvars, G=2, centering=C, device="cuda")
    rng = np.random.default_rng(60 + D)
    gs.work.copy_(torch.from_numpy(rng.standard_normal(tuple(gs.work.shape))))
    regrid(gs, ops, refine=[k for k in g.leaves if k.level == 0])
    torch.cuda.synchronize()
    assert np.array_equal(nanbits(gs.work.cpu().numpy()), nanbits(moved))


def _random_grown(D, seed):
    """A brick of 3^D roots on (0, 3)^D, one or two passes refining a seeded
    third of the leaves, each balanced."""
    rng = np.random.default_rng(seed)
    f = Forest((3,) * D, N=8, periodic=(False,) * D, extents=[(0.0, 3.0)] * D)
    for _ in range(int(rng.integers(1, 3))):
        pick = [k for k in f.leaves if rng.random() < 0.3]
        if pick:
            f.refine(pick)
            f.balance()
    return f


@pytest.mark.parametrize("seed", range(16))
def test_oracle_regrid_random_moves(seed):
    """Seeded regrids: a random forest, then a random set of complete
    families coarsened and of leaves refined, and balance.  The transfer of
    degree p-1 data is exact at every own point of every new block (cell or
    vertex sets, orders 2 and 4, 1-D to 3-D), and kept blocks keep their own
    points bit for bit."""
    rng = np.random.default_rng(7000 + seed)
    D, p, vertex = int(rng.integers(1, 4)), int(rng.choice([2, 4])), bool(rng.integers(2))
    grow = int(rng.integers(1 << 30))
    f, f_old = _random_grown(D, grow), _random_grown(D, grow)
    old = list(f.leaves)
    assert list(f_old.leaves) == old
    children = {}
    for k in old:
        if k.level > 0:
            children.setdefault(parentkey(k), []).append(k)
    families = [q for q, ch in children.items() if len(ch) == 2 ** D]
    coarse = [q for q in families if rng.random() < 0.4]
    if coarse:
        f.coarsen(coarse)
    fine = [k for k in f.leaves if k not in set(coarse) and rng.random() < 0.15]
    if fine:
        f.refine(fine)
    f.balance()
    C = ("vertex",) * D if vertex else ("cell",) * D
    poly = makepoly(D, p - 1)
    fs_old = FieldSet(f_old, 2, G=2, centering=C)
    fs_new = FieldSet(f, 2, G=2, centering=C)
    old_host = exact_values(fs_old, poly)
    want = exact_values(fs_new, poly)
    t = RegridTransfer(f, old, (2,) * D, C, np.float64, Operators(prolongation=p, restriction=p))
    got = oracle_regrid(t, old_host, np.full(tuple(fs_new.work.shape), np.nan), 2)
    own = (slice(None), slice(None)) + tuple(slice(2, 10 + int(vertex)) for _ in range(D))
    assert not np.isnan(got[own]).any()
    assert np.max(np.abs(got[own] - want[own])) < 1e-9
    index = {k: i for i, k in enumerate(old)}
    for b, k in enumerate(f.leaves):
        if k in index:
            assert np.array_equal(got[(b,) + own[1:]], old_host[(index[k],) + own[1:]])
