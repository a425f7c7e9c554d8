"""Stage 0 alone: ``UnifySchedule`` and ``unify`` (``src/unify.jl``), the
interface restriction of a flux set.  Restated from the reference's own
tests (``test/interface_tests.jl:21-138``) with their position oracle
(``test/ghost_oracles.jl:120-160, 400-485``): every coarse copy of a point a
finer block also holds comes back as the mean of the coincident fine values,
everything else keeps its value (NaN ghosts included), no target is
written twice, and mismatched schedules are refused.  On the GPU the
device unify is bit for bit the oracle's replay of the same schedule, on the
working array and on a state vector."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import Geometry, nanbits, nested_forest
from treeamr import FieldSet, GhostSchedule, Operators
from treeamr.storage import edgecentered, facecentered, vertexcentered
from treeamr.unify import UnifySchedule, unify


def interface_cases(D):
    return {1: [facecentered(1, 1)],
            2: [facecentered(2, 1), facecentered(2, 2), vertexcentered(2)],
            3: [facecentered(3, 1), facecentered(3, 3), edgecentered(3, 1)]}[D]


def arbitrary(x, v):
    """A value fixed by the exact position alone: a multiplicative hash of
    the integer coordinates, mapped to [-1, 1)."""
    with np.errstate(over="ignore"):                       # wrapping is the hash
        h = np.uint64(0x9E3779B97F4A7C15) * np.uint64(v + 1)
        for xd in x:
            h = (h ^ np.asarray(xd, dtype=np.uint64)) * np.uint64(0xBF58476D1CE4E5B9)
            h ^= h >> np.uint64(31)
    return (h >> np.uint64(11)).astype(np.float64) / float(1 << 53) * 2.0 - 1.0


def own_slices(fs):
    N = fs.forest.N
    return tuple(slice(g, g + N + cd) for g, cd in reversed(list(zip(fs.G, fs.c))))


def fill_arbitrary(fs, host, geo):
    f = fs.forest
    for b, k in enumerate(f.leaves):
        pts = geo.points(k, fs.G, fs.c, f.N)
        grids = np.meshgrid(*pts, indexing="ij")             # [d][i1, i2, ...]
        for v in range(fs.nvars):
            val = arbitrary(grids, v)
            host[(b, v) + own_slices(fs)] = np.transpose(val)


def closed_values(fs, host, geo):
    out = {}
    f = fs.forest
    for b, k in enumerate(f.leaves):
        pts = geo.points(k, fs.G, fs.c, f.N)
        own = host[(b, slice(None)) + own_slices(fs)]
        for I0 in np.ndindex(*[len(p) for p in pts]):
            key = (k.level,) + tuple(int(pts[d][I0[d]]) for d in range(f.D))
            out[key] = own[(slice(None),) + tuple(reversed(I0))]
    return out


def interface_targets(fs, values, geo):
    """``(block, 1-based stored index) -> expected values``
    (``test/ghost_oracles.jl:443-485``)."""
    f = fs.forest
    N, G, c, D = f.N, fs.G, fs.c, f.D
    boxes = {}
    for k in f.leaves:
        lo = np.array(geo.low(k))
        boxes.setdefault(k.level, []).append((lo, lo + (geo.scale >> k.level)))
    arr = {l: (np.array([b[0] for b in bx]), np.array([b[1] for b in bx]))
           for l, bx in boxes.items()}
    period = np.array([f.roots[d] * geo.scale if f.periodic[d] else 0 for d in range(D)])

    def holds(l, p):
        lo, hi = arr[l]
        ok = np.ones(len(lo), bool)
        for d in range(D):
            x = p[d]
            inside = (lo[:, d] <= x) & (x <= hi[:, d])
            if period[d]:
                inside |= (lo[:, d] <= x + period[d]) & (x + period[d] <= hi[:, d])
            ok &= inside
        return ok.any()

    out = {}
    for b, k in enumerate(f.leaves):
        l = k.level
        if l + 1 not in arr:
            continue
        half = 1 << (geo.L - l - 1)           # half a spacing of level l + 1
        shifts = list(np.ndindex(*[2 if c[e] == 0 else 1 for e in range(D)]))
        pts = geo.points(k, G, c, N)
        for I0 in np.ndindex(*[len(pp) for pp in pts]):
            if not any(c[d] == 1 and I0[d] in (0, N) for d in range(D)):
                continue
            p = [int(pts[d][I0[d]]) for d in range(D)]
            if not holds(l + 1, p):
                continue
            acc = np.zeros(fs.nvars)
            for sh in shifts:
                q = tuple(int(geo.wrap(e, p[e] + ((2 * sh[e] - 1) * half if c[e] == 0 else 0)))
                          for e in range(D))
                acc += values[(l + 1,) + q]
            out[(b, tuple(i + 1 + g for i, g in zip(I0, G)))] = acc / len(shifts)
    return out


def _unified(fs, s, host):
    return oracle.fill(s, host.copy(), fs.nvars, fs.factors_host, first=-1, last=0)


@pytest.mark.parametrize("D", [1, 2, 3])
def test_unify_makes_every_coarse_copy_the_fine_average(D):
    forest = nested_forest(D, N=8, periodic=(D % 2 == 1,) * D)
    assert len({k.level for k in forest.leaves}) >= 3
    for C in interface_cases(D):
        for G in (0, 1):
            fs = FieldSet(forest, 2, G=G, centering=C)
            geo = Geometry(forest)
            host = np.full(tuple(fs.work.shape), np.nan)
            fill_arbitrary(fs, host, geo)
            expected = interface_targets(fs, closed_values(fs, host, geo), geo)
            assert expected
            s = UnifySchedule(fs)
            out = _unified(fs, s, host)
            worst = 0.0
            targets = set()
            for (b, I), want in expected.items():
                sl = tuple(i - 1 for i in reversed(I))
                got = out[(b, slice(None)) + sl]
                worst = max(worst, float(np.max(np.abs(got - want))))
                targets.add((b,) + sl)
            assert worst <= 4 * np.finfo(np.float64).eps
            # everything else keeps its value, NaN ghosts included
            mask = np.ones(out.shape, bool)
            for t in targets:
                mask[(t[0], slice(None)) + t[1:]] = False
            assert np.array_equal(nanbits(out[mask]), nanbits(host[mask]))
            own = (slice(None), slice(None)) + tuple(
                slice(g, g + forest.N + cd) for g, cd in reversed(list(zip(fs.G, fs.c))))
            assert not np.isnan(out[own]).any()


@pytest.mark.parametrize("D", [2, 3])
def test_unify_writes_every_target_once(D):
    forest = nested_forest(D, N=8)
    for C in interface_cases(D):
        fs = FieldSet(forest, 1, G=1, centering=C)
        s = UnifySchedule(fs)
        counts = np.zeros((forest.nleaves(),) + tuple(reversed(s.stored)), dtype=np.int64)
        for g in s.unify:
            sl = tuple(slice(st.targetfirst - 1, st.targetfirst - 1 + st.ntarget)
                       for st in reversed(g.stencils))
            for tb in g.targetblocks:
                counts[(tb - 1,) + sl] += 1
        assert counts.max() <= 1
        assert all(np.all(np.diff(g.targetblocks) >= 0) for g in s.unify)


def test_cell_centred_set_has_no_interface():
    forest = nested_forest(2, N=8)
    with pytest.raises(ValueError, match="no shared point"):
        UnifySchedule(FieldSet(forest, 1, G=2))
    with pytest.raises(ValueError, match=r"facecentered\(2, d\)"):
        UnifySchedule(FieldSet(forest, 1, G=2))


def test_unify_refuses_a_mismatched_schedule():
    forest = nested_forest(2, N=8)
    fs = FieldSet(forest, 1, G=1, centering=facecentered(2, 1))
    s = UnifySchedule(fs)
    assert not s.isstale()
    with pytest.raises(ValueError, match="ghost width"):
        unify(FieldSet(forest, 1, G=2, centering=facecentered(2, 1)), s)
    with pytest.raises(ValueError, match="centering"):
        unify(FieldSet(forest, 1, G=1, centering=vertexcentered(2)), s)
    with pytest.raises(ValueError, match="carries"):
        unify(FieldSet(forest, 1, G=1, centering=facecentered(2, 1), T=np.float32), s)
    with pytest.raises(ValueError, match="different forest"):
        unify(FieldSet(nested_forest(2, N=8), 1, G=1, centering=facecentered(2, 1)), s)
    forest.refine(forest.leaves[0])
    assert s.isstale()
    with pytest.raises(ValueError, match="rebuild it"):
        unify(fs, s)
    assert "UnifySchedule{float64,2}" in repr(s)


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_unify_bit_exact(cuda_lib, D, T):
    from treeamr.state import gather, statevector
    forest = nested_forest(D, N=8, periodic=(D % 2 == 1,) * D)
    for C in interface_cases(D):
        fs = FieldSet(forest, 3, G=1, centering=C, T=T)
        host = np.full(tuple(fs.work.shape), np.nan, dtype=T)
        fill_arbitrary(fs, host, Geometry(forest))
        s = UnifySchedule(fs)
        expect = _unified(fs, s, host)
        fs.work = torch.from_numpy(host.copy()).cuda()
        fs.factors = fs.factors.cuda()
        assert unify(fs, s) is fs
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect))
        # the same on a state vector
        fs.work = torch.from_numpy(host.copy()).cuda()
        u = statevector(fs)
        gather(u, fs)
        assert unify(u, fs, s) is u
        fs.work.copy_(torch.from_numpy(expect))
        want = statevector(fs)
        gather(want, fs)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(u.cpu().numpy()), nanbits(want.cpu().numpy()))


@pytest.mark.gpu
def test_gpu_unify_with_a_ghost_schedule(cuda_lib):
    """``unify!(fs, ::GhostSchedule)``: stages P and 0 of the fill's own
    schedule, with its operators' restriction."""
    D = 3
    forest = nested_forest(D, N=8)
    fs = FieldSet(forest, 2, G=2, centering=vertexcentered(D))
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    rng = np.random.default_rng(3)
    host = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    expect = oracle.fill(s, host.copy(), fs.nvars, fs.factors_host, first=-1, last=0)
    fs.work = torch.from_numpy(host.copy()).cuda()
    fs.factors = fs.factors.cuda()
    unify(fs, s)
    torch.cuda.synchronize()
    assert np.array_equal(fs.work.cpu().numpy(), expect)


@pytest.mark.parametrize("seed", range(8))
def test_unify_random_forests(seed):
    """The interface restriction on seeded random forests (2 or 3 roots a
    side, each dimension periodic or not, one to three passes refining a
    random quarter of the leaves, balanced), for every interface centering
    of the dimension and G = 0, 1: each coarse copy is the fine mean, and
    nothing else moves."""
    from treeamr import Forest
    rng = np.random.default_rng(8000 + seed)
    D, roots = int(rng.integers(1, 4)), int(rng.integers(2, 4))
    periodic = tuple(bool(rng.integers(2)) for _ in range(D))
    forest = Forest((roots,) * D, N=8, periodic=periodic, extents=[(0.0, float(roots))] * D)
    for _ in range(int(rng.integers(1, 4 if D < 3 else 3))):
        pick = [k for k in forest.leaves if rng.random() < 0.25]
        if pick:
            forest.refine(pick)
            forest.balance()
    geo = Geometry(forest)
    for C in interface_cases(D):
        for G in (0, 1):
            fs = FieldSet(forest, 2, G=G, centering=C)
            host = np.full(tuple(fs.work.shape), np.nan)
            fill_arbitrary(fs, host, geo)
            expected = interface_targets(fs, closed_values(fs, host, geo), geo)
            out = _unified(fs, UnifySchedule(fs), host)
            targets = set()
            for (b, I), want in expected.items():
                sl = tuple(i - 1 for i in reversed(I))
                assert np.max(np.abs(out[(b, slice(None)) + sl] - want)) <= \
                    4 * np.finfo(np.float64).eps
                targets.add((b,) + sl)
            mask = np.ones(out.shape, bool)
            for t in targets:
                mask[(t[0], slice(None)) + t[1:]] = False
            assert np.array_equal(nanbits(out[mask]), nanbits(host[mask]))
