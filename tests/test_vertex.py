"""Vertex-centred layouts: closed blocks, stage 0 and stage P.

Restates the reference's closed-block properties (``test/closed_tests.jl``,
``test/ghost_oracles.jl:420-470`` ``closed_values``, ``test/reflect_tests.jl``,
``test/outflow_tests.jl``) on the oracle, then checks the CUDA engine against
the oracle bit for bit."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import (awkward_fill, boundary_from, exact_values, ghost_mask, makepoly, nanbits,
                      nested_forest)
from treeamr import (EvenParity, FieldSet, Forest, GhostSchedule, OddParity, Operators,
                     fill_ghosts, meshes, vertexcentered)
from treeamr.schedule import SELFIMAGE_TAG, UNIFY_TAG


def _own_copies_consistent(fs, out, periodic):
    """Every stored copy of every point of any block's closed range holds one
    value: the primary's (stage 0; ``closed_values``)."""
    f = fs.forest
    D, N = f.D, f.N
    G = fs.G
    L = f.maxlevel()
    vals, bad = {}, 0
    for b, k in enumerate(f.leaves):
        B = f.block_base(k)
        sc = 1 << (L - k.level)
        for idx in np.ndindex(*([N + 1] * D)):
            pos = tuple((B[d] + idx[d]) * sc for d in range(D))
            if periodic:
                pos = tuple(p % ((f.roots[d] * N) << L) for d, p in enumerate(pos))
            v = out[(b, slice(None)) + tuple(reversed([G[d] + idx[d] for d in range(D)]))]
            v = v.view(np.uint64)
            if pos in vals:
                bad += int(not np.array_equal(vals[pos], v))
            else:
                vals[pos] = v.copy()
    return bad, len(vals)


@pytest.mark.parametrize("D", [1, 2, 3])
def test_vertex_partition(D):
    f = nested_forest(D, N=8)
    fs = FieldSet(f, 1, G=2, centering=vertexcentered(D))
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    counts = s.write_counts()
    m = ghost_mask(fs)
    for b in range(f.nleaves()):
        assert (counts[b][m] == 1).all()
        assert (counts[b][~m] == 0).all()
    assert s.unify and UNIFY_TAG in s.stage_tags


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("p", [2, 4])
def test_vertex_exact_for_polynomials(D, p):
    f = nested_forest(D, N=8)
    fs = FieldSet(f, 2, G=2, centering=vertexcentered(D))
    ops = Operators(prolongation=p, restriction=p)
    s = GhostSchedule(fs, ops)
    for deg, exact_expected in ((p - 1, True), (p, False)):
        exact = exact_values(fs, makepoly(D, deg))
        host = exact.copy()
        host[:, :, ghost_mask(fs)] = np.nan
        fs.work.copy_(torch.from_numpy(host))
        out = oracle.fill_fieldset(fs, s, boundary_values=boundary_from(exact))
        assert not np.isnan(out).any()
        err = np.max(np.abs(out - exact))
        if exact_expected:
            assert err < 1e-10
        else:
            assert err > 1e-9


@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("periodic", [False, True])
def test_every_copy_of_a_shared_point_agrees(D, periodic):
    f = nested_forest(D, N=8, periodic=(periodic,) * D)
    fs = FieldSet(f, 2, G=2, centering=vertexcentered(D))
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    rng = np.random.default_rng(D)
    host = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    fs.work.copy_(torch.from_numpy(host))
    exact = host.copy()
    out = oracle.fill_fieldset(fs, s, boundary_values=boundary_from(exact))
    bad, n = _own_copies_consistent(fs, out, periodic)
    assert n > 0 and bad == 0


def _walls_forest(D, N=8, levels=2):
    refl = tuple((True, False) for _ in range(D))
    outf = tuple((False, True) for _ in range(D))
    f = Forest((2,) * D, N=N, reflecting=refl, outflow=outf, extents=[(0.0, 2.0)] * D)
    for _ in range(levels):
        f.refine(f.leaves[0])
        f.balance()
    return f


@pytest.mark.parametrize("D", [1, 2, 3])
def test_vertex_reflecting_parity_and_stage_p(D):
    f = _walls_forest(D)
    par = [(EvenParity,) * D, tuple(OddParity if d == 0 else EvenParity for d in range(D))]
    fs = FieldSet(f, 2, G=2, centering=vertexcentered(D), parity=par)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    assert s.selfimage and SELFIMAGE_TAG in s.stage_tags

    def fn(x, v):
        if v == 0:
            return sum((x[d] ** 2) * (0.5 + d) for d in range(D)) + 1.0
        return x[0] * (1.0 + sum(x[d] ** 2 for d in range(1, D)))
    exact = exact_values(fs, fn)
    host = exact.copy()
    host[:, :, ghost_mask(fs)] = np.nan
    fs.work.copy_(torch.from_numpy(host))
    out = oracle.fill_fieldset(fs, s)
    assert not np.isnan(out).any()
    G, N = 2, 8
    low = np.ones(out.shape[2:], bool)
    for a in np.indices(out.shape[2:]):
        low &= a < G + N + 1                       # leave out the outflow (high) ghosts
    assert np.max(np.abs(out - exact)[:, :, low]) < 1e-12
    # random data: stage P zeroes the odd variable on the reflecting wall plane
    rng = np.random.default_rng(3)
    fs.work.copy_(torch.from_numpy(rng.uniform(-1, 1, size=host.shape)))
    out = oracle.fill_fieldset(fs, s)
    for b, k in enumerate(f.leaves):
        if k.coords[0] == 0 and f.root_position(k.root)[0] == 0:
            assert not np.any(out[b, 1][..., G])
            assert np.any(out[b, 0][..., G])


@pytest.mark.parametrize("D", [1, 2, 3])
def test_vertex_outflow_ghost_is_the_wall_row(D):
    f = Forest((1,) * D, N=8, outflow=tuple((True, True) for _ in range(D)))
    fs = FieldSet(f, 1, G=2, centering=vertexcentered(D))
    rng = np.random.default_rng(7)
    fs.work.copy_(torch.from_numpy(rng.uniform(-1, 1, size=tuple(fs.work.shape))))
    out = oracle.fill_fieldset(fs, GhostSchedule(fs, Operators(prolongation=2, restriction=2)))
    G, N = 2, 8
    idx = np.indices(tuple(reversed(fs.stored)))
    near = [np.clip(idx[k], G, G + N) for k in range(D)]
    assert np.array_equal(out[0, 0], out[0, 0][tuple(near)])


# --- the CUDA engine against the oracle --------------------------------------

def _gpu_fill(fs, s, host, method):
    fs.work = torch.from_numpy(host.copy()).cuda()
    fs.factors = fs.factors.cuda()
    fill_ghosts(fs, s, method=method)
    torch.cuda.synchronize()
    return fs.work.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["fused", "plain"])
@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_vertex_walls_bit_exact(cuda_lib, method, D, T):
    f = _walls_forest(D)
    par = [(EvenParity,) * D] * 2 + [tuple(OddParity if e == d else EvenParity
                                           for e in range(D)) for d in range(D)]
    fs = FieldSet(f, len(par), G=2, centering=vertexcentered(D), parity=par, T=T)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    host = awkward_fill(tuple(fs.work.shape), T, seed=D)
    fs.work.copy_(torch.from_numpy(host))
    # NaNs and infinities under zero weights: the fused kernels take the
    # reference's CPU form of the sum, the plain kernel its device form
    expect = oracle.fill_fieldset(fs, s, one_tap=method == "fused")
    got = _gpu_fill(fs, s, host, method)
    assert np.array_equal(nanbits(got), nanbits(expect))


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("periodic", [False, True])
def test_gpu_vertex_nested_bit_exact(cuda_lib, D, periodic):
    f = nested_forest(D, N=8, periodic=(periodic,) * D)
    fs = FieldSet(f, 3, G=2, centering=vertexcentered(D))
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    rng = np.random.default_rng(11)
    host = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    fs.work.copy_(torch.from_numpy(host))
    expect = oracle.fill_fieldset(fs, s)
    got = _gpu_fill(fs, s, host, "fused")
    assert np.array_equal(nanbits(got), nanbits(expect))


# --- the two forms of the stencil sum ----------------------------------------

@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_one_tap_form_equals_full_sum_on_finite_data(D, T):
    """The reference's CPU form (one tap along a dimension whose column has a
    single nonzero weight) and its device form (every tap) give the same bits
    for finite data, ±0 and subnormals included (src/ghosts.jl:46-56); they
    part only where a NaN or an infinity sits under a zero weight."""
    f = _walls_forest(D)
    par = [(EvenParity,) * D, tuple(OddParity if d == 0 else EvenParity for d in range(D))]
    fs = FieldSet(f, len(par), G=2, centering=vertexcentered(D), parity=par, T=T)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    host = awkward_fill(tuple(fs.work.shape), T, seed=5 + D)
    finite = np.where(np.isfinite(host), host, T(0.25)).astype(T)
    fs.work.copy_(torch.from_numpy(finite))
    skip = oracle.fill_fieldset(fs, s, one_tap=True)
    full = oracle.fill_fieldset(fs, s, one_tap=False)
    assert np.array_equal(skip.view(np.uint8), full.view(np.uint8))
    # a vertex prolongation has columns with one nonzero weight
    singles = [st for g in s.all_groups() for st in g.stencils
               if st.order > 1 and any(np.count_nonzero(st.weights[:, i]) == 1
                                       for i in range(st.weights.shape[1]))]
    assert singles


@pytest.mark.gpu
@pytest.mark.parametrize("one_tap", [0, 1])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_one_tap_option_selects_the_form(cuda_lib, one_tap, T):
    """The fused fill's one_tap option: 1 is the oracle's CPU form, 0 its
    device form, bit for bit on data with NaNs and infinities."""
    from treeamr.ghosts import device_schedule
    D = 3
    f = _walls_forest(D)
    par = [(EvenParity,) * D, tuple(OddParity if d == 1 else EvenParity for d in range(D))]
    fs = FieldSet(f, len(par), G=2, centering=vertexcentered(D), parity=par, T=T)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    host = awkward_fill(tuple(fs.work.shape), T, seed=17)
    fs.work.copy_(torch.from_numpy(host))
    expect = oracle.fill_fieldset(fs, s, one_tap=bool(one_tap))
    other = oracle.fill_fieldset(fs, s, one_tap=not one_tap)
    assert not np.array_equal(nanbits(expect), nanbits(other))  # the data tell them apart
    fs.work = torch.from_numpy(host.copy()).cuda()
    fs.factors = fs.factors.cuda()
    ds = device_schedule(s, 0)
    ds.set_option("one_tap", one_tap)
    try:
        # both multiply paths: the integer pipe's meets the tables' zero
        # products in the full sum and must hand those points to the FP64 pipe
        for im in ((0, 1) if T == np.float64 else (0,)):
            ds.set_option("int_mul", im)
            fs.work.copy_(torch.from_numpy(host))
            fill_ghosts(fs, s)
            torch.cuda.synchronize()
            assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), im
    finally:
        ds.set_option("one_tap", 1)
        ds.set_option("int_mul", 0)


def _predicted_stage_groups(sched):
    """The stage groups restated from ``stage_groups`` (src/schedule.jl:2735-2931):
    after phase 1, a stage joins the group below it when its tag is the next
    one and none of its target boxes or source windows, per block, meets a
    target box of the group, nor its target boxes a source window of it."""
    import collections
    bytag = collections.defaultdict(list)
    for g in sched.groups:
        bytag[g.stage].append(g)

    def boxes(tag):
        out = []
        for g in bytag[tag]:
            w = [(st.targetfirst, st.targetfirst + st.ntarget - 1) for st in g.stencils]
            r = [(int(st.srcstart.min()), int(st.srcstart.max()) + st.order - 1)
                 for st in g.stencils]
            for tb, sb in zip(g.targetblocks, g.sourceblocks):
                out.append((int(tb), w, True))
                out.append((int(sb), r, False))
        return out

    def meets(a, b):
        return all(max(x[0], y[0]) <= min(x[1], y[1]) for x, y in zip(a, b))
    groups, W, R, prev = [], collections.defaultdict(list), collections.defaultdict(list), None
    for tag in sorted(bytag):
        if tag <= 1:
            prev = None
            continue
        acc = boxes(tag)
        joins = prev is not None and tag == prev + 1 and not any(
            any(meets(box, b) for b in W[blk]) or (wr and any(meets(box, b) for b in R[blk]))
            for blk, box, wr in acc)
        if not joins:
            W.clear()
            R.clear()
            groups.append([tag])
        else:
            groups[-1].append(tag)
        for blk, box, wr in acc:
            (W if wr else R)[blk].append(box)
        prev = tag
    merged = [g for g in groups if len(g) > 1]
    return len(merged), sum(len(g) for g in merged)


@pytest.mark.gpu
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_stage_groups_bit_exact(cuda_lib, T):
    """Consecutive prolongation stages that conflict nowhere run as one launch
    pair: the library finds the groups the restated rule predicts, and the
    fill with them equals the fill stage by stage and the oracle, bit for
    bit, on the walls mesh at 4^3 roots, N=16, 3 levels."""
    from treeamr.ghosts import device_schedule
    f, fs, ops = meshes.walls_setup(roots=4, N=16, levels=3, T=T)
    meshes.config_fill(fs, "walls", seed=3)
    sched = GhostSchedule(fs, ops)
    host = fs.work.numpy().copy()
    expect = oracle.fill(sched, host.copy(), fs.nvars, fs.factors_host)
    fs.work = torch.from_numpy(host.copy()).cuda()
    fs.factors = fs.factors.cuda()
    ds = device_schedule(sched, 0)
    assert ds.stage_groups() == _predicted_stage_groups(sched)
    assert ds.stage_groups()[0] >= 1
    for merge, staged in ((1, 0), (0, 0), (1, 1), (0, 1)):
        ds.set_option("merge_stages", merge)
        ds.set_option("staged", staged)
        fs.work.copy_(torch.from_numpy(host))
        fill_ghosts(fs, sched)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), (merge, staged)
