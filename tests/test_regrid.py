"""The regrid transfer (``src/regrid.jl:585-756, 942-955``): classification
of new leaves (copy, prolongation from the parent, restriction from the
children), exactness on polynomial data of degree p-1 for created and
coarsened blocks with kept blocks copied bit for bit (the properties of
``test/regrid_tests.jl``), and on the GPU the device transfer equal to the
oracle's replay of the same groups bit for bit."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import exact_values, makepoly, nanbits, nested_forest
from treeamr import FieldSet, Operators
from treeamr.forest import parentkey
from treeamr.regrid import REGRID_TAG, RegridTransfer, regrid, regrid_sources
from treeamr.schedule import COPY, PROLONG, RESTRICT, TransferGroup
from treeamr.storage import vertexcentered


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
                                     np.asarray(g.sourceblocks) + t.nnew, 0, REGRID_TAG)
                       for g in t.groups]

    def all_groups(self):
        return self.groups


def oracle_regrid(t, old_host, new_host, nvars):
    both = np.concatenate([new_host, old_host], axis=0)
    oracle.fill(_Concat(t), both, nvars, np.ones((nvars, 3 ** t.forest.D), t.T))
    return both[:t.nnew]


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
