"""The state vector and its copies to and from the working array
(``src/state.jl:1-160``): lengths and shapes on the CPU; on the GPU,
``scatter``/``gather`` against the oracle's slicing bit for bit on awkward
data, ghosts left untouched, and ``scatter_fill`` equal to the two steps."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import awkward_fill, nanbits, nested_forest
from treeamr import FieldSet, GhostSchedule, fill_ghosts, meshes
from treeamr.state import (gather, ownextents, scatter, scatter_fill, statearray, statelength,
                           statevector)
from treeamr.storage import vertexcentered


def _sets():
    out = []
    for D in (1, 2, 3):
        f = nested_forest(D, N=8)
        out.append(("cell", D, FieldSet(f, 2, G=2)))
        out.append(("vertex", D, FieldSet(f, 3, G=2, centering=vertexcentered(D))))
    return out


@pytest.mark.parametrize("k", range(6))
def test_statelength_and_shape(k):
    kind, D, fs = _sets()[k]
    own = ownextents(fs)
    assert own == tuple(fs.forest.N + (1 if kind == "vertex" else 0) for _ in range(D))
    n = statelength(fs)
    assert n == int(np.prod(own)) * fs.nvars * fs.nblocks()
    u = statevector(fs)
    assert u.shape == (n,) and not u.any()
    assert statearray(u, fs).shape == (fs.nblocks(), fs.nvars) + tuple(reversed(own))
    with pytest.raises(ValueError):
        statearray(u[:-1], fs)


def test_oracle_scatter_gather_round_trip():
    f = nested_forest(3, N=8)
    fs = FieldSet(f, 2, G=3)
    rng = np.random.default_rng(1)
    work = rng.uniform(-1, 1, size=tuple(fs.work.shape))
    u = oracle.gather(fs, work)
    assert u.size == statelength(fs)
    w2 = np.zeros_like(work)
    oracle.scatter(fs, w2, u)
    own = (slice(None), slice(None)) + tuple(slice(fs.G[0], fs.G[0] + 8) for _ in range(3))
    assert np.array_equal(w2[own], work[own])
    assert not w2[:, :, :3].any()


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(6))
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_gpu_scatter_gather_bit_exact(cuda_lib, k, T):
    kind, D, fs0 = _sets()[k]
    fs = FieldSet(fs0.forest, fs0.nvars, G=fs0.G[0], centering=fs0.centering, T=T,
                  device="cuda")
    host = awkward_fill(tuple(fs.work.shape), T, seed=k)
    fs.work.copy_(torch.from_numpy(host))
    u = statevector(fs)
    gather(u, fs)
    expect_u = oracle.gather(fs, host.copy())
    assert np.array_equal(nanbits(u.cpu().numpy()), nanbits(expect_u))
    # scatter a different state into the working array: ghosts untouched
    u2 = torch.from_numpy(awkward_fill((statelength(fs),), T, seed=100 + k)).cuda()
    scatter(fs, u2)
    expect_w = oracle.scatter(fs, host.copy(), u2.cpu().numpy())
    assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect_w))


@pytest.mark.gpu
def test_gpu_scatter_fill_equals_scatter_then_fill(cuda_lib):
    f, fs, ops = meshes.sphere_setup(nvars=2, roots=4, levels=2, device="cuda")
    s = GhostSchedule(fs, ops)
    g = torch.Generator(device="cuda").manual_seed(5)
    u = torch.rand(statelength(fs), dtype=fs.work.dtype, device="cuda", generator=g)
    fs.work.uniform_(-1, 1, generator=g)
    a = fs.work.clone()
    scatter_fill(fs, s, u)
    one = fs.work.clone()
    fs.work.copy_(a)
    scatter(fs, u)
    fill_ghosts(fs, s)
    assert torch.equal(one.view(torch.int64), fs.work.view(torch.int64))
    # and the interiors are the state, the ghosts the oracle's fill of them
    expect = oracle.fill_fieldset(fs, s)
    assert np.array_equal(nanbits(one.cpu().numpy()), nanbits(expect))
    with pytest.raises(ValueError):
        scatter(fs, u[:-1])
