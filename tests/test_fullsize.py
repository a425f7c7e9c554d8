"""Parity at the sizes the benchmark runs: the sphere mesh (8^3 periodic roots,
N=16, G=3, 3 levels, 4 Float64 variables), the walls mesh (8^3 roots, N=32,
G=2, vertex-centred, reflecting low and outflow high faces, 5 levels, 8
variables) in Float32 and Float64, and the batch of 64 uneven forests.

- Every fill is compared with the oracle's fill of the same data bit for bit
  (the fused kernels take the reference's CPU form of the sum, the plain one
  its device form; on finite data the two have the same bits), and that fill
  with the point-by-point oracle's, which derives every ghost from the
  forest's geometry without the product's schedule.
- Polynomial exactness at full size (``test/ghost_tests.jl:247-281``): data of
  degree 3 in each coordinate come back exact to 1e-10 of their scale at
  order 4 at every ghost, across every level jump of the mesh.  On the
  periodic sphere a ghost past the domain's face holds the polynomial at its
  wrapped position; on the walls mesh a ghost past a reflecting face holds
  the polynomial of the variable's parity at its mirror image (the data are
  chosen with that parity), and one past an outflow face the value at the
  face.
- The adjoint of the sphere with 2 Float64 variables passes the dot-product
  test to 1e-13.

Data are each workload's stated data (``meshes.config_fill``)."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import nanbits
from oracle import pointwise
from _props import NTHREADS, _dot, sphere_polynomial_error, walls_properties
from treeamr import FieldSet, GhostSchedule, Operators, fill_ghosts, meshes
from treeamr.ghosts import device_schedule
from treeamr.storage import vertexcentered

pytestmark = pytest.mark.gpu



@pytest.fixture(scope="module")
def sphere_forest():
    return meshes.sphere_forest(roots=8, N=16, levels=3)


@pytest.fixture(scope="module")
def walls_forest():
    return meshes.walls_forest(roots=8, N=32, levels=5)


def _oracle_expect(fs, sched):
    host = fs.work.cpu().numpy().copy()
    return oracle.fill(sched, host, fs.nvars, fs.factors_host, nthreads=NTHREADS)


def _same(got: torch.Tensor, expect: np.ndarray) -> int:
    """Points whose bits differ (NaN one pattern)."""
    g = got.cpu().numpy()
    return int(np.count_nonzero(nanbits(g) != nanbits(expect)))


def test_sphere_full_bit_exact(cuda_lib, sphere_forest):
    f = sphere_forest
    assert f.nleaves() == 14736
    fs = FieldSet(f, 4, G=3, T=np.float64, device="cuda")
    meshes.config_fill(fs, "sphere", seed=1)
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    start = fs.work.clone()
    expect = _oracle_expect(fs, sched)
    # the point-by-point oracle, which uses no schedule, agrees with the replay
    point = pointwise.fill(fs, start.cpu().numpy(), 4, nthreads=NTHREADS)
    assert np.array_equal(nanbits(point), nanbits(expect))
    del point
    ds = device_schedule(sched, 0)
    for method, staged, pair, share, soft in (("fused", 0, 0, 0, 0), ("fused", 1, 0, 0, 0),
                                              ("fused", 0, 1, 2, 1), ("fused", 0, 0, 2, 1),
                                              ("plain", 0, 0, 0, 0)):
        ds.set_option("staged", staged)
        ds.set_option("pair_vars", pair)
        ds.set_option("copy_share", share)
        ds.set_option("soft_add", soft)
        ds.set_option("int_mul", 1 if (staged or pair or share or soft) else 0)
        fs.work.copy_(start)
        fill_ghosts(fs, sched, method=method)
        torch.cuda.synchronize()
        assert _same(fs.work, expect) == 0, (method, staged, pair, share, soft)


def test_walls_full_bit_exact(cuda_lib, walls_forest):
    f = walls_forest
    assert f.nleaves() == 2374
    for T in (np.float32, np.float64):
        fs = FieldSet(f, 8, G=2, centering=vertexcentered(3), parity=meshes.walls_parities(),
                      T=T, device="cuda")
        meshes.config_fill(fs, "walls", seed=3)
        sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
        start = fs.work.clone()
        expect = _oracle_expect(fs, sched)
        point = pointwise.fill(fs, start.cpu().numpy(), 4, nthreads=NTHREADS)
        assert np.array_equal(nanbits(point), nanbits(expect)), np.dtype(T).name
        del point
        ds = device_schedule(sched, 0)
        for method, staged, pair, share, soft in (("fused", 0, 0, 0, 0), ("fused", 1, 0, 0, 0),
                                                  ("fused", 0, 1, 2, 1), ("fused", 0, 0, 2, 1),
                                                  ("plain", 0, 0, 0, 0)):
            ds.set_option("staged", staged)
            ds.set_option("pair_vars", pair)
            ds.set_option("copy_share", share)
            ds.set_option("soft_add", soft)
            ds.set_option("int_mul", 1 if (staged or pair or share or soft) else 0)
            fs.work.copy_(start)
            fill_ghosts(fs, sched, method=method)
            torch.cuda.synchronize()
            assert _same(fs.work, expect) == 0, (np.dtype(T).name, method, staged, pair, share,
                                                 soft)
        del fs, start, expect, ds
        torch.cuda.empty_cache()


def test_batch64_full_bit_exact(cuda_lib):
    fss, scheds, batch = meshes.forest_batch_setup(device="cuda")
    assert len(fss) == 64
    g = torch.Generator(device="cuda").manual_seed(9)
    batch.arena.uniform_(-1.0, 1.0, generator=g)
    before = batch.arena.cpu()
    batch.fill()
    torch.cuda.synchronize()
    after = batch.arena
    for m, (fs, s) in enumerate(zip(fss, scheds)):
        host = batch.member_view(before, m).numpy().copy()
        point = pointwise.fill(fs, host, 4, nthreads=NTHREADS)
        expect = oracle.fill(s, host, fs.nvars, fs.factors_host, nthreads=NTHREADS)
        assert np.array_equal(nanbits(point), nanbits(expect)), m
        assert _same(batch.member_view(after, m), expect) == 0, m


def test_sphere_full_polynomial_exact(cuda_lib, sphere_forest):
    fs = FieldSet(sphere_forest, 2, G=3, T=np.float64, device="cuda")
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    worst, scale = sphere_polynomial_error(fs, sched, "gpu")
    assert worst <= 1e-10 * scale, (worst, scale)


def test_walls_full_polynomial_and_outflow(cuda_lib, walls_forest):
    fs = FieldSet(walls_forest, 8, G=2, centering=vertexcentered(3),
                  parity=meshes.walls_parities(), T=np.float64, device="cuda")
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    worst, scale, bad = walls_properties(fs, sched, "gpu", margin=1.0 / 64)
    assert worst <= 1e-10 * scale, (worst, scale)
    assert bad == 0


def test_sphere_full_adjoint_dot(cuda_lib, sphere_forest):
    """The adjoint's workload: the sphere mesh with 2 Float64 variables,
    <A x, y> = <x, A^T y> to 1e-13 with seeded uniform x and y."""
    from treeamr.adjoint import fill_ghosts_adjoint
    f = sphere_forest
    fs = FieldSet(f, 2, G=3, T=np.float64, device="cuda")
    sched = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    g = torch.Generator(device="cuda").manual_seed(21)
    x = torch.empty_like(fs.work).uniform_(-1.0, 1.0, generator=g)
    y = torch.empty_like(fs.work).uniform_(-1.0, 1.0, generator=g)
    fs.work.copy_(x)
    fill_ghosts(fs, sched)
    aty = y.clone()
    fill_ghosts_adjoint(fs, sched, aty)
    torch.cuda.synchronize()
    lhs, rhs = _dot(fs.work, y), _dot(x, aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs)), (lhs, rhs)
