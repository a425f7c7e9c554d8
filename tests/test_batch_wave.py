"""Many forests in one launch, and RK4 for the wave equation over them.

The batch is a new capability (the reference fills one field set per call);
its oracle is the per-member fill, which must agree bit for bit.  The RK4
solver restates the reference's wave test (``test/wave.jl:49-110``) on the
batch; its adjoint is checked by the dot-product test of the whole multi-step
map and against central differences, with checkpointed recomputation."""
import numpy as np
import pytest
import torch

import oracle
from treeamr import GhostSchedule, fill_ghosts, meshes

pytestmark = pytest.mark.gpu


def _small_batch(T=np.float32, n=5, seed=7):
    return meshes.forest_batch_setup(n=n, seed=seed, T=T, max_roots=3, max_levels=2)


def test_batch_fill_equals_member_fills(cuda_lib):
    fss, scheds, batch = _small_batch(np.float32)
    g = torch.Generator(device="cuda").manual_seed(1)
    batch.arena.uniform_(-1, 1, generator=g)
    start = batch.arena.clone()
    # oracle: each member filled alone, on the CPU
    expect = []
    for m, (fs, s) in enumerate(zip(fss, scheds)):
        host = batch.member_view(start, m).cpu().numpy().copy()
        expect.append(oracle.fill(s, host, fs.nvars, fs.factors_host))
    batch.fill()
    torch.cuda.synchronize()
    for m in range(len(fss)):
        got = batch.member_view(batch.arena, m).cpu().numpy()
        assert np.array_equal(got.view(np.uint32), expect[m].view(np.uint32)), m
    # every grouping of the batch's work gives the same bits
    for opt, val in (("path_tiles", 1), ("copy_points", 4), ("tile_items", 48), ("staged", 1),
                     ("copy_share", 2), ("stencil_tile", 80)):
        batch.set_option(opt, val)
        batch.arena.copy_(start)
        batch.fill()
        torch.cuda.synchronize()
        for m in range(len(fss)):
            got = batch.member_view(batch.arena, m).cpu().numpy()
            assert np.array_equal(got.view(np.uint32), expect[m].view(np.uint32)), (opt, m)
    # and each member through its own fill gives the same
    alone = start.clone()
    for m, (fs, s) in enumerate(zip(fss, scheds)):
        fs.work = batch.member_view(alone, m)
        fill_ghosts(fs, s)
    assert torch.equal(alone.view(torch.int32), batch.arena.view(torch.int32))


def test_batch_of_walls_forests_equals_member_fills(cuda_lib):
    """Vertex-centred members with reflecting and outflow faces (the walls
    mesh's layout at two sizes): stages P and 0, mirrored copies with their
    factor column, and copies whose source rows are a table, not a step, all
    through the batch's shared-memory copy segments, bit for bit against each
    member's oracle fill, at one and at four copy points a lane."""
    from treeamr import FieldSet, Operators, meshes as M
    from treeamr.batch import ForestBatch
    from treeamr.storage import vertexcentered
    fss, scheds = [], []
    for roots, levels in ((2, 2), (3, 3)):
        f = M.walls_forest(roots=roots, N=16, levels=levels)
        fs = FieldSet(f, 8, G=2, centering=vertexcentered(3), parity=M.walls_parities(),
                      T=np.float64)
        fss.append(fs)
        scheds.append(GhostSchedule(fs, Operators(prolongation=4, restriction=4)))
    batch = ForestBatch(fss, scheds, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(4)
    batch.arena.uniform_(-1, 1, generator=g)
    start = batch.arena.clone()
    expect = []
    for m, (fs, s) in enumerate(zip(fss, scheds)):
        host = batch.member_view(start, m).cpu().numpy().copy()
        expect.append(oracle.fill(s, host, fs.nvars, fs.factors_host))
    for cp in (1, 4):
        batch.set_option("copy_points", cp)
        batch.arena.copy_(start)
        batch.fill()
        torch.cuda.synchronize()
        for m in range(len(fss)):
            got = batch.member_view(batch.arena, m).cpu().numpy()
            assert np.array_equal(got.view(np.uint64), expect[m].view(np.uint64)), (cp, m)


@pytest.mark.parametrize("T", [np.float32, np.float64])
def test_batch_autotune_keeps_results(cuda_lib, T):
    """The batch's tuner leaves a set of its choices, and the fill with them
    is each member's oracle fill bit for bit."""
    fss, scheds, batch = _small_batch(T, n=4, seed=11)
    g = torch.Generator(device="cuda").manual_seed(2)
    batch.arena.uniform_(-1, 1, generator=g)
    start = batch.arena.clone()
    best = batch.autotune(reps=1, sweeps=1)
    assert set(best) >= {name for name, _ in batch.TUNE} and batch.tuned_ms > 0
    for name, values in batch.TUNE:
        assert best[name] in values
    batch.arena.copy_(start)
    batch.fill()
    torch.cuda.synchronize()
    bits = np.uint32 if T == np.float32 else np.uint64
    for m, (fs, s) in enumerate(zip(fss, scheds)):
        host = batch.member_view(start, m).cpu().numpy().copy()
        expect = oracle.fill(s, host, fs.nvars, fs.factors_host)
        got = batch.member_view(batch.arena, m).cpu().numpy()
        assert np.array_equal(got.view(bits), expect.view(bits)), m


@pytest.mark.parametrize("T", [np.float32, np.float64])
def test_batch_adjoint_equals_member_adjoints(cuda_lib, T):
    """The batched adjoint (one launch per pass and stage for every forest)
    equals each member's own adjoint bit for bit, and its transpose identity
    holds against the oracle's forward fill of each member."""
    from treeamr.adjoint import fill_ghosts_adjoint
    fss, scheds, batch = _small_batch(T, n=5, seed=3)
    g = torch.Generator(device="cuda").manual_seed(6)
    y = torch.rand(batch.arena.shape, dtype=batch.arena.dtype, device="cuda", generator=g)
    got = y.clone()
    batch.fill_adjoint(got)
    alone = y.clone()
    for m, (fs, s) in enumerate(zip(fss, scheds)):
        view = batch.member_view(alone, m)
        fill_ghosts_adjoint(fs, s, view)
    torch.cuda.synchronize()
    bits = torch.int64 if T == np.float64 else torch.int32
    assert torch.equal(got.view(bits), alone.view(bits))
    if T == np.float64:
        rng = np.random.default_rng(2)
        for m, (fs, s) in enumerate(zip(fss, scheds)):
            x = rng.uniform(-1, 1, size=tuple(fs.work.shape))
            ax = oracle.fill(s, x.copy(), fs.nvars, fs.factors_host)
            ym = batch.member_view(y, m).cpu().numpy()
            aty = batch.member_view(got, m).cpu().numpy()
            lhs, rhs = float(np.dot(ax.ravel(), ym.ravel())), float(np.dot(x.ravel(), aty.ravel()))
            assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), abs(rhs))


def test_batch_rejects_a_short_arena(cuda_lib):
    import ctypes as C
    from treeamr import _native
    fss, scheds, batch = _small_batch(np.float32, n=2)
    short = batch.arena[: batch.arena.numel() // 2]
    with pytest.raises(_native.TamError, match="outside the arena"):
        batch.fill(short.contiguous())


def test_wave_rhs_matches_torch(cuda_lib):
    from treeamr.wave import WaveSolver
    fss, scheds, batch = _small_batch(np.float64, n=3)
    solver = WaveSolver(batch)
    g = torch.Generator(device="cuda").manual_seed(2)
    x = torch.rand(batch.arena.shape, dtype=torch.float64, device="cuda", generator=g)
    out = torch.zeros_like(x)
    solver.rhs(x, out)
    for m, fs in enumerate(fss):
        xv = batch.member_view(x, m)
        ov = batch.member_view(out, m)
        G, N = fs.G[0], fs.forest.N
        o = slice(G, G + N)
        u = xv[:, 0]
        lap = (u[:, G + 1:G + N + 1, o, o] + u[:, G - 1:G + N - 1, o, o] +
               u[:, o, G + 1:G + N + 1, o] + u[:, o, G - 1:G + N - 1, o] +
               u[:, o, o, G + 1:G + N + 1] + u[:, o, o, G - 1:G + N - 1] - 6 * u[:, o, o, o])
        h2 = torch.tensor([float(fs.forest.spacing(k.level)) ** 2 for k in fs.forest.leaves],
                          dtype=torch.float64, device="cuda").view(-1, 1, 1, 1)
        assert torch.allclose(ov[:, 1, o, o, o], lap / h2, rtol=1e-12, atol=1e-9)
        assert torch.equal(ov[:, 0, o, o, o], xv[:, 1, o, o, o])


def test_wave_graph_equals_eager(cuda_lib):
    from treeamr.wave import WaveSolver
    fss, scheds, batch = _small_batch(np.float32)
    meshes.wave_initial(batch)
    solver = WaveSolver(batch)
    y0 = batch.arena.clone()
    eager = y0.clone()
    for _ in range(4):
        solver.step(eager)
    y = y0.clone()
    graph = solver.capture(y, steps=2)
    y.copy_(y0)
    graph.replay()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(y.view(torch.int32), eager.view(torch.int32))
    assert torch.isfinite(y).all()


def test_native_rk4_graph_equals_eager(cuda_lib):
    """``tam_graph_capture_rk4``: the library's own graph of RK4 steps
    replays the eager steps bit for bit."""
    from treeamr.wave import WaveSolver
    fss, scheds, batch = _small_batch(np.float32)
    meshes.wave_initial(batch)
    solver = WaveSolver(batch)
    y0 = batch.arena.clone()
    eager = y0.clone()
    for _ in range(4):
        solver.step(eager)
    y = y0.clone()
    graph = solver.native_graph(y, steps=2)
    torch.cuda.synchronize()
    assert torch.equal(y, y0)                       # capture runs nothing
    graph.launch()
    graph.launch()
    torch.cuda.synchronize()
    assert torch.equal(y.view(torch.int32), eager.view(torch.int32))


def test_native_autotune(cuda_lib):
    """``tam_autotune`` leaves the fastest options set, and a fill with them
    is the oracle's bit for bit."""
    from treeamr.autotune import autotune
    from treeamr.ghosts import device_schedule, fill_ghosts
    f, fs, ops = meshes.quadrant_setup()
    s = GhostSchedule(fs, ops)
    fs.work = fs.work.cuda()
    fs.factors = fs.factors.cuda()
    host = np.random.default_rng(9).uniform(size=tuple(fs.work.shape))
    fs.work.copy_(torch.from_numpy(host))
    best = autotune(fs, s)
    assert set(best) == {"tile_items", "threads", "int_mul", "merge_stages", "path_tiles",
                         "staged", "pair_vars", "block_order", "copy_points",
                         "copy_share", "soft_add", "stencil_tile"} and s._tuned_ms > 0
    ds = device_schedule(s, 0)
    assert ds.options()["tile_items"] == best["tile_items"]
    fs.work.copy_(torch.from_numpy(host))
    fill_ghosts(fs, s)
    expect = oracle.fill(s, host.copy(), fs.nvars, fs.factors_host)
    assert np.array_equal(fs.work.cpu().numpy(), expect)


def test_wave_adjoint_dot_product(cuda_lib):
    """<M^n x, y> = <x, (M^T)^n y> for n = 10 RK4 steps, Float64."""
    from treeamr.wave import WaveSolver
    fss, scheds, batch = _small_batch(np.float64)
    solver = WaveSolver(batch)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(batch.arena.shape, dtype=torch.float64, device="cuda", generator=g) - 0.5
    yv = torch.rand(batch.arena.shape, dtype=torch.float64, device="cuda", generator=g) - 0.5
    mx = x.clone()
    for _ in range(10):
        solver.step(mx)
    mty = yv.clone()
    for _ in range(10):
        solver.step_adjoint(mty)
    lhs = torch.dot(mx, yv).item()
    rhs = torch.dot(x, mty).item()
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))


def test_wave_gradient_checkpointed(cuda_lib):
    """The gradient of L = sum_n sum(w * y_n^2) over 10 steps: checkpoints every
    2 steps give the same as every step, and central differences agree."""
    from treeamr.wave import WaveSolver
    fss, scheds, batch = _small_batch(np.float64, n=3)
    solver = WaveSolver(batch)
    g = torch.Generator(device="cuda").manual_seed(4)
    y0 = torch.rand(batch.arena.shape, dtype=torch.float64, device="cuda", generator=g) - 0.5
    w = torch.rand(batch.arena.shape, dtype=torch.float64, device="cuda", generator=g)

    def loss(y):
        y = y.clone()
        total = 0.0
        for _ in range(10):
            solver.step(y)
            total += torch.sum(w * y * y).item()
        return total

    grad2 = solver.gradient(y0, 10, lambda y: 2 * w * y, checkpoint=2)
    grad1 = solver.gradient(y0, 10, lambda y: 2 * w * y, checkpoint=1)
    assert torch.equal(grad1, grad2)
    rng = np.random.default_rng(0)
    # owned points of the first member, where the gradient is not trivially 0
    fs = fss[0]
    G, N = fs.G[0], fs.forest.N
    view = batch.member_view(torch.arange(y0.numel(), device="cuda"), 0)
    idx = view[:, :, G:G + N, G:G + N, G:G + N].reshape(-1)
    # L is exactly quadratic in y0 (linear dynamics), so central differences
    # have no truncation error at any h; h = 1e-3 keeps the cancellation
    # error of a ~1e10 sum below 1e-6 of the gradient
    h = 1e-3
    for k in rng.choice(idx.cpu().numpy(), size=8, replace=False):
        yp = y0.clone()
        ym = y0.clone()
        yp[k] += h
        ym[k] -= h
        fd = (loss(yp) - loss(ym)) / (2 * h)
        gk = grad2[k].item()
        assert abs(fd - gk) <= 1e-5 * max(1.0, abs(gk)), (k, fd, gk)
