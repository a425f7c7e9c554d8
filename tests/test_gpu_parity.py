"""Parity of the CUDA engine with the oracle, through the C ABI.

Every fill is compared with the oracle's fill of the same data bit for bit:
the kernels evaluate the reference's expression in the reference's order
with no fused multiply-add, so there is no tolerance to state (a bound of
2 ulp in Float64 and 4 in Float32 for restriction and prolongation would
be met with 0).  NaN is compared as one pattern
(``test/helpers/ghost.jl:191-219``)."""
import numpy as np
import pytest
import torch

import oracle
from _helpers import (awkward_fill, exact_values, ghost_mask, makepoly, nanbits, nested_forest)
from treeamr import (EvenParity, FieldSet, Forest, GhostSchedule, OddParity, Operators,
                     fill_ghosts)
from treeamr import meshes

pytestmark = pytest.mark.gpu

METHODS = ["fused", "plain"]


def _gpu_vs_oracle(fs_host, ops, method, *, host=None, boundary=False, exact=None):
    """Fill a copy of ``fs_host``'s data on the GPU and with the oracle."""
    s = GhostSchedule(fs_host, ops)
    if host is None:
        host = fs_host.work.cpu().numpy().copy()
    fs_host.work = torch.from_numpy(host.copy())
    fs_host.factors = fs_host.factors.cpu()
    bv = None
    if boundary:
        def bv(h, fs_, regions):
            for r in regions:
                sl = tuple(slice(a - 1, z) for a, z in reversed(r.region))
                h[(r.block, slice(None)) + sl] = exact[(r.block, slice(None)) + sl]
    # the fused kernels take the reference's CPU form of the sum, the plain
    # kernel its device form (src/ghosts.jl:28-56)
    expect = oracle.fill_fieldset(fs_host, s, boundary_values=bv, one_tap=method == "fused")
    fs = fs_host
    fs.work = torch.from_numpy(host.copy()).cuda()
    fs.factors = fs.factors.cuda()

    hook = None
    if boundary:
        def hook(fsd, regions):
            h = fsd.work.cpu().numpy()
            bv(h, fsd, regions)
            fsd.work.copy_(torch.from_numpy(h).cuda())
    fill_ghosts(fs, s, boundary=hook, method=method)
    torch.cuda.synchronize()
    got = fs.work.cpu().numpy()
    return got, expect


@pytest.mark.parametrize("method", METHODS)
def test_quadrant_bit_exact(cuda_lib, method):
    f, fs, ops = meshes.quadrant_setup()
    meshes.random_fill(fs, seed=11)
    got, expect = _gpu_vs_oracle(fs, ops, method)
    assert np.array_equal(nanbits(got), nanbits(expect))


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
@pytest.mark.parametrize("p,G,N", [(2, 1, 4), (4, 2, 8), (6, 3, 8)])
def test_nested_bit_exact(cuda_lib, method, D, T, p, G, N):
    if D == 3 and p == 6:
        pytest.skip("order 6 runs in 1-D and 2-D, as the reference's test does")
    f = nested_forest(D, N=N)
    fs = FieldSet(f, 3, G=G, T=T)
    exact = exact_values(fs, makepoly(D, 2))
    rng = np.random.default_rng(D * 100 + p)
    host = exact.copy()
    host[:, :, ghost_mask(fs)] = rng.uniform(-9, 9, size=host[:, :, ghost_mask(fs)].shape)
    got, expect = _gpu_vs_oracle(fs, Operators(prolongation=p, restriction=p), method,
                                 host=host, boundary=True, exact=exact)
    assert np.array_equal(nanbits(got), nanbits(expect))


@pytest.mark.parametrize("method", METHODS)
def test_sphere_order6_bit_exact(cuda_lib, method):
    """The sphere mesh's order-6 variant, PV(6,6) in 3-D (216 taps a
    prolonged point), on a small case of the same construction: 2^3
    periodic roots, N=16, G=3, 2 levels, 4 Float64 variables."""
    f, fs, ops = meshes.sphere_setup(roots=2, levels=2, p=6)
    meshes.random_fill(fs, seed=13)
    got, expect = _gpu_vs_oracle(fs, ops, method)
    assert np.array_equal(nanbits(got), nanbits(expect))


def test_sphere_order6_integer_pipe_multiply_bit_exact(cuda_lib):
    """The order-6 products have up to 53 significant bits: with the
    multiplies on the integer pipe (mul_full) the fill is the oracle's bit for
    bit, on seeded data and on awkward data (zeros, subnormals, infinities and
    NaNs, which hand their points back to the FP64 pipe)."""
    from treeamr.ghosts import device_schedule
    for fill in ("random", "awkward"):
        f, fs, ops = meshes.sphere_setup(roots=2, levels=2, p=6)
        if fill == "random":
            meshes.random_fill(fs, seed=14)
            host = fs.work.numpy().copy()
        else:
            host = awkward_fill(tuple(fs.work.shape), np.float64, seed=15)
            fs.work = torch.from_numpy(host.copy())
        s = GhostSchedule(fs, ops)
        expect = oracle.fill_fieldset(fs, s, one_tap=True)
        fs.work = torch.from_numpy(host).cuda()
        fs.factors = fs.factors.cuda()
        ds = device_schedule(s, 0)
        ds.set_option("int_mul", 1)
        fill_ghosts(fs, s)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), fill


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_awkward_data_bit_exact(cuda_lib, method, D, T):
    """+-0, NaN, +-Inf and subnormals through copies, restrictions and
    prolongations (``test/ghost_tests.jl:507-560``)."""
    N = 6 if D == 3 else 8
    f = Forest((2,) * D, N=N, periodic=(True,) * D)
    f.refine(f.leaves[0])
    f.balance()
    fs = FieldSet(f, 3, G=2, T=T)
    host = awkward_fill(tuple(fs.work.shape), T, seed=D)
    got, expect = _gpu_vs_oracle(fs, Operators(prolongation=4, restriction=4), method, host=host)
    assert np.array_equal(nanbits(got), nanbits(expect))


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("D", [2, 3])
def test_reflecting_outflow_bit_exact(cuda_lib, method, D):
    refl = tuple((True, False) for _ in range(D))
    outf = tuple((False, True) for _ in range(D))
    f = Forest((2,) * D, N=8, reflecting=refl, outflow=outf, extents=[(0.0, 2.0)] * D)
    f.refine(f.leaves[0])
    f.balance()
    parity = [(EvenParity,) * D] * 2 + [tuple(OddParity if e == d else EvenParity
                                              for e in range(D)) for d in range(D)]
    fs = FieldSet(f, len(parity), G=2, parity=parity)
    host = awkward_fill(tuple(fs.work.shape), np.float64, seed=5)
    got, expect = _gpu_vs_oracle(fs, Operators(prolongation=4, restriction=4), method, host=host)
    assert np.array_equal(nanbits(got), nanbits(expect))


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_sphere_small_bit_exact(cuda_lib, T):
    """The sphere mesh at a reduced root count (4^3 roots, 2 levels)."""
    f, fs, ops = meshes.sphere_setup(nvars=2, T=T, roots=4, levels=2)
    meshes.random_fill(fs, seed=3)
    for method in METHODS:
        got, expect = _gpu_vs_oracle(fs, ops, method)
        assert np.array_equal(nanbits(got), nanbits(expect))


def test_fused_equals_plain_and_is_idempotent(cuda_lib):
    f, fs, ops = meshes.sphere_setup(nvars=2, roots=4, levels=2, device="cuda")
    meshes.random_fill(fs, seed=9)
    s = GhostSchedule(fs, ops)
    a = fs.work.clone()
    fill_ghosts(fs, s, method="plain")
    plain = fs.work.clone()
    fs.work.copy_(a)
    fill_ghosts(fs, s, method="fused")
    fused = fs.work.clone()
    assert torch.equal(plain.view(torch.int64), fused.view(torch.int64))
    fill_ghosts(fs, s, method="fused")
    assert torch.equal(fs.work.view(torch.int64), fused.view(torch.int64))


def test_interiors_untouched_on_gpu(cuda_lib):
    f, fs, ops = meshes.sphere_setup(nvars=1, roots=4, levels=2, device="cuda")
    meshes.random_fill(fs, seed=2)
    before = fs.work.clone()
    fill_ghosts(fs, GhostSchedule(fs, ops))
    inter = (slice(None), slice(None)) + fs.interior()
    assert torch.equal(fs.work[inter], before[inter])
    assert not torch.equal(fs.work, before)


def test_layout_mismatch_refused(cuda_lib):
    f = Forest((2, 2), N=8, periodic=(True, True))
    fs1 = FieldSet(f, 1, G=2, device="cuda")
    fs2 = FieldSet(f, 1, G=3, device="cuda")
    s = GhostSchedule(fs1, Operators(prolongation=4, restriction=4))
    with pytest.raises(ValueError, match="G="):
        fill_ghosts(fs2, s)


def test_bad_descriptor_rejected_before_launch(cuda_lib):
    """A stencil window outside the stored extent is refused at upload."""
    import ctypes as C
    from treeamr import _native
    f = Forest((2, 2), N=8, periodic=(True, True))
    fs = FieldSet(f, 1, G=2)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    d = _native.Descriptor(s)
    d.srcstart[0] = 100
    ctx = _native.context(0)
    h = C.c_void_p()
    rc = cuda_lib.tam_schedule_upload(ctx, d.ref(), C.byref(h))
    assert rc == -1
    assert "outside" in _native.last_error(ctx)
    d.srcstart[0] = 1
    d.targetblocks[0] = 99
    assert cuda_lib.tam_schedule_upload(ctx, d.ref(), C.byref(h)) == -1


def test_integer_pipe_multiply_matches_hardware(cuda_lib):
    """The Float64 multiply the fused fill runs on the integer pipe equals the
    hardware multiply in every bit, over 2^26 pairs of every data pattern."""
    import ctypes as C
    from treeamr import _native
    ctx = _native.context(0)
    bad = C.c_int64(-1)
    for seed in (1, 2, 3):
        _native.check(cuda_lib.tam_selftest(ctx, 1, 1 << 26, seed, C.byref(bad)), ctx,
                      "tam_selftest")
        assert bad.value == 0


def test_integer_pipe_wide_multiply_matches_hardware(cuda_lib):
    """The Float64 multiply of weights of any width (order 6) on the integer
    pipe equals the hardware multiply in every bit wherever it does not hand
    the pair back, over 3 x 2^26 pairs, products near the normal range's
    edges among them."""
    import ctypes as C
    from treeamr import _native
    ctx = _native.context(0)
    bad = C.c_int64(-1)
    for seed in (1, 2, 3):
        _native.check(cuda_lib.tam_selftest(ctx, 3, 1 << 26, seed, C.byref(bad)), ctx,
                      "tam_selftest")
        assert bad.value == 0


def test_integer_pipe_add_matches_hardware(cuda_lib):
    """The Float64 add a stencil row's last tap may take on the integer pipe
    equals the hardware add in every bit wherever it does not hand the pair
    back, over 3 x 2^26 pairs weighted to its hard cases (equal and adjacent
    exponents, cancellations, the edges of the normal range)."""
    import ctypes as C
    from treeamr import _native
    ctx = _native.context(0)
    bad = C.c_int64(-1)
    for seed in (1, 2, 3):
        _native.check(cuda_lib.tam_selftest(ctx, 2, 1 << 26, seed, C.byref(bad)), ctx,
                      "tam_selftest")
        assert bad.value == 0


def test_launch_options_change_no_bit(cuda_lib):
    """Every launch option of the fused fill gives the same bits."""
    from treeamr.ghosts import device_schedule
    f, fs, ops = meshes.sphere_setup(nvars=3, roots=4, levels=2)
    meshes.random_fill(fs, seed=21)
    host = fs.work.numpy().copy()
    s = GhostSchedule(fs, ops)
    expect = oracle.fill_fieldset(fs, s)
    fs.work = torch.from_numpy(host).cuda()
    fs.factors = fs.factors.cuda()
    ds = device_schedule(s, 0)
    for ti, th, im, cp, bo, pt, ms, sg, pv, cs, sa, st in (
            (16, 64, 0, 1, 3, 0, 1, 1, 1, 1, 1, 0),
            (37, 96, 1, 2, 1, 1, 0, 1, 0, 0, 1, 48),
            (512, 512, 1, 4, 0, 1, 1, 0, 1, 2, 1, 16),
            (64, 128, 1, 1, 2, 1, 1, 0, 0, 2, 1, 128),
            (4096, 128, 0, 2, 1, 0, 0, 1, 1, 4, 0, 0)):
        opts = {"tile_items": ti, "threads": th, "int_mul": im, "one_tap": 1,
                "copy_points": cp, "block_order": bo, "path_tiles": pt, "merge_stages": ms,
                "staged": sg, "pair_vars": pv, "copy_share": cs, "soft_add": sa,
                "stencil_tile": st}
        for k, v in opts.items():
            ds.set_option(k, v)
        assert ds.options() == opts
        fs.work.copy_(torch.from_numpy(host))
        fill_ghosts(fs, s)
        torch.cuda.synchronize()
        assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect)), opts
    with pytest.raises(Exception):
        ds.set_option("threads", 100)
    with pytest.raises(Exception):
        ds.set_option("copy_points", 3)
    with pytest.raises(Exception):
        ds.set_option("copy_share", -1)


def test_autotune_keeps_results(cuda_lib):
    from treeamr.autotune import autotune
    f, fs, ops = meshes.sphere_setup(nvars=2, roots=4, levels=2)
    meshes.random_fill(fs, seed=5)
    host = fs.work.numpy().copy()
    s = GhostSchedule(fs, ops)
    expect = oracle.fill_fieldset(fs, s)
    fs.work = torch.from_numpy(host).cuda()
    fs.factors = fs.factors.cuda()
    best = autotune(fs, s, reps=1, tile_items=(64, 256), threads=(128, 256))
    assert set(best) == {"tile_items", "threads", "int_mul"}
    fs.work.copy_(torch.from_numpy(host))
    fill_ghosts(fs, s)
    torch.cuda.synchronize()
    assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(expect))


def test_host_pipeline_equals_device_fill(cuda_lib):
    """tam_fill_host through HostPipeline: states held in page-locked host
    memory, filled three at a time on three streams, equal the device fill
    bit for bit; in place and into a separate output."""
    from treeamr.host import HostPipeline
    f, fs, ops = meshes.sphere_setup(nvars=2, roots=4, levels=2)
    s = GhostSchedule(fs, ops)
    fs.work = fs.work.cuda()
    fs.factors = fs.factors.cuda()
    states = []
    for k in range(5):
        g = torch.Generator(device="cuda").manual_seed(40 + k)
        states.append(torch.rand(fs.work.shape, dtype=fs.work.dtype, device="cuda", generator=g))
    expect = []
    for x in states:
        fs.work.copy_(x)
        fill_ghosts(fs, s)
        expect.append(fs.work.clone())
    pipe = HostPipeline(fs, s, depth=3)
    ins = [x.cpu().pin_memory() for x in states]
    outs = [torch.empty_like(h).pin_memory() for h in ins]
    for k in range(5):
        if k % 2:
            pipe.submit(ins[k])                  # in place
        else:
            pipe.submit(ins[k], outs[k])
    pipe.synchronize()
    for k in range(5):
        got = ins[k] if k % 2 else outs[k]
        assert torch.equal(got.view(torch.int64), expect[k].cpu().view(torch.int64))
    with pytest.raises(ValueError):
        pipe.submit(ins[0][:1])


def test_host_pipeline_own_uploads_equal_device_fill(cuda_lib):
    """tam_fill_host_own: only the own points go up (read by a kernel from
    the page-locked host buffer); the filled array that comes back equals
    the device fill bit for bit, whatever the host buffer's ghosts held.
    A schedule with hook regions, and pageable host memory, are refused."""
    from treeamr.host import HostPipeline
    f, fs, ops = meshes.sphere_setup(nvars=2, roots=4, levels=2)
    s = GhostSchedule(fs, ops)
    assert not s.boundaries
    fs.work = fs.work.cuda()
    fs.factors = fs.factors.cuda()
    states, expect = [], []
    for k in range(4):
        g = torch.Generator(device="cuda").manual_seed(60 + k)
        x = torch.rand(fs.work.shape, dtype=fs.work.dtype, device="cuda", generator=g)
        states.append(x)
        fs.work.copy_(x)
        fill_ghosts(fs, s)
        expect.append(fs.work.clone())
    pipe = HostPipeline(fs, s, depth=3, own=True)
    ins = []
    for x in states:
        h = x.cpu()
        h[:, :, torch.from_numpy(ghost_mask(fs))] = float("nan")     # never uploaded
        ins.append(h.pin_memory())
    outs = [torch.empty_like(h).pin_memory() for h in ins]
    for k in range(4):
        pipe.submit(ins[k], outs[k] if k % 2 else None)
    pipe.synchronize()
    for k in range(4):
        got = outs[k] if k % 2 else ins[k]
        assert torch.equal(got.view(torch.int64), expect[k].cpu().view(torch.int64))
    assert pipe.own_bytes() * 2 < ins[0].numel() * ins[0].element_size()
    with pytest.raises(Exception, match="page-locked"):
        pipe.submit(states[0].cpu())
    fw = nested_forest(2, N=8)
    fw_s = FieldSet(fw, 1, G=2, device="cuda")
    with pytest.raises(ValueError, match="hook"):
        HostPipeline(fw_s, GhostSchedule(fw_s, Operators(prolongation=4, restriction=4)),
                     own=True)


# --- edge cases: no transfers, a block its own neighbour, ragged variable chunks ------------

@pytest.mark.parametrize("method", METHODS)
def test_a_schedule_without_transfers_changes_nothing(cuda_lib, method):
    """A lone root with no periodic dimension has no neighbour: its schedule
    has no group, and the fill (and its adjoint) leaves every bit as it was."""
    from treeamr.adjoint import fill_ghosts_adjoint
    f = Forest((1, 1, 1), N=8)
    fs = FieldSet(f, 2, G=2)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    assert not [g for g in s.groups if g.ntransfers()]
    host = awkward_fill(tuple(fs.work.shape), np.float64, seed=4)
    fs.work = torch.from_numpy(host.copy()).cuda()
    fill_ghosts(fs, s, method=method)
    fill_ghosts_adjoint(fs, s)
    torch.cuda.synchronize()
    assert np.array_equal(nanbits(fs.work.cpu().numpy()), nanbits(host))


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_a_lone_periodic_root_is_its_own_neighbour(cuda_lib, method, T):
    """One root per periodic dimension (``test/ghost_tests.jl:455-466``): the
    block is its own neighbour in all 26 directions, and every ghost is the
    own point a period away, bit for bit (the periodic tiling), as the
    oracle's fill."""
    N, G = 8, 2
    f = Forest((1, 1, 1), N=N, periodic=(True, True, True))
    fs = FieldSet(f, 3, G=G, T=T)
    host = np.random.default_rng(6).uniform(-1, 1, size=tuple(fs.work.shape)).astype(T)
    got, expect = _gpu_vs_oracle(fs, Operators(prolongation=4, restriction=4), method, host=host)
    assert np.array_equal(nanbits(got), nanbits(expect))
    own = host[0][:, G:G + N, G:G + N, G:G + N]
    idx = (np.arange(N + 2 * G) - G) % N
    tiled = own[:, idx][:, :, idx][:, :, :, idx]
    assert np.array_equal(got[0].view(np.uint64 if T == np.float64 else np.uint32),
                          tiled.view(np.uint64 if T == np.float64 else np.uint32))


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("T", [np.float64, np.float32])
@pytest.mark.parametrize("nvars", [1, 5, 11])
def test_ragged_variable_counts_bit_exact(cuda_lib, method, T, nvars):
    """Variable counts that leave ragged tails in the kernels' chunks (8
    variables a copy chunk, 4 or 1 a stencil chunk): copies, restrictions
    and prolongations in 3-D, bit for bit as the oracle."""
    f = nested_forest(3, N=8, periodic=(True,) * 3)
    fs = FieldSet(f, nvars, G=2, T=T)
    host = np.random.default_rng(nvars).uniform(-1, 1, size=tuple(fs.work.shape)).astype(T)
    got, expect = _gpu_vs_oracle(fs, Operators(prolongation=4, restriction=4), method, host=host)
    assert np.array_equal(nanbits(got), nanbits(expect))
