"""The bench line's host-side arithmetic, on the CPU: which stages each
kernel's roofline covers, and the layout's sector counts in 32- and 64-byte
units."""
import numpy as np

from treeamr import meshes
from treeamr.schedule import GhostSchedule


def _walls_small():
    f, fs, ops = meshes.walls_setup(roots=2, N=16, levels=2)
    return fs, GhostSchedule(fs, ops)


def test_kernel_rooflines_split_copy_and_stencil_stages():
    import bench
    fs, s = _walls_small()
    tags = sorted({g.stage for g in s.groups})
    kinds = {t: {g.unit() for g in s.groups if g.stage == t} for t in tags}
    stage_ms = {t: [0.5, 0.5] for t in tags}
    stage_bytes = {t: 1_000_000 * (i + 1) for i, t in enumerate(tags)}
    out = bench.kernel_rooflines(s, stage_ms, stage_bytes, peak=1000.0)
    copies = [t for t in tags if kinds[t] == {True}]
    stencils = [t for t in tags if kinds[t] == {False}]
    assert out["fused_copy_kernel"]["stages"] == copies
    assert out["fused_stage_kernel"]["stages"] == stencils
    for name, tt in (("fused_copy_kernel", copies), ("fused_stage_kernel", stencils)):
        k = out[name]
        assert k["ms"] == 0.5 * len(tt)
        assert k["algorithmic_bytes"] == sum(stage_bytes[t] for t in tt)
        assert abs(k["achieved"] - k["algorithmic_bytes"] / (k["ms"] * 1e-3) / 1e9) < 1e-9
        assert abs(k["frac"] - k["achieved"] / 1000.0) < 1e-12
    # a stage with both kinds is in neither
    mixed = {t: [0.5] for t in tags}
    out2 = bench.kernel_rooflines(s, mixed, stage_bytes, peak=1000.0)
    assert set(out2) <= {"fused_copy_kernel", "fused_stage_kernel"}


def test_sector_counts_in_wider_units_are_no_smaller():
    """Counting the same accesses in 64-byte units can only merge sectors into
    fewer, larger units: bytes never fall below the 32-byte count, the
    algorithmic bytes do not change, and every count covers the bytes the
    copies actually move."""
    import bench
    fs, s = _walls_small()
    esize = np.dtype(fs.T).itemsize
    a = bench.sector_minimum(s, fs.nvars, esize, 1, unit=32)
    b = bench.sector_minimum(s, fs.nvars, esize, 1, unit=64)
    assert a["unit_bytes"] == 32 and b["unit_bytes"] == 64
    assert a["algorithmic_bytes"] == b["algorithmic_bytes"]
    for key in ("sectors_read_bytes", "sectors_written_bytes", "minimum_bytes",
                "minimum_bytes_with_rmw"):
        assert b[key] >= a[key], key
    # each written point is in some written sector: the writes cover half the algorithmic bytes
    assert a["sectors_written_bytes"] >= a["algorithmic_bytes"] // 2


def test_clock_sampler_holds_the_load_for_its_samples(tmp_path, monkeypatch):
    """The sampler runs the step until nvidia-smi's first sample is written,
    keeps running it after the timed region until the window is long enough,
    and reads clocks and throttle reasons from what nvidia-smi wrote (a fake
    one here, writing a sample every 50 ms)."""
    import os
    import bench
    fake = tmp_path / "nvidia-smi"
    fake.write_text("#!/bin/sh\nwhile true; do\n"
                    "  echo '0, 2070, 2070, 901.5, 0x4, Not Active, Not Active, Not Active, Active'\n"
                    "  sleep 0.05\ndone\n")
    fake.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    calls = {"fn": 0, "sync": 0}

    def fn():
        calls["fn"] += 1

    def sync():
        calls["sync"] += 1
    with bench.ClockSampler(0) as clk:
        clk.wait_first(fn, sync)
        clk.hold(fn, sync, seconds=0.4)
    out = clk.summary()
    assert out["samples"] >= 3
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
    assert clk.held > 0 and calls["fn"] == clk.before + clk.held
    assert calls["sync"] * 10 == calls["fn"]
    assert "window" in out


def test_clock_sampler_without_nvidia_smi_runs_nothing(tmp_path, monkeypatch):
    import bench
    monkeypatch.setenv("PATH", str(tmp_path))
    ran = []
    with bench.ClockSampler(0) as clk:
        clk.wait_first(lambda: ran.append(1), lambda: None)
        clk.hold(lambda: ran.append(1), lambda: None)
    assert not ran
    assert clk.summary()["reasons"] == ["nvidia-smi unavailable"]


def test_a_failing_side_workload_keeps_the_line():
    """On one GPU a side workload that raises is recorded as its error; the
    others and the headline go on.  Under torchrun it raises."""
    import pytest
    import bench
    workloads = {}

    def bad(x):
        raise MemoryError(f"no room for {x}")
    bench.run_side(workloads, "good", 1, lambda a, b: a + b, 2, 3)
    bench.run_side(workloads, "bad", 1, bad, "the batch")
    assert workloads["good"] == 5
    assert workloads["bad"] == {"error": "MemoryError: no room for the batch"}
    with pytest.raises(MemoryError):
        bench.run_side(workloads, "bad2", 2, bad, "it")
    assert "bad2" not in workloads


def test_dot_test_helper_on_a_matrix():
    """The bench's dot-product test on a dense map and its transpose: a
    residual at rounding, the array's contents kept; a wrong transpose is
    caught."""
    import torch
    import bench
    n = 64
    g = torch.Generator().manual_seed(0)
    A = torch.randn(n, n, dtype=torch.float64, generator=g)
    work = torch.randn(n, dtype=torch.float64, generator=g)
    before = work.clone()

    def fill(t):
        t.copy_(A @ t)

    def adjoint(t):
        t.copy_(A.T @ t)
    out = bench.dot_test(work, fill, adjoint, 3)
    assert out["relative_residual"] < 1e-13 and out["bound"] == 1e-13
    assert torch.equal(work, before)
    assert bench.dot_test(work, fill, fill, 3)["relative_residual"] > 1e-6


def test_written_sector_counts_equal_the_oracles_writes():
    """The layout's written and partly written sectors, counted by the bench
    from the schedule, equal a brute-force count of the points each stage of
    the oracle's fill actually writes (its targets set to NaN after the
    earlier stages, every one a number afterwards), per variable plane as the
    bench counts them, in 32- and 64-byte units, on a small walls mesh."""
    import oracle
    import bench
    from treeamr import FieldSet, Operators
    from treeamr.storage import vertexcentered
    f = meshes.walls_forest(roots=2, N=8, levels=2)
    fs = FieldSet(f, 2, G=2, centering=vertexcentered(3), parity=meshes.walls_parities()[:2],
                  T=np.float64)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    shape, tags = tuple(fs.work.shape), sorted({g.stage for g in s.groups})
    for tag in tags:
        host = np.random.default_rng(0).uniform(1, 2, size=shape)
        prev = [t for t in tags if t < tag]
        if prev:
            host = oracle.fill(s, host, fs.nvars, fs.factors_host, first=prev[0], last=prev[-1])
        for g in s.groups:
            if g.stage == tag:
                sl = tuple(slice(st.targetfirst - 1, st.targetfirst - 1 + st.ntarget)
                           for st in reversed(g.stencils))
                for tb in g.targetblocks:
                    host[(tb - 1, slice(None)) + sl] = np.nan
        before = np.isnan(host)
        out = oracle.fill(s, host, fs.nvars, fs.factors_host, first=tag, last=tag)
        assert not np.isnan(out).any()
        for unit in (32, 64):
            m = bench.sector_minimum(s, fs.nvars, 8, tag, stencils=True, unit=unit)
            written = partial = 0
            for v in range(fs.nvars):
                mask = np.zeros(shape, bool)
                mask[:, v] = before[:, v]
                sec, cnt = np.unique(np.flatnonzero(mask.ravel()) * 8 // unit,
                                     return_counts=True)
                written += sec.size
                partial += int((cnt < unit // 8).sum())
            assert m["sectors_written_bytes"] == written * unit, (tag, unit)
            assert m["partly_written_bytes"] == partial * unit, (tag, unit)
