"""The bench's N > 1 path on the CPU: replicas only, timed alone and joined by
the maximum over ranks, with the reference arm printed by rank 0 alone.
Two gloo ranks stand in for two GPUs."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        got = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 15.0, 1: 15.0}


def test_max_over_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_prints_on_rank_zero_only(rank):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
               MASTER_ADDR="127.0.0.1", MASTER_PORT="29555")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--roots", "2", "--levels", "1", "--nvars", "1",
                        "--steps", "1", "--warmup", "1"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    if rank:
        assert lines == []
    else:
        line = json.loads(lines[-1])
        assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
        assert line["cpu_baseline"]["kind"] == "port"


def test_fill_error_states_the_sum_rounding():
    """The error the bench states for a fill: the oracle's sums against a
    double-double (Float64) or float64 (Float32) evaluation of the same
    stencils, a few units in the last place of the terms' magnitude (a
    sequential sum of n terms is within n of them); an error planted in
    one filled ghost shows."""
    import bench
    from _helpers import nested_forest
    from treeamr import FieldSet, GhostSchedule, Operators
    import oracle
    f = nested_forest(3, N=8, periodic=(True,) * 3)
    for T in (np.float64, np.float32):
        fs = FieldSet(f, 2, G=2, T=T)
        s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
        host = np.random.default_rng(1).uniform(-1, 1, size=tuple(fs.work.shape)).astype(T)
        out = oracle.fill(s, host, 2, fs.factors_host)
        e = bench.fill_error(s, out, out, 2, fs.factors_host)
        assert e["points"] > 0
        assert 0 < e["max_ulp_of_terms"] <= 64
        assert e["max_abs"] < (1e-14 if T == np.float64 else 1e-5)
        # a planted error in one filled ghost shows
        g = next(g for g in s.groups if g.kind == "prolong" and g.stage >= 2)
        st = g.stencils
        at = (int(g.targetblocks[0]) - 1, 0) + tuple(s_.targetfirst - 1 for s_ in reversed(st))
        bad = out.copy()
        bad[at] += T(1e-3)

        class One:                                  # that group alone, every transfer
            forest, groups = s.forest, [g]
        e2 = bench.fill_error(One, out, bad, 2, fs.factors_host, per_group=10 ** 6)
        assert e2["max_abs"] > 5e-4


def test_sector_minimum_counts_every_copied_element():
    """The layout's sector minimum the bench states for a stage's unit
    copies equals a brute-force count over every copied element, on a small
    2-D mesh (2 x 2 periodic roots, one refined, N=8, G=2, 3 Float32
    variables): the distinct 32-byte sectors read and written, and those
    written in part."""
    import bench
    from treeamr import FieldSet, Forest, GhostSchedule, Operators
    from treeamr.schedule import PHASE1_TAG
    f = Forest((2, 2), N=8, periodic=(True, True))
    f.refine(f.leaves[0])
    f.balance()
    fs = FieldSet(f, 3, G=2, T=np.float32)
    s = GhostSchedule(fs, Operators(prolongation=4, restriction=4))
    got = bench.sector_minimum(s, fs.nvars, 4, PHASE1_TAG)
    S1, S2 = s.stored[0], s.stored[1]
    vol = S1 * S2
    rd, wr = set(), {}
    for g in s.groups:
        if g.stage != PHASE1_TAG or not g.unit():
            continue
        s1, s2 = g.stencils
        for t, src in zip(g.targetblocks, g.sourceblocks):
            for v in range(fs.nvars):
                for j in range(s2.ntarget):
                    for i in range(s1.ntarget):
                        ta = (((int(t) - 1) * fs.nvars + v) * vol +
                              (s2.targetfirst - 1 + j) * S1 + s1.targetfirst - 1 + i) * 4
                        sa = (((int(src) - 1) * fs.nvars + v) * vol +
                              (int(s2.srcstart[j]) - 1) * S1 + int(s1.srcstart[i]) - 1) * 4
                        wr[ta // 32] = wr.get(ta // 32, 0) + 1
                        rd.add(sa // 32)
    partial = {k for k, n in wr.items() if n < 8}
    assert got["sectors_written_bytes"] == 32 * len(wr)
    assert got["sectors_read_bytes"] == 32 * len(rd)
    assert got["partly_written_bytes"] == 32 * len(partial)
    assert got["minimum_bytes_with_rmw"] == 32 * (len(rd | partial) + len(wr))
