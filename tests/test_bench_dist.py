"""Multi-rank host logic of bench.py on CPU (gloo, world size 2): every rank reconstructs its
own disjoint clouds (the job's shards), the job's time is the slowest rank's (all_reduce MAX),
and the whole-job rates count the clouds of all ranks.  The reference arm runs on rank 0
only; other ranks exit without work."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r was (r + 1) times slower than rank 0 on every leg
        totals = [10.0 * (rank + 1), 20.0 * (rank + 1), 30.0 * (rank + 1), 40.0 * (rank + 1)]

        def all_max(vals):
            t = torch.tensor(vals, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return t.tolist()

        rates = bench.job_rates(world, 5, 8, totals, all_max)
        seeds = bench.rank_clouds(rank, 8)
        gathered = [None] * world
        dist.all_gather_object(gathered, seeds)
        q.put((rank, rates, gathered))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_rank_and_shard_the_clouds():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    try:
        out = sorted((q.get(timeout=180) for _ in range(2)), key=lambda x: x[0])
    finally:
        for p in ps:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [p.exitcode for p in ps] == [0, 0]
    for rank, rates, gathered in out:
        assert rates["max_totals_ms"] == [20.0, 40.0, 60.0, 80.0]
        assert rates["plain"] == pytest.approx(2 * 5 / 0.020)
        assert rates["plain_e2e"] == pytest.approx(2 * 5 / 0.040)
        assert rates["served"] == pytest.approx(2 * 8 * 5 / 0.060)
        assert rates["served_e2e"] == pytest.approx(2 * 8 * 5 / 0.080)
        s0, s1 = gathered
        assert len(set(s0)) == 8 and not set(s0) & set(s1)
    # both ranks report the same job figures
    assert out[0][1] == out[1][1]


def test_single_rank_rates_and_clouds():
    r = bench.job_rates(1, 10, 4, [100.0, 200.0, 50.0, 80.0])
    assert r["plain"] == pytest.approx(100.0)
    assert r["served"] == pytest.approx(4 * 10 / 0.05)
    assert bench.rank_clouds(0, 4) == [0, 1, 2, 3]


def test_reference_arm_runs_on_rank_zero_only(capsys):
    class Args:
        workload = "torus_ellipsoid200k"
        steps = 1
        warmup = 0
    assert bench.run_reference(Args(), 1, 2) is None
    assert capsys.readouterr().out == ""
