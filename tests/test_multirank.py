"""The N > 1 path of bench.py as world-size-2 gloo ranks on the CPU: replicas only (each rank
its own seeded image), no data-path collective, the timing reduced as the max over ranks, the
whole-job throughput counting every rank's pixels, one JSON line from rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(td, 1.0 + 2.0 * rank, device="cpu")     # rank 1 is slower
        seed = bench.replica_seed(rank)
        seeds = [None] * world
        td.all_gather_object(seeds, seed)
        q.put((rank, ms, seeds))
    finally:
        td.destroy_process_group()


def test_two_rank_replicas_reduce_max_time():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [3.0, 3.0]            # both ranks see the slowest rank's time
    assert got[0][2] == got[1][2] and len(set(got[0][2])) == 2   # distinct replica images


def test_aggregate_counts_every_rank():
    sys.path.insert(0, ROOT)
    import bench
    one = bench.aggregate_mpix(1, 4096 * 4096, 47e-6)
    assert abs(bench.aggregate_mpix(2, 4096 * 4096, 47e-6) - 2 * one) < 1e-6


def test_reference_arm_prints_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup = 1, 0
    bench.run_reference(Args(), rank=1, world=2)
    assert capsys.readouterr().out == ""
