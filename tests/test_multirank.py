"""The benchmark's multi-rank path on CPU with gloo, world size 2: each rank
gets its own clause shard, the step time is the slowest rank's, and the
whole-job throughput counts every rank's checks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    from gpusharesat_gb300 import workloads as W
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        wl = W.make_scale(seed=bench.shard_seed(rank), n_vars=2 ** 10, n_clauses=500)
        my_time = 0.5 + rank  # rank 1 is the slower one
        slowest = bench.max_over_ranks(my_time, world, "cpu")
        out.put((rank, slowest, int(wl.lits[:50].sum()), bench.job_throughput(wl.n_clauses * 1024, world, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_and_slowest_rank_timing():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res[0][1] == res[1][1] == 1.5            # both ranks see the slowest time
    assert res[0][2] != res[1][2]                   # different shards
    assert res[0][3] == res[1][3] == 500 * 1024 * 2 / 1.5
