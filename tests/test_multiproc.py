"""The N>1 bench path on CPU: two gloo ranks, one replica volume each (different seeds), step
times combined by max over ranks, whole-job rate = all ranks' voxels / the slowest rank."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [0.5, 2.0][rank]  # rank 1 is the slow one
        worst, rate = bench.whole_job_rate(local, 1000, world, torch.device("cpu"))
        dist.barrier()
        q.put((rank, bench.replica_seed(rank), worst, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_by_max():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [2, 3]  # distinct replica volumes
    for _, _, worst, rate in got:
        assert worst == 2.0
        assert rate == pytest.approx(2 * 1000 / 2.0 / 1e9)
