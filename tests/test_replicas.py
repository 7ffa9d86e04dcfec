"""The multi-replica logic of bench.py on CPU: two gloo ranks, each timing its
own replica; every rank must see the slowest rank's time, and the whole-job
throughput counts both replicas' work over that time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_env() == (rank, world, rank)
    mine = [1.0 + rank, 10.0 - rank, 0.5 * (rank + 1)]
    got = bench.reduce_max_over_ranks(dist, mine)
    out.put((rank, got, bench.job_throughput(world, 1000, got[0])))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_max():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, got, thr in results:
        assert got == [2.0, 10.0, 1.0]
        assert thr == pytest.approx(2 * 1000 / 2e-3)


def test_single_process_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max_over_ranks(None, [3, 4.5]) == [3.0, 4.5]
    assert bench.job_throughput(1, 2_073_600, 1.0) == pytest.approx(2.0736e9)
