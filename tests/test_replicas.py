"""The multi-GPU form of this path is N independent replicas (one process per GPU, no data
exchange): bench.py takes the slowest rank's time and counts every rank's work.  Checked
here with world_size 2 over gloo on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    ws, r, local = bench.dist_env()
    t = bench.max_over_ranks(1.5 + rank)          # rank 1 is the slower replica
    v = bench.replica_value(10, t, ws)
    dist.barrier()
    q.put((r, ws, local, t, v))
    dist.destroy_process_group()


def test_replicas_report_the_slowest_rank_and_all_work():
    world = 2
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, ws, local, t, v) in enumerate(res):
        assert (rank, ws, local) == (r, world, r)
        assert t == 2.5                             # max over ranks
        assert v == pytest.approx(10 * world / 2.5)  # all ranks' units over the slowest time


def test_single_process_is_its_own_job():
    import bench
    assert bench.max_over_ranks(3.0) == 3.0
    assert bench.replica_value(5, 2.0, 1) == 2.5
