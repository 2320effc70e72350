"""Multi-GPU host logic of bench.py on the CPU: world size 2 over gloo.

The solve does not shard (independent problems per replica, no collective on the data
path); the only cross-rank steps are the barriers around the timed region and the
maximum of the per-rank times. These run here as two gloo processes on 127.0.0.1.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_env()
        dist.barrier()
        t = bench.max_over_ranks(10.0 + 5.0 * rank, torch.device("cpu"))
        q.put((r, ws, local, t, bench.replica_seed(0, r)))
    finally:
        dist.destroy_process_group()


def test_two_rank_timing_reduction():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(world))
    assert [r[0] for r in res] == [0, 1] and all(r[1] == world for r in res)
    assert all(r[3] == 15.0 for r in res)          # the job time is the slowest rank's
    assert len({r[4] for r in res}) == world        # each replica has its own problem
