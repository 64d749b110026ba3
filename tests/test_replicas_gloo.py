"""bench.py's multi-GPU mode runs independent replicas (the path does not
shard); its only cross-rank logic is the barrier and the max/sum reductions
of the timings.  Checked here with two gloo ranks on CPU."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    dist = bench.dist_init(world)
    bench.barrier(dist)
    mx = bench.reduce_max(dist, 10.0 + rank)
    sm = bench.reduce_sum(dist, 3.0)
    out[rank] = (mx, sm)
    dist.destroy_process_group()


def test_two_rank_reductions():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    assert out[0] == (11.0, 6.0) and out[1] == (11.0, 6.0)


def test_single_rank_is_identity():
    import bench
    assert bench.reduce_max(None, 4.5) == 4.5 and bench.reduce_sum(None, 2.0) == 2.0
    assert bench.dist_init(1) is None
