"""bench.py --gpus N runs N independent replicas of the workload (the path
has no data exchange between GPUs); the host logic around them -- rank
discovery, the barrier and the max over ranks of the step time -- runs here
as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    dist.init_process_group("gloo", init_method="env://")
    try:
        w, r, local = bench.dist_env()
        assert (w, r, local) == (world, rank, rank)
        bench.barrier(w)
        t = bench.max_over_ranks(0.5 + rank, w)        # the slowest replica's step time
        out.put((rank, t))
    finally:
        dist.destroy_process_group()


def test_two_replicas_agree_on_the_slowest_step_time():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = dict(out.get(timeout=10) for _ in range(2))
    assert got == {0: 1.5, 1: 1.5}


def test_single_process_is_its_own_max():
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25
