"""The replicas path of bench.py on the CPU: two gloo ranks, each with its own step time, combine
to the slowest rank's time and a whole-job throughput of world x per-rank units (no GPU, no
collective on any data path)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.rank_info()
        assert (r, w, local) == (rank, world, rank)
        t, tw, ws = bench.combine_ranks(1.0 + rank, 2.0 + 3 * rank, 256, dist)
        out.put((rank, t, tw, ws))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, tw, ws in res:
        assert ws == 2 and t == 2.0 and tw == 5.0


def test_single_process_combine_is_identity():
    import bench
    assert bench.combine_ranks(1.5, 2.5, 256, None) == (1.5, 2.5, 1)

