"""The benchmark's N-GPU mode is replicas (independent batches, no data exchange): each rank takes
its own slice of instances, and the job's time is the slowest rank's.  Two gloo ranks on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(1.5 + rank, world)
    sl = bench.instance_slice(4, rank)
    dist.destroy_process_group()
    q.put((rank, t, sl.start, sl.stop))


def test_two_gloo_ranks_share_nothing_and_report_the_slowest():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [r[1] for r in res] == [2.5, 2.5]
    assert [(r[2], r[3]) for r in res] == [(0, 4), (4, 8)]
