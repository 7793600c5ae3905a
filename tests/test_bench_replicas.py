"""bench.py's N > 1 path (independent replicas, max-over-ranks timing) on
world-size-2 gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path[:0] = [REPO, os.path.join(REPO, "offshore-sph_gb300")]
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        # rank r took 1 + r seconds for 10 steps of 1000 fluid particles
        el, value = bench.replica_value(1.0 + rank, 1000, 10, world, "cpu")
        q.put((rank, el, value))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, el, value in got:
        assert el == pytest.approx(2.0)
        assert value == pytest.approx(2 * 1000 * 10 / 2.0)


def test_single_rank_needs_no_process_group():
    sys.path[:0] = [REPO, os.path.join(REPO, "offshore-sph_gb300")]
    import bench
    el, value = bench.replica_value(0.5, 1000, 10, 1, "cpu")
    assert el == 0.5 and value == pytest.approx(20000.0)
