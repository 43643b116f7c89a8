"""The multi-GPU form of the bench is N independent replicas (one rank per
GPU, no data-path collective): whole-job frames/s = frames of all ranks over
the slowest rank's time.  Checked here with two gloo ranks on the host."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, secs, steps, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        q.put((rank, bench.replica_rate(secs[rank], steps, world, "cpu")))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("secs", [(1.0, 2.0), (3.5, 0.5)])
def test_two_replicas_report_the_slowest_rank(secs):
    world, steps = 2, 10
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, secs, steps, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(world))
    slow = max(secs)
    for r in range(world):
        rate, sec = got[r]
        assert sec == pytest.approx(slow)
        assert rate == pytest.approx(steps * world / slow)


def test_one_replica_needs_no_process_group():
    import bench
    assert bench.replica_rate(2.0, 20, 1) == (10.0, 2.0)
