"""The multi-GPU form is replicas only (independent pictures / streams per
rank, no exchange step); what crosses ranks is the timing: bench.py takes the
slowest rank's time and all ranks' units.  Checked here with two gloo ranks on
the CPU (127.0.0.1 rendezvous)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seconds = [0.5, 2.0][rank]                       # rank 1 is the slow replica
    slowest = bench.reduce_max(seconds, "cpu")
    rate = bench.aggregate_rate(1000, seconds, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, slowest, rate))


def test_replica_timing_gloo_world2():
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, rate in got:
        assert slowest == pytest.approx(2.0)
        assert rate == pytest.approx(2 * 1000 / 2.0)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5, "cpu") == 3.5
    assert bench.aggregate_rate(10, 2.0, "cpu") == 5.0
