"""The bench's N>1 path on the CPU: two `gloo` ranks aggregate their replica times as the
bench does under torchrun (slowest rank's time, all ranks' units), with no GPU."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                          RANK=str(rank), WORLD_SIZE=str(world))
        sys.path.insert(0, str(ROOT))
        import torch.distributed as dist

        import bench

        dist.init_process_group("gloo", rank=rank, world_size=world)
        try:
            # rank r processed 5 units in 1 + r seconds; rank 1 is the slowest
            rate, secs = bench.replica_rate(5, 1.0 + rank, world, "cpu")
            # a GFLOP-valued unit, as the pair workload aggregates it
            grate, _ = bench.replica_rate(7.92 * 3, 0.5 * (rank + 1), world, "cpu")
            dist.barrier()
        finally:
            dist.destroy_process_group()
        q.put((rank, rate, secs, grate))
    except BaseException as e:  # reported to the parent, which fails the test
        q.put((rank, repr(e), None, None))


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_rate(10, 2.0, 1) == (5.0, 2.0)


@pytest.mark.timeout(120)
def test_replica_rate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, rate, secs, grate = q.get(timeout=100)
        out[rank] = (rate, secs, grate)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank in range(2):
        rate, secs, grate = out[rank]
        assert secs is not None, rate
        assert secs == 2.0
        assert rate == pytest.approx(2 * 5 / 2.0)
        assert grate == pytest.approx(2 * 7.92 * 3 / 1.0)
