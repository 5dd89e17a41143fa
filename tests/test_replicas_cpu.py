"""The multi-GPU path is replicas only: every rank solves its own request and
the benchmark reports the whole job's freq-points/s over the slowest rank's
time.  These tests run that host logic as two gloo ranks on the CPU."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_local = [800.0, 1250.0][rank]               # rank 1 is the slow one
    ms = bench.slowest_rank_ms(ms_local)
    value = bench.replica_value(ms, 5, 256, world)
    w = bench.workload(rank)
    dist.barrier()
    q.put((rank, ms, value, w["distance"].tolist()))
    dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_distinct_stacks():
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, v0, d0), (r1, ms1, v1, d1) = res
    assert ms0 == ms1 == 1250.0                     # both ranks see the slowest rank's time
    assert v0 == v1 == pytest.approx(256 * 2 / (1250.0 / 5 / 1000.0))
    assert not np.allclose(d0, d1)                  # each rank solves its own seeded stack


def test_single_process_identity():
    sys.path.insert(0, REPO)
    import bench
    assert bench.slowest_rank_ms(42.0) == 42.0
    assert bench.replica_value(1000.0, 5, 256, 1) == pytest.approx(1280.0)
