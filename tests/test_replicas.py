"""bench.py's multi-GPU mode: one replica per rank, the time of the slowest rank, the whole-job
rate over all ranks.  Run as two gloo ranks on the CPU (no GPU involved)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    r, w = bench.init_replicas()
    t = bench.max_over_ranks(1.0 + rank, w)           # rank 1 is the slower replica
    rate = bench.replica_rate(1_000_000, t, w)
    import torch.distributed as dist
    dist.destroy_process_group()
    out.put((r, w, t, rate))


def test_two_replicas_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == 2.0 for r in res)                 # both see the slowest rank's time
    assert all(abs(r[3] - 1.0) < 1e-12 for r in res)      # 2 ranks x 1e6 units / 2 s = 1 M/s


def test_single_process_is_one_replica():
    import bench
    os.environ.pop("WORLD_SIZE", None)
    assert bench.init_replicas()[1] == 1
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_rate(2_000_000, 2.0, 1) == 1.0
