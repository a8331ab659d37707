"""The multi-GPU form of the benchmark: independent replicas, one process per
GPU, no data-path collective (the path does not shard: every rank runs the
whole job on its own block of realizations).  Its host side — process-group
set-up from the launcher's environment, the barrier around the timed region,
the maximum of the ranks' times, and disjoint draw seeds per rank — runs
here as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    ws, r, local = bench.dist_setup(None)
    bench.barrier(ws)
    slowest = bench.max_over_ranks(ws, 10.0 + r)  # rank r "took" 10 + r ms
    seeds = [bench.replica_seed(1000 + i) for i in range(3)]
    bench.barrier(ws)
    dist.destroy_process_group()
    q.put((r, ws, local, slowest, seeds))


def test_two_gloo_replicas():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ws0, l0, m0, s0), (r1, ws1, l1, m1, s1) = got
    assert (r0, r1) == (0, 1) and ws0 == ws1 == 2 and (l0, l1) == (0, 1)
    assert m0 == m1 == 11.0  # every rank reports the slowest rank's time
    assert not set(s0) & set(s1)  # replicas draw disjoint realizations
