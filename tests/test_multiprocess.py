"""Replicas-only multi-GPU host logic, run as two gloo ranks on the CPU:
barrier, max-over-ranks timing, event partitioning and the whole-job rate
that bench.py reports for --gpus N."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    from trax_gb300 import gen
    dist = bench.Dist()
    try:
        dist.barrier()
        B = 3
        first = bench.replica_first_event(rank, B)
        b = gen.generate_batch(gen.WORKLOADS["single-muon-100trk"], B, first_event=first)
        # rank 1 is "slower": the job time is the slowest rank's
        value, ms, events = bench.aggregate_rate(dist, B, 10, 100.0 * (rank + 1))
        q.put((rank, first, float(b.x[0]), value, ms, events))
    finally:
        dist.close()


def test_two_gloo_ranks_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    (r0, f0, x0, v0, ms0, e0), (r1, f1, x1, v1, ms1, e1) = res
    assert (f0, f1) == (0, 3)            # disjoint events per replica
    assert x0 != x1                      # different seeded events
    assert ms0 == ms1 == 200.0           # max over ranks
    assert e0 == e1 == 6                 # all ranks' events
    assert v0 == v1 == pytest.approx(6 * 10 / 0.2)
