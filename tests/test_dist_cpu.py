"""The multi-GPU path of bench.py is replicas: every rank renders its own
request stream and the job reports all ranks' frames over the slowest rank's
time, with no collective on the data path.  Checked on CPU with two gloo
ranks (the aggregation is backend-independent)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import sys

    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench
    from swegl_gb300 import scenes as S

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = bench.env_rank()
    step_ms = 100.0 * (rank + 1)  # rank 1 is the slow one
    slowest = bench.max_over_ranks(torch, dist, step_ms, device="cpu")
    total = bench.sum_over_ranks(torch, dist, 10.0, device="cpu")
    fps = bench.replica_throughput(256, w, slowest)
    reqs = S.serving_requests(4, seed=60 + rank)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, r, w, slowest, total, fps, [(k, v.w, v.h) for (_, k, v) in reqs]))


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(i, 2, port, q)) for i in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, rr0, w0, slow0, tot0, fps0, reqs0), (r1, rr1, w1, slow1, tot1, fps1, reqs1) = out
    assert (rr0, rr1, w0, w1) == (0, 1, 2, 2)
    assert slow0 == slow1 == 200.0           # the job waits for the slowest replica
    assert tot0 == tot1 == 20.0
    assert fps0 == pytest.approx(2 * 256 / 0.2)
    assert reqs0 != reqs1                     # each replica serves its own stream
