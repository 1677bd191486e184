"""Multi-GPU replicas logic on CPU: two gloo ranks (spawned processes) run
their own seeded frames through the FP64 oracle, combine step times by
max-over-ranks and report the whole-job rate -- the structure bench.py uses
with NCCL on GPUs.  No collective touches the data path."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle
    from cos_gb300 import replicas, synth
    r, _, w = replicas.env()
    dist = replicas.init("gloo")
    x = synth.cube(24, 2, 16, [10.0], seed=100 + r)          # this rank's own frame
    P = oracle.capon(x, 0.01, 8, 1)["P"]
    replicas.barrier(dist)
    ms = replicas.max_over_ranks(dist, 1.0 + r)              # rank r "took" 1 + r ms
    rate = replicas.aggregate_rate(P.size, ms, w)
    out.put((r, w, ms, rate, float(P.sum()), replicas.shard(256, r, w)))
    replicas.finalize(dist)


def test_two_gloo_ranks_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, ms0, rate0, s0, sh0), (r1, w1, ms1, rate1, s1, sh1) = res
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert ms0 == ms1 == 2.0                                   # the slowest rank's time on every rank
    assert rate0 == rate1 == pytest.approx(2 * 22 * 2 / 2e-3)  # 2 ranks x (2 beams x 22 pixels) / 2 ms
    assert s0 != s1                                            # independent frames
    assert sh0 == (0, 128) and sh1 == (128, 256)


def test_single_process_is_the_identity():
    from cos_gb300 import replicas
    assert replicas.init("gloo") is None or int(os.environ.get("WORLD_SIZE", "1")) > 1
    assert replicas.max_over_ranks(None, 3.5) == 3.5
    assert replicas.aggregate_rate(1000, 2.0, 1) == pytest.approx(5e5)
    assert [replicas.shard(10, r, 3) for r in range(3)] == [(0, 3), (3, 6), (6, 10)]
