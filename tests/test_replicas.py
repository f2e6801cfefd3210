"""The N>1 host path of bench.py (independent replicas, barrier + max-over-ranks timing) with two
gloo ranks on the CPU.  Each rank runs its own flume replica through the CPU oracle, so the test
also checks that replicas do not interact."""
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


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import time
    from avalancheflume3d_gb300 import replicas
    from oracle.pyoracle import Oracle, OracleRun, dense_state
    from tests.states import flume_system
    r = replicas.from_env()
    replicas.init(r, backend="gloo")
    n = 200
    sys_, fun = flume_system(n, time=0.0)
    pp = dense_state(n, 40 + rank, sys_, box=(1.0, 8.0, 26.0))   # a different flume per rank
    run = OracleRun(Oracle(), sys_, fun, pp)
    run.seed_accel()
    replicas.barrier(r)
    t0 = time.perf_counter()
    run.step(3 + rank, cc0=0)                                     # ranks take different times
    dt = time.perf_counter() - t0
    replicas.barrier(r)
    slowest = replicas.max_over_ranks(r, dt)
    value = replicas.aggregate_throughput(r, n * 3, dt)
    q.put((rank, dt, slowest, value, run.pp["rr"].sum()))
    replicas.finalize(r)


def test_two_gloo_ranks_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, dt0, s0, v0, x0), (r1, dt1, s1, v1, x1) = out
    assert s0 == s1 == max(dt0, dt1)              # every rank sees the slowest time
    assert v0 == v1 == pytest.approx(2 * 200 * 3 / max(dt0, dt1))
    assert x0 != x1                               # independent replicas


def test_single_rank_defaults(monkeypatch):
    from avalancheflume3d_gb300 import replicas
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    r = replicas.from_env()
    assert (r.rank, r.world, r.local, r.distributed) == (0, 1, 0, False)
    assert replicas.max_over_ranks(r, 1.5) == 1.5
    assert replicas.aggregate_throughput(r, 100.0, 2.0) == 50.0
