"""Replica runs on the CPU: two gloo ranks, barrier and max-over-ranks timing,
whole-job throughput (the bench's N > 1 path without a GPU)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    from aerojax_gb300 import replicas
    w, r = replicas.init("gloo")
    assert (w, r) == (world, rank)
    replicas.barrier()
    ms = 10.0 + 5.0 * rank            # rank 1 is the slowest
    m = replicas.max_over_ranks(ms)
    out[rank] = (m, replicas.throughput(1000, 4, m, w))
    replicas.finalize()


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    assert abs(res[0][1] - 2 * 1000 * 4 / 15e-3 / 1e6) < 1e-9


def test_single_process_defaults():
    from aerojax_gb300 import replicas
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.throughput(10, 2, 1.0, 1) == 10 * 2 / 1e-3 / 1e6
