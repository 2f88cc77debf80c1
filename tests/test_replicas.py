"""The replica coordination of bench.py on two CPU processes (gloo): barrier,
maximum over ranks, whole-job rate."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from hydrodynamicsgpu_gb300.replicas import Replicas
    r = Replicas()
    r.barrier()
    seconds = 1.0 + rank          # rank 1 is the slow one
    out[rank] = (r.max(seconds), r.rate(100.0, seconds), r.world)
    r.barrier()
    r.close()


def test_two_replicas_max_and_rate():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(k, 2, port, out)) for k in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        for k in range(2):
            mx, rate, world = out[k]
            assert world == 2 and mx == 2.0 and rate == 100.0 * 2 / 2.0


def test_single_process_needs_no_group(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    from hydrodynamicsgpu_gb300.replicas import Replicas
    r = Replicas()
    assert r.world == 1 and r.max(3.5) == 3.5 and r.rate(10.0, 2.0) == 5.0
    r.barrier()
    r.close()
