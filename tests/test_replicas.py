"""The multi-GPU path is N independent replicas: a barrier around the timed region and
max/sum reductions of per-rank results, no data-path collective.  Checked with two gloo
ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from sandengine_gb300.replicas import Replicas
    rep = Replicas("gloo")
    rep.barrier()
    mx = rep.max(10.0 * (rank + 1))
    sm = rep.sum(1.5)
    rep.barrier()
    rep.close()
    q.put((rank, mx, sm))


def test_two_gloo_replicas_reduce():
    import multiprocessing as mp
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 20.0, 3.0), (1, 20.0, 3.0)]


def test_single_process_is_a_no_op(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    from sandengine_gb300.replicas import Replicas
    rep = Replicas("gloo")
    assert rep.world_size == 1 and rep.max(3.0) == 3.0 and rep.sum(2.0) == 2.0
    rep.barrier()
    rep.close()
