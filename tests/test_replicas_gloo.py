"""bench.py's multi-GPU mode is replicas only (independent solves, no data-path
collective); its barrier and max-over-ranks timing run over world_size 2
gloo ranks on CPU here."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist("gloo")
    d.barrier()
    m = d.max(float(10 * rank + 3))
    d.close()
    q.put((rank, m))


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 13.0, 1: 13.0}


def test_single_rank_env_defaults(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench
    assert bench.dist_env() == (1, 0, 0)
    d = bench.Dist("gloo")
    assert d.max(2.5) == 2.5
