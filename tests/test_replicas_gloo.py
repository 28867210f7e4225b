"""World-size-2 gloo test of the replica benchmark path (CPU only): every
rank times its own replica; the reported step time is the maximum over
ranks and every rank sees the same value."""
import multiprocessing as mp
import os
import sys
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from parrsb_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, l = replicas.dist_env()
    replicas.barrier(w)
    t = replicas.max_over_ranks(1.5 + rank, w)   # rank 1 is the slow replica
    s = replicas.sum_over_ranks(10, w)            # units processed by all ranks
    dist.destroy_process_group()
    q.put((r, w, t, s))


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [x[0] for x in res] == [0, 1]
    assert all(x[1] == 2 and x[2] == 2.5 and x[3] == 20.0 for x in res)


def test_single_rank_is_identity(monkeypatch):
    from parrsb_gb300 import replicas
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.dist_env() == (0, 1, 0)
    assert replicas.max_over_ranks(3.0, 1) == 3.0
