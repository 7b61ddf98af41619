"""Multi-rank measurement path (replicas only) with gloo on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, values, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from fermicc.replicas import max_over_ranks
    out[rank] = max_over_ranks(values[rank], world)
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    values = [1.25, 3.5]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == 3.5


def test_single_rank_is_identity():
    from fermicc.replicas import max_over_ranks
    assert max_over_ranks(2.0, 1) == 2.0
