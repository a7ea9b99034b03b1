"""Replicas over several ranks (gloo, CPU): the timing collectives the bench
uses -- barrier, max of times, sum of work -- and the per-rank seeding."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from acctricnt_gb300 import replicas
    r, w, _ = replicas.setup()
    replicas.barrier(w)
    mx = replicas.max_over_ranks(10.0 * (r + 1), w)
    sm = replicas.sum_over_ranks(r + 1, w)
    out.put((r, w, mx, sm, replicas.rank_seed(1, r)))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_gloo_replica_collectives(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, mx, sm, seed) in enumerate(res):
        assert rank == r and w == world
        assert mx == 10.0 * world
        assert sm == world * (world + 1) / 2
        assert seed == 1 + r
