"""Replica mode across ranks (gloo, world size 2, CPU): disjoint shares, max-over-ranks timing."""
import os

import pytest

from scip_gb300 import replicas


def test_split_covers_everything_once():
    for total in (0, 1, 7, 4096):
        for world in (1, 2, 3, 8):
            seen = [i for r in range(world) for i in replicas.split(total, world, r)]
            assert seen == list(range(total))


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = replicas.rank_env()
    local_ms = 10.0 + 5.0 * r  # rank 1 is the slower replica
    ms = replicas.max_over_ranks(local_ms)
    rate = replicas.aggregate_rate(4096, w, ms)
    share = replicas.split(4096, w, r)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, ms, rate, len(share), replicas.node_seed(3, r)))


def test_two_gloo_ranks_agree_on_the_slowest_step():
    mp = pytest.importorskip("torch.multiprocessing")
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[2] for o in out] == [15.0, 15.0]
    assert all(o[3] == pytest.approx(2 * 4096 / 0.015) for o in out)
    assert [o[4] for o in out] == [2048, 2048]
    assert out[0][5] != out[1][5]
