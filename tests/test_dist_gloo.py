"""Multi-rank host logic on CPU (gloo, world size 2)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from bosonsupremacy_gb300.dist import cuts_needed, shard_sites


def test_shard_sites_cover_every_site_once():
    for M in (2, 3, 8, 16, 50, 144, 216):
        for world in (1, 2, 3, 4, 8):
            if world > M:
                continue
            r = shard_sites(M, world)
            assert len(r) == world
            assert r[0][0] == 0 and r[-1][1] == M
            assert all(a < b for a, b in r)
            assert all(r[i][1] == r[i + 1][0] for i in range(world - 1))


def test_shard_cuts_cover_every_cut_once():
    from bosonsupremacy_gb300.dist import shard_cuts
    for M in (3, 8, 16, 50, 144, 216):
        for world in (1, 2, 3, 4, 8):
            if world > M - 1:
                continue
            r = shard_cuts(M, world)
            assert len(r) == world and r[0][0] == 0 and r[-1][1] == M - 1
            assert all(a < b for a, b in r) and all(r[i][1] == r[i + 1][0] for i in range(world - 1))


def test_rank_world_from_environment(monkeypatch):
    from bosonsupremacy_gb300.dist import rank_world
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("LOCAL_RANK", raising=False)
    assert rank_world() == (0, 1, 0)
    monkeypatch.setenv("RANK", "3")
    monkeypatch.setenv("WORLD_SIZE", "4")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert rank_world() == (3, 4, 1)


def test_cuts_needed():
    assert cuts_needed((0, 5), 10) == (0, 5)
    assert cuts_needed((5, 10), 10) == (4, 9)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from bosonsupremacy_gb300.dist import reduce_max, shard_sites
    plan = shard_sites(144, world)
    mx = reduce_max(float(rank + 1) * 10.0)
    q.put((rank, plan[rank], mx))
    dist.destroy_process_group()


def test_gloo_two_ranks_reduce_and_plan():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [o[2] for o in out] == [20.0, 20.0]
    assert out[0][1][1] == out[1][1][0]  # contiguous, disjoint
