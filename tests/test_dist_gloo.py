"""The multi-process path of bench.py (replicas, no data-path collective) on CPU with gloo."""

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    r, w, lr = bench.dist_env()
    assert (r, w, lr) == (rank, world, rank)
    d = bench.Dist(w)
    d.barrier()
    mx = d.reduce(10.0 * (rank + 1), "max")
    sm = d.reduce(100.0 + rank, "sum")
    d.barrier()
    d.close()
    out.put((rank, mx, sm))


def test_two_rank_barrier_and_reductions():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 20.0, 201.0), (1, 20.0, 201.0)]


def test_partition_is_deterministic_balanced_and_complete():
    from opensurgsim_gb300 import mesh, shard

    scenes = mesh.scenes_batch(count=256)
    w = [shard.mesh_weight(s.mesh) for s in scenes]
    for k in (1, 2, 3, 4, 8):
        bins = shard.partition(w, k)
        assert bins == shard.partition(w, k)
        flat = sorted(i for b in bins for i in b)
        assert flat == list(range(len(w)))
        loads = [sum(w[i] for i in b) for b in bins]
        assert max(loads) <= sum(w) / k + max(w) + 1e-9


def _shard_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    from opensurgsim_gb300 import shard

    d = bench.Dist(world)
    scenes = bench.batch_scenes(32)
    mine = shard.partition([shard.mesh_weight(s.mesh) for s in scenes], world)[rank]
    tets = sum(scenes[i].mesh.num_tets for i in mine)
    total = d.reduce(tets, "sum")
    d.close()
    out.put((rank, tuple(mine), total, sum(s.mesh.num_tets for s in scenes)))


def test_two_ranks_shard_the_batch_without_overlap():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    a, b = set(res[0][1]), set(res[1][1])
    assert not (a & b) and len(a | b) == 32
    assert res[0][2] == res[0][3] == res[1][2]
