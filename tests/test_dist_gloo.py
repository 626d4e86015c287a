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


def test_shard_weight_tracks_oracle_cg_iterations():
    """The shard weight's iteration model against the oracle's CG iteration counts for one step of
    a spread of batch meshes (stiff and soft, small and larger): within 35% on each, and the
    weight orders the meshes' measured solve work (nodes x iterations) almost perfectly."""
    import numpy as np

    from opensurgsim_gb300 import mesh, shard
    from oracle import oracle as O

    scenes = mesh.scenes_batch(count=256)
    order = sorted(range(len(scenes)), key=lambda i: scenes[i].mesh.num_nodes)
    picks = order[:120:10]  # 12 meshes of 500 to ~4,000 nodes, E across the batch's range
    est, meas, work_est, work = [], [], [], []
    for i in picks:
        s = scenes[i]
        model = O.OracleModel.from_scene(s)
        assert model.step(1e-3, 1) == 0
        it = model.last_stats.cg_iterations
        e = shard.expected_cg_iterations(s.mesh)
        est.append(e)
        meas.append(it)
        work_est.append(shard.mesh_weight(s.mesh))
        work.append(s.mesh.num_nodes * (it + shard.ELEMENT_ITERS))
    est, meas = np.array(est), np.array(meas)
    assert np.max(np.abs(est - meas) / meas) <= 0.35, list(zip(est.round(1), meas))
    rank = lambda a: np.argsort(np.argsort(a))  # noqa: E731
    rho = np.corrcoef(rank(np.array(work_est)), rank(np.array(work)))[0, 1]
    assert rho >= 0.95, rho
