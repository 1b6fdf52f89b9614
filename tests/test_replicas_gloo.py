"""The N > 1 path of bench.py (independent replicas, one per GPU) on CPU:
two gloo ranks run the host logic the GPU ranks run — per-rank workloads,
barrier, and the whole-job aggregate (all ranks' work over the slowest
rank's time)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist(ws, rank, backend="gloo")
    sims = bench.make_workload("plummer_disk", 256, rank)
    first_x = float(sims[0]["x"][0])
    d.barrier()
    # rank r did (r + 1) * 1e9 interactions in (10 + r) ms
    value, t_max, work = bench.aggregate(d, (rank + 1) * 1e9, 10.0 + rank)
    out.put((rank, value, t_max, work, first_x))
    d.close()


def test_two_gloo_replicas_aggregate_like_the_gpu_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, t_max, work, _ in res:
        assert t_max == 11.0  # the slowest rank
        assert work == 3e9  # every rank's work
        assert value == pytest.approx(3e9 / 11e-3)
    # each replica simulates its own seeded collection
    assert res[0][4] != res[1][4]


def _shard_rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist(ws, rank, backend="gloo")
    sims = bench.make_workload("ensemble", 0, rank, ws)
    ids = sorted((len(b["x"]), round(float(b["x"].sum()), 6)) for b in sims)  # a fingerprint of each collection
    work = sum(len(b["x"]) * (len(b["x"]) - 1) for b in sims)
    total = d.sum(work)
    d.barrier()
    out.put((rank, len(sims), work, total, ids))
    d.close()


def test_ensemble_splits_over_gloo_ranks_without_exchange():
    """--workload ensemble with two ranks: each rank derives the same split of
    the 512 collections on its own; together they hold every collection once,
    with the pair work balanced."""
    mp = pytest.importorskip("torch.multiprocessing")
    import bench
    from nbodygo_gb300 import workloads as W

    sizes = [len(b["x"]) for b in W.ensemble(seed=5)]
    whole = sum(n * (n - 1) for n in sizes)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] + res[1][1] == 512
    assert res[0][3] == res[1][3] == whole  # the job's work, summed over ranks
    assert abs(res[0][2] - res[1][2]) <= 0.01 * whole  # balanced to 1 %
    assert not set(res[0][4]) & set(res[1][4])  # no collection on both ranks
    # the split is a partition of every collection
    shards = bench.shard_collections(sizes, 4)
    assert sorted(k for s in shards for k in s) == list(range(512))
