"""Replica (multi-GPU) host logic on CPU with torch.distributed gloo, world
size 2: the serving stream is sharded by request with no data-path
collective, each rank's shard is disjoint and together they cover the
stream, and the whole-job numbers are reduced as bench.py does (max over
ranks for time)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from qibo_gb300.serving import make_stream, merge_stats, shard_requests

        reqs = make_stream(37, rate=0.0, seed=4, nmin=4, nmax=6, dmin=2, dmax=3, nshots=10)
        mine = shard_requests(reqs, rank, world)
        ids = torch.zeros(len(reqs), dtype=torch.int64)
        for r in mine:
            ids[r.rid] = 1
        dist.all_reduce(ids)  # every request counted exactly once
        fake = {"requests": len(mine), "wall_s": 1.0 + rank, "p50_ms": 5.0 * (rank + 1), "p99_ms": 9.0 * (rank + 1)}
        t = torch.tensor([fake["wall_s"]], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        gathered = [None] * world
        dist.all_gather_object(gathered, fake)
        merged = merge_stats(gathered)
        q.put((rank, ids.tolist(), float(t.item()), merged))
    finally:
        dist.destroy_process_group()


def test_request_sharding_and_reduction_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ids, tmax, merged in out:
        assert ids == [1] * 37
        assert tmax == 2.0
        assert merged["requests"] == 37 and merged["wall_s"] == 2.0 and merged["p99_ms"] == 18.0


def test_shard_rejects_bad_rank():
    from qibo_gb300.serving import make_stream, shard_requests

    with pytest.raises(ValueError):
        shard_requests(make_stream(3, 0.0, nmin=3, nmax=3, dmin=1, dmax=1), 2, 2)
