"""The N > 1 host path of bench.py and the serving replicas, on two CPU processes (gloo backend).

bench.py --gpus N runs N independent replicas (one process per GPU): every rank times its own work, the
step time is the maximum over ranks, and the serving stream is spread round-robin over the replicas with
whole-job statistics merged on every rank.  No GPU is used: the solves are replaced by a fake.
"""
import os
import socket
import time

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _FakeSolve:
    def __call__(self, req, stream, keep, preconditioner="gmg"):
        time.sleep(0.002)

        class R:
            status, outer_iterations, iterations, rel_residual = 0, 1, 1, 1e-12
            t_setup, t_solve = 0.0, 0.001

        return R(), None, float(req.rid), 10 * req.n


class _FakeStream:  # the fake solve needs no stream; the server's warm-up synchronises it
    def synchronize(self):
        pass


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from mrhyde_gb300 import serving

        out = {"max": bench.max_over_ranks(1.5 + rank, dist, "cpu")}
        serving.solve_request = _FakeSolve()
        torch.cuda.Stream = _FakeStream
        reqs = serving.poisson_stream(rate=2000.0, count=24, edge=(4, 6), seed=3)
        mine = serving.shard(reqs, rank, world)
        ids = [None] * world
        dist.all_gather_object(ids, sorted(r.rid for r in mine))
        out["ids"] = ids
        whole = bench.serve_replicated(reqs, 3, False, rank, world, dist)
        out["whole"] = {k: whole[k] for k in ("requests", "ok", "replicas")}
        out["dof"] = whole["dof_per_s"] * whole["wall_s"]
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        assert res[r]["max"] == 2.5                     # max over ranks, seen by every rank
        ids = res[r]["ids"]
        assert sorted(ids[0] + ids[1]) == list(range(24)) and not set(ids[0]) & set(ids[1])
        assert res[r]["whole"] == {"requests": 24, "ok": 24, "replicas": 2}
    from mrhyde_gb300 import serving
    total = sum(10 * q.n for q in serving.poisson_stream(rate=2000.0, count=24, edge=(4, 6), seed=3))
    assert abs(res[0]["dof"] - total) < 1e-6 * total
