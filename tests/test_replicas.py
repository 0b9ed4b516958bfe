"""Multi-GPU runs are independent replicas (the step has no data exchange): the
bench's rank plumbing is exercised here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, out):
    os.environ.update({"WORLD_SIZE": str(ws), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, REPO)
    import bench
    rep = bench.Replicas(backend="gloo")
    rep.barrier()
    got = rep.max(10.0 + rank)       # per-rank times: the job time is the slowest rank
    total = rep.max(rank * 100.0)
    rep.close()
    out.put((rank, got, total))


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 11.0, 100.0), (1, 11.0, 100.0)]


def test_single_rank_is_a_no_op(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "1")
    sys.path.insert(0, REPO)
    import bench
    rep = bench.Replicas()
    rep.barrier()
    assert rep.max(3.5) == 3.5
    rep.close()


def test_each_rank_builds_its_own_replica_scene():
    """Ranks seed their scene with seed + rank: replicas are independent simulations."""
    src = open(os.path.join(REPO, "bench.py")).read()
    assert "build_scene(args.seed + rank," in src or "build_scene(args.seed + rank)" in src
