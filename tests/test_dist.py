r"""The multi-process paths of bench.py on CPU: two gloo ranks on 127.0.0.1.

The workloads shard with no exchange between ranks (replicas of the single
solve; round-robin shares of the batched problems), so the only collectives
are the timing barrier, the max of the ranks' times and the gather of the
batched problems' results.  These run here without a GPU.
"""

import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_init(argparse.Namespace(impl="reference"), backend="gloo")
    out = {"world": w, "rank": r, "local": local}
    items = list(range(64))
    out["shard"] = bench.shard(items, r, w)
    bench.barrier(w)
    out["max"] = bench.max_over_ranks(10.0 * (r + 1), w)
    parts = [None] * w
    dist.all_gather_object(parts, {r: len(out["shard"])})
    out["gathered"] = parts
    dist.destroy_process_group()
    q.put(out)


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort(key=lambda d: d["rank"])
    assert [d["world"] for d in results] == [2, 2]
    # round-robin shards are disjoint and cover every problem
    a, b = results[0]["shard"], results[1]["shard"]
    assert not set(a) & set(b) and sorted(a + b) == list(range(64))
    assert a[:3] == [0, 2, 4] and b[:3] == [1, 3, 5]
    # max over ranks of (10, 20)
    assert results[0]["max"] == results[1]["max"] == 20.0
    assert results[0]["gathered"] == [{0: 32}, {1: 32}]


def test_single_process_defaults():
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        if k in os.environ:
            pytest.skip("running under a launcher")
    assert bench.dist_init(argparse.Namespace(impl="ours")) == (1, 0, 0)
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.shard([1, 2, 3], 0, 1) == [1, 2, 3]
