"""The multi-process path of bench.py on CPU: two gloo ranks (replicas only,
no data-path collective) check the barrier, the max-over-ranks timing
reduction and the reference arm, which runs on rank 0 alone."""
from __future__ import annotations

import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import argparse

    import bench
    w, r, _, pg = bench.dist_setup()
    out = {"rank": r, "world": w}
    out["max"] = bench.max_over_ranks(pg, 1.5 + r)
    bench.barrier(pg)
    args = argparse.Namespace(workload="c2c_1024x4096", steps=1, warmup=1, impl="reference", batch=0,
                              no_cpu_baseline=False)
    res = bench.run_reference(args, w, r, pg)
    out["reference"] = None if res is None else {k: res[k] for k in ("impl", "n_gpus", "unit", "value")}
    bench.barrier(pg)
    pg.destroy_process_group()
    q.put(out)


def test_two_gloo_ranks_reduce_and_run_the_reference_arm_on_rank0():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    by_rank = {r["rank"]: r for r in results}
    assert set(by_rank) == {0, 1}
    for r in results:
        assert r["world"] == 2 and r["max"] == 2.5
    ref = by_rank[0]["reference"]
    assert ref["impl"] == "reference" and ref["n_gpus"] == 2 and ref["unit"] == "GFLOP/s" and ref["value"] > 0
    assert by_rank[1]["reference"] is None  # the other ranks do no work
