"""The bench's multi-rank path on CPU: two gloo ranks, as torchrun starts them.

Each rank advances its own replica; the only collectives are the barrier
around the timed region and the max over ranks of the elapsed time. These
tests run both ranks as spawned processes on 127.0.0.1.
"""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    r, w, lr = bench.dist_env()
    d = bench.Dist(w)
    d.barrier()
    got = d.max(10.0 * (r + 1))
    d.barrier()
    d.close()

    class Args:
        steps, warmup = 1, 0

    # the reference arm runs on rank 0 only; the other ranks return at once
    ran = None
    if r != 0:
        ran = bench.run_reference(Args(), r, w)
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump({"rank": r, "world": w, "local": lr, "max": got, "ref": ran}, f)


def test_two_gloo_ranks_barrier_and_max(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r, d in enumerate(res):
        assert d["rank"] == r and d["world"] == world and d["local"] == r
        assert d["max"] == 10.0 * world
    assert res[1]["ref"] is None


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist(1)
    d.barrier()
    assert d.max(3.5) == 3.5
    d.close()
