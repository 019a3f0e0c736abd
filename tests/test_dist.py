"""The bench's multi-rank path on CPU: two gloo ranks, as torchrun starts them.

Each rank advances its own replicas; the only collectives are the barrier
around the timed region, the max over ranks of the elapsed time and the
gather of per-replica results. The batched replicas are split over the ranks
by the LPT rule (implicit_dpd_gb300.partition). These tests run the ranks as
spawned processes on 127.0.0.1; the replicas step through the CPU oracle.
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


def test_lpt_partition_covers_every_replica_once_and_balances():
    sys.path.insert(0, ROOT)
    from implicit_dpd_gb300 import configs
    from implicit_dpd_gb300.partition import imbalance, lpt_partition

    sizes = [len(r["state"]["pos"]) for r in configs.mdpd_replicas(256)]
    for ranks in (1, 2, 3, 4, 8):
        parts, loads = lpt_partition(sizes, ranks)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        assert loads == [sum(sizes[i] for i in p) for p in parts]
        mean = sum(sizes) / ranks
        assert max(loads) <= mean + max(sizes)  # the LPT bound
        assert imbalance(loads) < 1.02  # 256 uneven replicas deal out evenly
    # 5 -> rank 0, 4 -> rank 1, 3 -> rank 1 (4 < 5), 3 -> rank 0, 3 -> rank 1
    assert lpt_partition([5, 4, 3, 3, 3], 2) == ([[0, 3], [1, 2, 4]], [8, 10])


def _replica_rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench

    r, w, _ = bench.dist_env()
    d = bench.Dist(w)
    res = bench.replica_observables_cpu(small_replicas(), r, w, d, steps=3)
    d.close()
    with open(os.path.join(out_dir, f"rep{r}.json"), "w") as f:
        json.dump(res, f)


def small_replicas():
    sys.path.insert(0, ROOT)
    from implicit_dpd_gb300 import configs

    return configs.mdpd_replicas(6, n_min=300, n_max=900)


def test_partitioned_replicas_gather_to_the_one_rank_result(tmp_path):
    """Two gloo ranks each step their LPT share of six small replicas (CPU
    oracle, Warren form) and gather the per-replica kinetic temperatures:
    every replica is stepped by exactly one rank, and the gathered values
    equal those of one rank stepping all six."""
    world = 2
    mp.start_processes(_replica_rank_main, args=(world, _free_port(), str(tmp_path)),
                       nprocs=world, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rep{r}.json")) for r in range(world)]
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench

    one = bench.replica_observables_cpu(small_replicas(), 0, 1, bench.Dist(1), steps=3)
    assert sorted(res[0]["stepped_here"] + res[1]["stepped_here"]) == list(range(6))
    assert res[0]["owner"] == res[1]["owner"] and set(res[0]["owner"]) == {0, 1}
    assert res[0]["temperature"] == res[1]["temperature"] == one["temperature"]
