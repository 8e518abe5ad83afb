"""The multi-GPU path is replicas only: each rank checks its own seeded
shard of edges, the job's time is the max over ranks, rank 0 reports.  These
tests run that host logic as world-size-2 gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import sys

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, local = bench.dist_env()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(world)
    # the slowest replica sets the job time
    t = bench.reduce_max(1.0 + rank, world)
    scene, q1, q2, N = bench.workload(rank)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), t=t, q1=q1[:64], N=N[:64])
    bench.barrier(world)
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_max(tmp_path):
    world, port = 2, _free_port()
    mp.spawn(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    r0, r1 = np.load(tmp_path / "rank0.npz"), np.load(tmp_path / "rank1.npz")
    assert float(r0["t"]) == float(r1["t"]) == 2.0
    # every rank gets its own seeded shard (weak scaling, no data exchange)
    assert not np.array_equal(r0["q1"], r1["q1"])
    assert r0["q1"].shape == r1["q1"].shape


def test_reference_arm_other_ranks_do_nothing(monkeypatch):
    import sys

    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup = 3, 3

    # rank 1 of the reference arm exits 0 without work (rank 0 alone runs it)
    assert bench.run_reference(A()) == 0


def _rank_fail_main(rank, world, port, out_dir):
    """Rank 1 leaves between steps (raises before the next barrier); rank 0
    learns of it from the process group within its short timeout instead of
    waiting forever, and records the error."""
    import datetime
    import sys

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=5))
    bench.barrier(world)                      # step 1: both ranks
    if rank == 1:
        os._exit(0)                           # leaves with nothing in flight
    try:
        bench.reduce_max(1.0, world)          # step 2: the peer is gone
        outcome = "returned"
    except Exception as e:                    # noqa: BLE001 - any process-group error counts
        outcome = "error: " + type(e).__name__
    with open(os.path.join(out_dir, "rank0.txt"), "w") as f:
        f.write(outcome)
    os._exit(0)


def test_failed_rank_is_detected_by_the_other(tmp_path):
    world, port = 2, _free_port()
    ctx = mp.spawn(_rank_fail_main, args=(world, port, str(tmp_path)), nprocs=world, join=False)
    for p in ctx.processes:
        p.join(timeout=60)
    alive = [p for p in ctx.processes if p.is_alive()]
    for p in alive:
        p.kill()
    assert not alive, "a rank hung instead of failing"
    outcome = (tmp_path / "rank0.txt").read_text()
    assert outcome.startswith("error:"), outcome


def test_bench_spawns_its_own_replicas():
    """`bench.py --gpus 2` without torchrun starts two replica processes
    itself (gloo in the dry run: no GPU work) and rank 0 alone prints one
    line whose n_gpus is the world size."""
    import json
    import subprocess
    import sys

    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--dry-run", "--steps", "3",
                        "--warmup", "3"], capture_output=True, text=True, timeout=300,
                       env={k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["config"]["parallelism"] == "replicas x2"
    assert d["config"]["edges_total"] == 2 * d["config"]["edges_per_step"]
