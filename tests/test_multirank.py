"""The multi-rank path of bench.py on CPU (world size 2, gloo, 127.0.0.1).  The path
shards by replicas only: every rank runs its own batch (distinct seeds), nothing
is exchanged during the run, and the one collective, outside the timed region,
takes the slowest rank's time for the whole-job value."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    seeds = [sp["seed"] for sp in bench.rank_replica_specs(rank)]
    everyone = [None] * world
    dist.all_gather_object(everyone, seeds)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
    value = bench.job_value(ms, world, bench.N_REPLICAS, 100)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, f"rank{rank}.json"), "w") as f:
        json.dump({"seeds": everyone, "ms": ms, "value": value}, f)


def test_two_ranks_run_disjoint_batches_and_take_the_slowest_time(tmp_path):
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    mp.start_processes(_rank, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r in res:
        assert r["ms"] == 15.0  # the slower rank's time on both ranks
        assert r["value"] == pytest.approx(2 * 64 * 100 / 0.015)
    s0, s1 = res[0]["seeds"]
    assert len(s0) == len(s1) == 64 and not set(s0) & set(s1)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1", MASTER_PORT="29599")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "3", "--warmup", "3"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
