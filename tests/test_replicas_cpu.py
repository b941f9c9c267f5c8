"""Multi-GPU form (replicas): one process per GPU, its own seed, no data exchange, the
job's time the slowest rank's. Checked here with world_size-2 gloo process groups on
CPU, and with the benchmark's reference arm under torchrun (rank 0 alone works)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    from petrichor_gb300 import replicas
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    secs = [0.75, 1.25][rank]
    job = replicas.max_over_ranks(secs, dist)
    seed = replicas.replica_seed(1, rank)
    seeds = [None] * world
    dist.all_gather_object(seeds, seed)
    value = replicas.job_throughput(world, 1000.0, job)
    dist.destroy_process_group()
    with open(os.path.join(out, f"rank{rank}.json"), "w") as f:
        json.dump({"job": job, "seeds": seeds, "value": value}, f)


def test_replica_bookkeeping_over_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r in res:
        assert r["job"] == 1.25              # the slowest rank's time
        assert r["seeds"] == [1, 2]          # distinct streams per replica
        assert r["value"] == 2 * 1000.0 / 1.25


def test_reference_arm_runs_on_rank_zero_only():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={port}", os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--small",
           "--ref-seconds", "0.05"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
