"""The N > 1 host path of bench.py on CPU (gloo, world size 2): each rank
steps its own replicas (no collective on the data path), the job rate sums
the ranks' beads over the slowest rank's time, and the reference arm prints
one line from rank 0 only."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    nbeads = 1000 * (rank + 1)          # uneven shards
    t_ms = 10.0 * (rank + 1)            # rank 1 is the slowest
    value, t_max, beads = bench.job_rate(nbeads, 96, 5, t_ms, world)
    out[rank] = (value, t_max, beads)
    dist.barrier()
    dist.destroy_process_group()


def test_job_rate_sums_beads_over_slowest_rank():
    port = free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for rank in (0, 1):
        value, t_max, beads = out[rank]
        assert beads == 3000 and t_max == 20.0
        assert value == pytest.approx(3000 * 96 * 5 / 0.020)


def test_ranks_shard_distinct_replica_batches():
    # rank k steps config 4 drawn with seed 4 + 1000 k: same shape, other chains
    from xmd_gb300 import synth
    lens0 = synth.c4_lengths(seed=4, count=256)
    lens1 = synth.c4_lengths(seed=4 + 1000, count=256)
    assert len(lens0) == len(lens1) == 256 and not (lens0 == lens1).all()


def test_reference_arm_prints_once_under_torchrun():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--md-steps", "1"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=str(ROOT))
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, res.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0
    assert rec["cpu_baseline"]["cores"] >= 1 and rec["e2e"]["h2d_bytes_per_step"] == 0
    # the CPU arm maps the oracle's library only, never the engine's
    assert rec["libraries_loaded"] == ["liboracle.so"], rec["libraries_loaded"]
    # the same config as the engine arm would report for these arguments
    import bench
    assert rec["config"] == bench.workload_config(rec["config"]["beads_per_gpu"], 256, 1, 3, 1)
