"""The N > 1 host paths of bench.py on CPU: gloo ranks (world size 2) for the whole-job reduction,
and the reference arm under torch.distributed.run (rank 0 alone prints one JSON line)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench

    out[rank] = bench.job_totals(dist, 1.0 + rank, 10.0 * (rank + 1), 3.0)
    dist.destroy_process_group()


def test_job_totals_take_max_time_and_summed_counts_over_gloo_ranks():
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, free_port(), out), nprocs=2, join=True)
        assert out[0] == out[1] == (2.0, 30.0, 6.0)


def test_job_totals_without_a_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.job_totals(None, 1.5, 2.0) == (1.5, 2.0)


def test_reference_arm_under_torchrun_prints_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--workload", "cornell256",
           "--ref-seconds", "1"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["metric"] == "segments/s" and rec["value"] > 0
    assert rec["e2e"]["h2d_bytes_per_step"] == 0 and rec["cpu_baseline"]["kind"] == "port"
