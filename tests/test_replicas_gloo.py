"""Multi-GPU runs are independent replicas (no collective on the data path):
the bench's rank handling, max-over-ranks and single-line output, exercised on
CPU with two gloo ranks through the reference arm (the oracle), which runs on
rank 0 only."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun_prints_one_line(tmp_path):
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "0", "--grid", "64", "--cpu-budget", "2"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=str(tmp_path), env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"


def test_allmax_over_gloo_ranks(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "allmax.py"
    script.write_text(
        "import os, sys\n"
        f"sys.path.insert(0, {str(ROOT)!r})\n"
        "import bench\n"
        "world, rank, local = bench.dist_setup('gloo')\n"
        "v = bench.allmax(world, float(rank + 1))\n"
        "bench.barrier(world)\n"
        "sys.stdout.write(f'RANK {rank} {v}\\n')\n"
        "sys.stdout.flush()\n")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(script)]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    vals = sorted(l.split() for l in out.stdout.splitlines() if l.startswith("RANK"))
    assert [v[2] for v in vals] == ["2.0", "2.0"]
