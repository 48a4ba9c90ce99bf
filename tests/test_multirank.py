"""The multi-rank side of bench.py on CPU: two gloo ranks on 127.0.0.1.

The codec has no exchange step (N GPUs run N independent replicas), so the
only cross-rank logic is the timing reduction -- every rank reports the
slowest rank's time -- and rank 0 alone printing the result line."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


_WORKER = r"""
import os, sys, json
sys.path.insert(0, os.environ["BENCH_ROOT"])
import torch.distributed as dist
import bench
rank, world, _ = bench.dist_env()
dist.init_process_group("gloo")
got = bench.max_over_ranks(1.5 + rank, world, "cpu")
with open(os.path.join(os.environ["OUT_DIR"], f"rank{rank}.json"), "w") as f:
    json.dump({"rank": rank, "max": got}, f)
dist.destroy_process_group()
"""


def _launch(args, timeout=240, out_dir=""):
    env = dict(os.environ, BENCH_ROOT=ROOT, OMP_NUM_THREADS="1", OUT_DIR=str(out_dir))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port())] + args
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def test_max_over_ranks_gloo(tmp_path):
    worker = tmp_path / "worker.py"
    worker.write_text(_WORKER)
    p = _launch([str(worker)], out_dir=tmp_path)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in (0, 1)]
    assert [l["rank"] for l in lines] == [0, 1]
    assert all(l["max"] == 2.5 for l in lines)  # both ranks see the slower one


def test_max_over_ranks_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25


def test_reference_arm_two_ranks():
    """`bench.py --impl reference` under torchrun: rank 0 alone times the CPU
    codec and prints the one JSON line; rank 1 exits 0 without work."""
    pytest.importorskip("torch")
    p = _launch(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
                 "--edge", "64"])
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(l) for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["cores"] >= 1
