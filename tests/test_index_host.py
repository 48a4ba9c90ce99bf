"""The parallel index's host step (gzfp_index_host.h: following the true
chain of block starts through the walkers' merges), built for the host
with g++ and run inside a CPU model of the whole index on synthetic
streams: the assembled offsets are the true chain, and chains that cannot
be joined are refused.  CPU only."""
from __future__ import annotations

import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_index_model(tmp_path):
    exe = str(tmp_path / "index_model")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "cuzfp_gb300", "csrc"),
                    "-o", exe, os.path.join(ROOT, "tests", "cpp", "index_model.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
