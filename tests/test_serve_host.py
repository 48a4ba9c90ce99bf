"""The request server's host-side output arena (gzfp_arena.h), built for
the host with g++ and checked against an interval model on randomised
alloc / release sequences: first fit, alignment, no overlap, refusals only
when no gap fits, peak accounting and full merging.  CPU only."""
from __future__ import annotations

import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_arena_against_model(tmp_path):
    exe = str(tmp_path / "arena_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "cuzfp_gb300", "csrc"),
                    "-o", exe, os.path.join(ROOT, "tests", "cpp", "arena_check.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
