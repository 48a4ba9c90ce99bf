"""Host-side logic of the library, built with g++ on its own (CUDA-free
headers) and checked by C++ programs under tests/cpp against models or
properties.  CPU only.

* the request server's output arena (gzfp_arena.h) against an interval
  model: first fit, alignment, no overlap, refusals only when no gap fits,
  peak accounting, full merging;
* the parallel index's host step (gzfp_index_host.h) inside a CPU model of
  the whole index on synthetic streams: the assembled offsets are the true
  chain, and chains that cannot be joined are refused;
* the host-staged calls' slab decomposition (gzfp_slabs.h) over 20,000
  random shapes, bit budgets and scalar sizes: slabs tile the layers,
  planes and stream words exactly, start on stream words, and stay within
  the size target."""
from __future__ import annotations

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("program", ["arena_check", "index_model", "slabs_check"])
def test_host_logic(tmp_path, program):
    exe = str(tmp_path / program)
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Werror", "-Wno-unknown-pragmas",
                    "-I", os.path.join(ROOT, "cuzfp_gb300", "csrc"),
                    "-o", exe, os.path.join(ROOT, "tests", "cpp", program + ".cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
