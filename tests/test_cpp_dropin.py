"""A C++ program written against the cuZFP header interface (include/cuZFP.h)
compiles unchanged, links to libgzfp.so and passes cuZFP's own sanity
round trips."""
from __future__ import annotations

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "sanity.cpp")
EXE = os.path.join(ROOT, "tests", "_build", "cuzfp_sanity")


def build_exe():
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    cuda = "/usr/local/cuda"
    lib_dir = os.path.join(ROOT, "cuzfp_gb300")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    "-I" + cuda + "/include", SRC, "-o", EXE, "-L" + lib_dir, "-lgzfp",
                    "-L" + cuda + "/lib64", "-lcudart", "-Wl,-rpath," + lib_dir,
                    "-Wl,-rpath," + cuda + "/lib64"], check=True)


def test_dropin_header_compiles(gz):
    build_exe()
    assert os.path.exists(EXE)


@pytest.mark.gpu
def test_dropin_sanity_roundtrips(gz, cuda):
    build_exe()
    r = subprocess.run([EXE], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
