"""A C++ program written against the cuZFP header interface (include/cuZFP.h)
compiles unchanged, links to libgzfp.so and passes cuZFP's own sanity
round trips; a plain C program drives the C ABI (include/gzfp.h)."""
from __future__ import annotations

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "sanity.cpp")
EXE = os.path.join(ROOT, "tests", "_build", "cuzfp_sanity")
C_SRC = os.path.join(ROOT, "tests", "cpp", "c_abi.c")
C_EXE = os.path.join(ROOT, "tests", "_build", "gzfp_c_abi")


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


def build_c_exe():
    os.makedirs(os.path.dirname(C_EXE), exist_ok=True)
    lib_dir = os.path.join(ROOT, "cuzfp_gb300")
    subprocess.run(["gcc", "-std=c99", "-O1", "-Wall", "-I" + os.path.join(ROOT, "include"),
                    C_SRC, "-o", C_EXE, "-L" + lib_dir, "-lgzfp", "-lm",
                    "-Wl,-rpath," + lib_dir], check=True)


def test_c_caller_compiles(gz):
    build_c_exe()
    assert os.path.exists(C_EXE)


@pytest.mark.gpu
def test_c_caller_runs(gz, cuda):
    build_c_exe()
    r = subprocess.run([C_EXE], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
