"""Shared fixtures.  `-m "not gpu"` runs on any machine; `-m gpu` needs a
CUDA device and the built libgzfp.so."""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA codec")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as o
    o.build_port()
    return o


@pytest.fixture(scope="session")
def ref(orc):
    if not orc.ref_available():
        orc.build_ref()
    if not orc.ref_available():
        pytest.skip("reference zfp build not available (no reference tree on this machine)")
    return orc


HOSTCODEC_SRC = os.path.join(ROOT, "tests", "hostcodec", "host_codec.cpp")
HOSTCODEC_LIB = os.path.join(ROOT, "tests", "_build", "libhostcodec.so")


@pytest.fixture(scope="session")
def hostcodec():
    """Host build of the kernels' per-thread code (see host_codec.cpp)."""
    import ctypes
    srcs = [HOSTCODEC_SRC] + [os.path.join(ROOT, "cuzfp_gb300", "csrc", f)
                              for f in ("gzfp_block.cuh", "gzfp_array.cuh")]
    if (not os.path.exists(HOSTCODEC_LIB)
            or max(os.path.getmtime(s) for s in srcs) > os.path.getmtime(HOSTCODEC_LIB)):
        os.makedirs(os.path.dirname(HOSTCODEC_LIB), exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wno-unknown-pragmas",
                        "-o", HOSTCODEC_LIB, HOSTCODEC_SRC], check=True)
    lib = ctypes.CDLL(HOSTCODEC_LIB)
    A = [ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_double]
    lib.hc_compress.restype = ctypes.c_size_t
    lib.hc_compress.argtypes = A + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.hc_decompress.restype = ctypes.c_int
    lib.hc_decompress.argtypes = A + [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    S = [ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint] + [ctypes.c_longlong] * 3 + \
        [ctypes.c_double]
    lib.hc_compress_strided.restype = ctypes.c_size_t
    lib.hc_compress_strided.argtypes = S + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.hc_decompress_strided.restype = ctypes.c_size_t
    lib.hc_decompress_strided.argtypes = S + [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.hc_compress_aligned.restype = ctypes.c_size_t
    lib.hc_compress_aligned.argtypes = A + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    G = [ctypes.c_int] + [ctypes.c_uint] * 6 + [ctypes.c_int]  # type, dims, zfp parameters
    for fn in (lib.hc_block_offsets, lib.hc_compress_params, lib.hc_decompress_params):
        fn.restype = ctypes.c_uint64
    lib.hc_block_offsets.argtypes = G + [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.hc_compress_params.argtypes = G + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.hc_decompress_params.argtypes = G + [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    return lib


@pytest.fixture(scope="session")
def gz():
    """The product package (CUDA codec through its C ABI)."""
    import cuzfp_gb300
    return cuzfp_gb300


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
