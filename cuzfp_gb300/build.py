"""Build libgzfp.so (the CUDA codec and its C ABI) in-tree for sm_103a.

Each translation unit under csrc/ is compiled by nvcc in parallel, then
linked into cuzfp_gb300/libgzfp.so.  Objects go to cuzfp_gb300/_build/.
A unit is rebuilt when it or any header under csrc/ or include/ is newer
than its object.  The units in RDC_UNITS launch kernels from the device and
are compiled as relocatable device code; the link then runs the device
linker and adds the CUDA device runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgzfp.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I" + CSRC, "-I" + INCLUDE]
RDC_UNITS = {"gzfp_serve_queue.cu", "gzfp_serve_req_f32.cu", "gzfp_serve_req_f64.cu",
             "gzfp_serve_req_i32.cu", "gzfp_serve_req_i64.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgzfp.so")


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj: str, src: str, newest_header: float) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or newest_header > t


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link libgzfp.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    srcs = _sources()
    newest = max((os.path.getmtime(h) for h in _headers()), default=0.0)
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, s, newest):
            todo.append((s, o))

    def compile_one(so):
        s, o = so
        rdc = ["-rdc=true"] if os.path.basename(s) in RDC_UNITS else []
        cmd = [cc] + NVCC_FLAGS + rdc + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(s)}:\n{r.stdout}\n{r.stderr}")
        return o

    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(compile_one, todo))
    if todo or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [cc] + ARCH + ["-shared", "-rdc=true", "-o", tmp] + objs + ["-lcudadevrt"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
