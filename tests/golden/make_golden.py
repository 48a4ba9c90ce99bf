"""Regenerate the golden fixtures from the reference's own zfp 0.5.0 build.

Run in a checkout that has the reference tree (the build reads its zfp
sources):  python tests/golden/make_golden.py [--ints | --headed | --modes]
Writes tests/golden/small_cases.npz, tests/golden/manifest.json,
tests/golden/int_cases.npz, tests/golden/headed_cases.npz and
tests/golden/mode_cases.npz (only one of the last three with a flag).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from tests import cases, golden_io  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def main() -> None:
    if not orc.build_ref():
        raise SystemExit("reference tree not found; cannot regenerate golden fixtures")
    # small cases, stored in full
    rng = np.random.default_rng(20261203)
    arrays = {}
    k = 0
    while k < 24:
        a, rate = cases.random_case(rng, max_edge=(200, 24, 10))
        if cases.has_saturating_blocks(a):
            continue
        s = orc.ref_compress(a, rate)
        d = orc.ref_decompress(s, a.shape, a.dtype, rate)
        nm = f"rand{k:02d}_{a.ndim}d_{a.dtype.name}"
        arrays[nm + "__input"] = a
        arrays[nm + "__stream"] = s
        arrays[nm + "__output"] = d
        arrays[nm + "__rate"] = np.array(rate)
        k += 1
    for i, (a, rate) in enumerate(cases.edge_cases()):
        if cases.has_saturating_blocks(a):
            continue
        s = orc.ref_compress(a, rate)
        d = orc.ref_decompress(s, a.shape, a.dtype, rate)
        nm = f"edge{i:02d}_{a.ndim}d_{a.dtype.name}"
        arrays[nm + "__input"] = a
        arrays[nm + "__stream"] = s
        arrays[nm + "__output"] = d
        arrays[nm + "__rate"] = np.array(rate)
    np.savez_compressed(os.path.join(OUT, "small_cases.npz"), **arrays)

    # generated cases, stored as digests
    specs = []
    for dt in ("float32", "float64"):
        for d in (1, 2, 3):
            rates = (2, 8, 32) if dt == "float32" else (1, 4, 16, 64)
            for r in rates:
                specs.append({"name": f"testzfp_{d}d_{dt}_r{r}", "gen": "testzfp", "dims": d,
                              "dtype": dt, "rate": r})
    specs.append({"name": "smooth_noisy_64cube_f32_r16", "gen": "smooth_noisy_3d", "n": 64,
                  "seed": 0, "dtype": "float32", "rate": 16})
    for r in (8, 16, 32):
        specs.append({"name": f"sinusoids_36cube_f64_r{r}", "gen": "sinusoids",
                      "shape": [36, 37, 38], "count": 16, "kmax": 32, "seed": 1,
                      "dtype": "float64", "rate": r})
    for r in (4, 12, 24):
        specs.append({"name": f"walk_1d_f32_r{r}", "gen": "random_walk", "n": 100003, "seed": 2,
                      "dtype": "float32", "rate": r})
        specs.append({"name": f"sinusoids_2d_f32_r{r}", "gen": "sinusoids", "shape": [253, 255],
                      "count": 8, "kmax": 64, "seed": 3, "dtype": "float32", "rate": r})
        specs.append({"name": f"sinusoids_2d_f64_r{r}", "gen": "sinusoids", "shape": [127, 126],
                      "count": 8, "kmax": 64, "seed": 4, "dtype": "float64", "rate": r})
    for sp in specs:
        a = golden_io.generate(sp)
        s = orc.ref_compress(a, sp["rate"])
        d = orc.ref_decompress(s, a.shape, a.dtype, sp["rate"])
        sp["shape_out"] = list(a.shape)
        sp["input_sha256"] = golden_io.sha(a)
        sp["stream_bytes"] = int(s.nbytes)
        sp["stream_sha256"] = golden_io.sha(s)
        sp["output_sha256"] = golden_io.sha(d)
    with open(os.path.join(OUT, "manifest.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "reference": "zfp 0.5.0 as vendored by cuZFP (src/thirdparty_builtin/zfp-0.5.0),"
                                " built by oracle/Makefile",
                   "cases": specs}, f, indent=1)
    print(f"{len([k for k in arrays if k.endswith('__rate')])} small cases, {len(specs)} manifest cases")


def write_int_cases() -> None:
    """Integer arrays of whole blocks, coded by the reference's per-block
    integer API (zfp 0.5.0's zfp_compress takes no integer fields), stored in
    full in tests/golden/int_cases.npz."""
    if not orc.build_ref():
        raise SystemExit("reference tree not found; cannot regenerate golden fixtures")
    rng = np.random.default_rng(20261204)
    arrays = {}
    k = 0
    while k < 24:
        a, rate = cases.int_case(rng, max_edge=(256, 32, 12), whole_blocks=True)
        if orc.stream_bytes(a.shape, a.dtype, rate) == 0:
            continue
        s = orc.ref_compress(a, rate)
        d = orc.ref_decompress(s, a.shape, a.dtype, rate)
        nm = f"int{k:02d}_{a.ndim}d_{a.dtype.name}"
        arrays[nm + "__input"] = a
        arrays[nm + "__stream"] = s
        arrays[nm + "__output"] = d
        arrays[nm + "__rate"] = np.array(rate)
        k += 1
    np.savez_compressed(os.path.join(OUT, "int_cases.npz"), **arrays)
    print(f"{k} integer cases")


def write_headed_cases() -> None:
    """Streams with zfp's full header in front (zfp_write_header with
    ZFP_HEADER_FULL, then zfp_compress on the same bit stream), one per
    scalar type and dimensionality plus the 64-bit mode form for doubles
    above 2048 bits per block, stored in full in tests/golden/headed_cases.npz."""
    if not orc.build_ref():
        raise SystemExit("reference tree not found; cannot regenerate golden fixtures")
    rng = np.random.default_rng(20261205)
    arrays = {}
    k = 0
    # integer arrays in whole blocks: the reference codes them block by block
    plan = [(dt, shape, rate)
            for dt in ("float32", "float64", "int32", "int64")
            for shape, rate in (((204 if dt.startswith("int") else 203,), 9.5),
                                ((20, 36), 6.0), ((12, 8, 16), 12.0))]
    plan += [("float64", (37, 21), 160.0), ("float64", (150,), 600.0),
             ("float32", (5, 6, 7), 3.0), ("float64", (9, 10, 11), 32.0)]
    for dt, shape, rate in plan:
        a = np.cumsum(rng.standard_normal(shape), axis=-1)
        a = (a * 4096).astype(dt) if dt.startswith("int") else a.astype(dt)
        s = orc.ref_compress_headed(a, rate)
        d = orc.ref_decompress_headed(s, a.shape, a.dtype, rate)
        nm = f"headed{k:02d}_{a.ndim}d_{a.dtype.name}"
        arrays[nm + "__input"] = a
        arrays[nm + "__stream"] = s
        arrays[nm + "__output"] = d
        arrays[nm + "__rate"] = np.array(rate)
        k += 1
    np.savez_compressed(os.path.join(OUT, "headed_cases.npz"), **arrays)
    print(f"{k} headed cases")


def write_mode_cases() -> None:
    """Streams of zfp's fixed-precision and fixed-accuracy modes and of
    other parameter sets (zfp_stream_set_precision / _accuracy / _params,
    then zfp_compress; integer arrays through the per-block API), stored in
    full in tests/golden/mode_cases.npz with their parameters."""
    if not orc.build_ref():
        raise SystemExit("reference tree not found; cannot regenerate golden fixtures")
    rng = np.random.default_rng(20261206)
    arrays = {}
    plan = []
    for dt in ("float32", "float64"):
        plan += [(dt, (203,), ("precision", 14)), (dt, (20, 36), ("accuracy", 1e-4)),
                 (dt, (12, 9, 16), ("precision", 30)), (dt, (10, 11, 13), ("accuracy", 1e-9))]
    for dt in ("int32", "int64"):
        plan += [(dt, (64,), ("precision", 20)), (dt, (8, 12, 16), ("params", (64, 900, 48, -1074)))]
    plan += [("float64", (33, 17), ("params", (100, 700, 40, -40)))]
    for k, (dt, shape, (kind, v)) in enumerate(plan):
        a = np.cumsum(rng.standard_normal(shape), axis=-1)
        a = (a * 4096).astype(dt) if dt.startswith("int") else a.astype(dt)
        pr = (orc.mode_precision(a.dtype, v, lib=orc.ref()) if kind == "precision" else
              orc.mode_accuracy(a.dtype, v, lib=orc.ref()) if kind == "accuracy" else v)
        s = orc.ref_compress_params(a, pr)
        d = orc.ref_decompress_params(s, a.shape, a.dtype, pr)
        nm = f"mode{k:02d}_{kind}_{a.ndim}d_{a.dtype.name}"
        arrays[nm + "__input"] = a
        arrays[nm + "__stream"] = s
        arrays[nm + "__output"] = d
        arrays[nm + "__params"] = np.array(pr, np.int64)
    np.savez_compressed(os.path.join(OUT, "mode_cases.npz"), **arrays)
    print(f"{len(plan)} mode cases")


if __name__ == "__main__":
    if sys.argv[1:] == ["--ints"]:
        write_int_cases()
    elif sys.argv[1:] == ["--headed"]:
        write_headed_cases()
    elif sys.argv[1:] == ["--modes"]:
        write_mode_cases()
    else:
        main()
        write_int_cases()
        write_headed_cases()
        write_mode_cases()
