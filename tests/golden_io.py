"""Golden fixtures made by the reference's own zfp 0.5.0 build
(tests/golden/make_golden.py).

Two kinds of case live in tests/golden:
* small_cases.npz -- full input, stream and decompressed output arrays;
* manifest.json   -- inputs regenerated from a named seeded generator,
  with SHA-256 digests of the input bytes, the reference stream and the
  reference output.
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

from tests import zfp_pins

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def generate(spec: dict) -> np.ndarray:
    """Rebuild a manifest input from its generator spec."""
    from cuzfp_gb300 import synth  # noqa: deferred, pure numpy
    kind = spec["gen"]
    dt = np.dtype(spec["dtype"])
    if kind == "testzfp":
        return zfp_pins.field(dt, spec["dims"])
    if kind == "smooth_noisy_3d":
        return synth.smooth_noisy_3d(spec["n"], spec["seed"], dt)
    if kind == "sinusoids":
        return synth.sinusoids(tuple(spec["shape"]), spec["count"], spec["kmax"], spec["seed"], dt)
    if kind == "random_walk":
        return synth.random_walk(spec["n"], spec["seed"], dt)
    raise ValueError(kind)


def manifest() -> list[dict]:
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)["cases"]


def small_cases(fname: str = "small_cases.npz") -> list[dict]:
    z = np.load(os.path.join(GOLDEN, fname))
    names = sorted({k.rsplit("__", 1)[0] for k in z.files})
    out = []
    for nm in names:
        out.append({"name": nm, "input": z[nm + "__input"], "stream": z[nm + "__stream"],
                    "output": z[nm + "__output"], "rate": float(z[nm + "__rate"])})
    return out


def load_all() -> list[dict]:
    """Full-array golden cases: the small floating-point ones and the
    integer ones (int_cases.npz)."""
    return small_cases() + small_cases("int_cases.npz")


def headed_cases() -> list[dict]:
    """Streams that start with zfp's full header (headed_cases.npz)."""
    return small_cases("headed_cases.npz")


def mode_cases() -> list[dict]:
    """Streams of zfp's other modes (mode_cases.npz): each case carries its
    (minbits, maxbits, maxprec, minexp)."""
    z = np.load(os.path.join(GOLDEN, "mode_cases.npz"))
    names = sorted({k.rsplit("__", 1)[0] for k in z.files})
    return [{"name": nm, "input": z[nm + "__input"], "stream": z[nm + "__stream"],
             "output": z[nm + "__output"], "params": tuple(int(v) for v in z[nm + "__params"])}
            for nm in names]
