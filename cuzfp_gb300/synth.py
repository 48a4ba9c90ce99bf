"""Seeded synthetic fields for tests and benchmarks.

The reference publishes no dataset for this path; these generators stand in
for it with the shapes, sizes and value distributions of the workloads the
codec is measured on.  Fields are built in float64 (numpy PCG64 for all
random draws) and cast to the target dtype.  The device variants evaluate
the same formulas with torch on a CUDA device for the large cases.
"""
from __future__ import annotations

import math

import numpy as np


def smooth_noisy_3d(n: int = 64, seed: int = 0, dtype=np.float32) -> np.ndarray:
    """f = sin(x/8) cos(y/5) + 0.5 sin((x+z)/11) + N(0, 1e-3), on n^3 points."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    f = np.sin(x / 8.0) * np.cos(y / 5.0) + 0.5 * np.sin((x + z) / 11.0)
    f = f + rng.normal(0.0, 1e-3, size=f.shape)
    return f.astype(dtype)


def _waves(rng: np.random.Generator, dims: int, count: int, kmax: int):
    """Integer wavevectors with |k| uniform in [1, kmax], amplitude 1/|k|^2,
    uniform phases."""
    waves = []
    while len(waves) < count:
        mag = rng.uniform(1.0, kmax)
        d = rng.normal(size=dims)
        d /= np.linalg.norm(d)
        k = np.rint(d * mag).astype(np.int64)
        kk = float(np.sqrt((k * k).sum()))
        if kk == 0.0:
            continue
        waves.append((k, 1.0 / (kk * kk), rng.uniform(0.0, 2.0 * math.pi)))
    return waves


def sinusoids(shape, count: int = 16, kmax: int = 32, seed: int = 0,
              dtype=np.float64) -> np.ndarray:
    """Sum of `count` random-phase sinusoids over a C-ordered grid of `shape`
    (1-3 dims); each axis spans one period of the unit wavevector."""
    rng = np.random.default_rng(seed)
    dims = len(shape)
    out = np.zeros(shape, np.float64)
    axes = [np.arange(n, dtype=np.float64) / n for n in shape]
    for k, amp, ph in _waves(rng, dims, count, kmax):
        # sin(sum_i 2 pi k_i x_i + ph) as the imaginary part of a separable
        # product of per-axis phasors
        term = np.exp(1j * ph) * np.ones((1,) * dims, np.complex128)
        for i in range(dims):
            shp = [1] * dims
            shp[i] = shape[i]
            term = term * np.exp(2j * math.pi * k[i] * axes[i]).reshape(shp)
        out += amp * term.imag
    return out.astype(dtype)


def sinusoids_device(shape, count: int = 16, kmax: int = 32, seed: int = 0,
                     dtype=None, device: str = "cuda"):
    """`sinusoids` evaluated with torch on `device` (same waves and formula)."""
    import torch
    dtype = dtype or torch.float64
    rng = np.random.default_rng(seed)
    dims = len(shape)
    out = torch.zeros(shape, dtype=torch.float64, device=device)
    for k, amp, ph in _waves(rng, dims, count, kmax):
        term = torch.full((1,) * dims, complex(math.cos(ph), math.sin(ph)),
                          dtype=torch.complex128, device=device)
        for i in range(dims):
            shp = [1] * dims
            shp[i] = shape[i]
            x = torch.arange(shape[i], dtype=torch.float64, device=device) / shape[i]
            term = term * torch.polar(torch.ones_like(x), 2 * math.pi * float(k[i]) * x).reshape(shp)
        out += amp * term.imag
    return out.to(dtype)


def random_walk(n: int, seed: int = 0, dtype=np.float32) -> np.ndarray:
    """Cumulative sum of N(0, 1) steps."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.standard_normal(n)).astype(dtype)


def random_walk_device(n: int, seed: int = 0, dtype=None, device: str = "cuda"):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    steps = torch.randn(n, generator=g, dtype=torch.float64, device=device)
    return torch.cumsum(steps, 0).to(dtype or torch.float32)


def error_stats(orig: np.ndarray, dec: np.ndarray) -> dict:
    """Rate-distortion figures against the float64 original (max abs error,
    RMSE, PSNR), as printed by the zfp tool (zfp-0.5.0/utils/zfp.c:29-57)."""
    o = orig.astype(np.float64).ravel()
    d = dec.astype(np.float64).ravel()
    err = d - o
    mse = float(np.mean(err * err)) if o.size else 0.0
    rng = float(o.max() - o.min()) if o.size else 0.0
    rmse = math.sqrt(mse)
    psnr = 20 * math.log10(rng / (2 * rmse)) if rmse > 0 and rng > 0 else float("inf")
    return {"maxe": float(np.max(np.abs(err))) if o.size else 0.0, "rmse": rmse, "psnr": psnr}
