"""Seeded parity cases shared by the CPU and GPU suites."""
from __future__ import annotations

import numpy as np

RATES = [0.5, 1, 2, 3.3, 4, 8, 12, 16, 17.7, 24, 32, 48, 64]


def random_case(rng: np.random.Generator, max_edge=(300, 40, 14)):
    """One random (array, rate) pair: 1-3 dims, ragged edges, f32/f64 and a
    mix of value distributions (smooth, rough, wide dynamic range, sparse,
    tiny magnitudes near the denormal range)."""
    dims = int(rng.integers(1, 4))
    dt = np.float32 if rng.random() < 0.5 else np.float64
    if dims == 1:
        shape = (int(rng.integers(1, max_edge[0])),)
    elif dims == 2:
        shape = tuple(int(v) for v in rng.integers(1, max_edge[1], 2))
    else:
        shape = tuple(int(v) for v in rng.integers(1, max_edge[2], 3))
    n = int(np.prod(shape))
    kind = int(rng.integers(0, 7))
    if kind == 0:
        a = rng.standard_normal(n)
    elif kind == 1:
        a = np.cumsum(rng.standard_normal(n))
    elif kind == 2:
        a = rng.standard_normal(n) * 10.0 ** rng.integers(-30, 30, n)
    elif kind == 3:
        a = np.where(rng.random(n) < 0.5, 0.0, rng.standard_normal(n))
    elif kind == 4:
        a = np.sin(np.arange(n) / 7.0) * 1e5
    elif kind == 5:
        a = rng.standard_normal(n) * (1e-300 if dt == np.float64 else 1e-40)
    else:
        a = np.where(rng.random(n) < 0.9, 0.0, rng.standard_normal(n) * 1e3)
    rate = float(rng.choice(RATES))
    return a.astype(dt).reshape(shape), rate


def edge_cases():
    """Hand-picked cases: empty-ish shapes, every edge remainder, all-zero
    blocks, signed zeros, denormals, extreme exponents, constant blocks."""
    out = []
    for dt in (np.float32, np.float64):
        for shape in [(1,), (2,), (3,), (4,), (5,), (7,), (1, 1), (1, 5), (5, 1), (3, 7),
                      (4, 4), (1, 1, 1), (1, 2, 3), (3, 2, 1), (4, 4, 4), (5, 6, 7), (9, 1, 9)]:
            n = int(np.prod(shape))
            base = (np.arange(n, dtype=np.float64) - n / 3).reshape(shape)
            out.append((base.astype(dt), 8.0))
        info = np.finfo(dt)
        out.append((np.zeros((8, 8, 8), dt), 16.0))
        out.append((np.full((4, 4, 4), -0.0, dt), 16.0))
        out.append((np.full((6, 6, 6), 1.0, dt), 4.0))
        den = np.arange(1, 65, dtype=np.float64).reshape(4, 4, 4)
        out.append(((den * float(info.smallest_subnormal)).astype(dt), 16.0))
        out.append(((den * float(info.tiny)).astype(dt), 16.0))
        out.append(((den / 64.0 * float(info.max)).astype(dt), 16.0))
        out.append(((-den / 64.0 * float(info.max)).astype(dt), 32.0))
        alt = np.where(np.arange(64) % 2 == 0, 1.0, -1.0).reshape(4, 4, 4) * float(info.max) / 2
        out.append((alt.astype(dt), 64.0))
        out.append(((np.arange(4096, dtype=np.float64) % 17).reshape(16, 16, 16).astype(dt), 2.0))
    return out


def has_saturating_blocks(a: np.ndarray) -> bool:
    """True if some block's largest magnitude m is in (0, 2^-98) (float) or
    (0, 2^-962) (double).  There zfp 0.5.0's scale factor 2^(P-2-emax)
    overflows to inf and its float->int cast is undefined in C: the oracle and
    the CUDA codec saturate (IEEE / AArch64 / CUDA semantics), an x86-64
    build of the reference returns INT_MIN instead, so such arrays are left
    out of oracle-versus-x86-reference comparisons only."""
    lim = 2.0 ** -98 if a.dtype == np.float32 else 2.0 ** -962
    m = np.abs(a.astype(np.float64))
    pad = [(0, (-s) % 4) for s in m.shape]
    m = np.pad(m, pad)
    shp = []
    for s in m.shape:
        shp += [s // 4, 4]
    m = m.reshape(shp)
    m = m.max(axis=tuple(range(1, 2 * a.ndim, 2)))
    return bool(np.any((m > 0) & (m < lim)))


def int_case(rng, max_edge=(300, 40, 14), whole_blocks=False, wide=False):
    """A random int32 / int64 array and rate: smooth walks and white noise,
    with magnitudes inside zfp's integer range (|v| < 2^(P-2)) unless
    `wide`, which draws from the whole type range (the codec wraps)."""
    dims = int(rng.integers(1, 4))
    if whole_blocks:
        shape = tuple(4 * int(rng.integers(1, max(2, max_edge[dims - 1] // 4))) for _ in range(dims))
    else:
        shape = tuple(int(rng.integers(1, max_edge[dims - 1] + 1)) for _ in range(dims))
    dt = np.int32 if rng.random() < 0.5 else np.int64
    bits = 32 if dt == np.int32 else 64
    n = int(np.prod(shape))
    kind = rng.integers(0, 3)
    if wide:
        info = np.iinfo(dt)
        a = rng.integers(info.min, info.max, n, dtype=dt, endpoint=True)
    elif kind == 0:  # white noise at a random scale
        lim = 1 << int(rng.integers(1, bits - 2))
        a = rng.integers(-lim, lim, n, dtype=np.int64)
    elif kind == 1:  # random walk
        step = 1 << int(rng.integers(0, bits // 2))
        a = np.cumsum(rng.integers(-step, step + 1, n, dtype=np.int64))
        a = np.clip(a, -(1 << (bits - 3)), (1 << (bits - 3)))
    else:  # mostly zero with a few spikes
        a = np.zeros(n, np.int64)
        idx = rng.integers(0, n, max(1, n // 50))
        a[idx] = rng.integers(-(1 << (bits - 3)), 1 << (bits - 3), idx.size)
    a = np.asarray(a).astype(dt).reshape(shape)
    rate = float(rng.choice([0.5, 1, 2.25, 4, 8, 12.5, 16, 24, 32, 48, 64]))
    return a, rate
