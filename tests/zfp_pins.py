"""Known-answer pins from the reference's zfp regression test
(zfp-0.5.0/tests/testzfp.cpp, TEST_SIZE 4).

The test's input fields (precomputed in zfp-0.5.0/tests/fields.c) are
regenerated here from the generator the test itself uses for its larger
sizes (the polynomial of testzfp.cpp:34-43 sampled as in :47-72); the
checksums below, copied from testzfp.cpp:475-486, prove that the arrays are
identical to the fixture.
"""
from __future__ import annotations

import math

import numpy as np

# Jenkins one-at-a-time hashes of the input fields (testzfp.cpp:475-486)
CHECKSUM = {
    "float32": (0xdad6fd69, 0x000f8df1, 0x60993f48),
    "float64": (0x8d95b1fd, 0x96a0e601, 0x66e77c83),
}

# fixed-rate max-error bounds (testzfp.cpp:498-509); rates are 2, 8, 32 for
# float and 1, 4, 16, 64 for double (:494); the double table lists three
# values per row, so its fourth entry (rate 64) is zero
EMAX = {
    "float32": ((1.998e+00, 7.767e-03, 0.000e+00),
                (2.356e-01, 3.939e-04, 7.451e-09),
                (2.479e-01, 1.525e-03, 7.451e-08)),
    "float64": ((1.998e+00, 9.976e-01, 1.360e-05, 0.0),
                (2.944e+00, 2.491e-02, 2.578e-06, 0.0),
                (6.103e-01, 3.253e-02, 6.467e-06, 0.0)),
}


def jenkins(data: bytes) -> int:
    h = 0
    for c in data:
        h = (h + c) & 0xFFFFFFFF
        h = (h + (h << 10)) & 0xFFFFFFFF
        h ^= h >> 6
    h = (h + (h << 3)) & 0xFFFFFFFF
    h ^= h >> 11
    h = (h + (h << 15)) & 0xFFFFFFFF
    return h


def _poly(x, dt):
    # x - 3 x^2 + 4 x^4 evaluated as x + x^2 (4 x^2 - 3), each step rounded
    x = dt(x)
    xx = dt(x * x)
    yy = dt(dt(4) * xx - dt(3))
    return dt(x + dt(xx * yy))


def field(dt, d: int, m: int = 4) -> np.ndarray:
    """The m^6-value test field for dimensionality d (C order, x fastest)."""
    dt = np.dtype(dt).type
    n = m ** 6
    nx, ny, nz = {1: (n, 1, 1), 2: (m ** 3, m ** 3, 1), 3: (m * m, m * m, m * m)}[d]

    def axis(k):
        c = np.array([dt(dt(2 * i - k + 1) / dt(k)) for i in range(k)], dtype=dt)
        return np.array([_poly(v, dt) for v in c], dtype=dt) if k > 1 else np.ones(1, dt)

    fx, fy, fz = axis(nx), axis(ny), axis(nz)
    # (fx * fy) * fz, each product rounded to the field type
    out = (fx[None, None, :] * fy[None, :, None]).astype(dt) * fz[:, None, None]
    out = out.astype(dt)
    shape = {1: (nx,), 2: (ny, nx), 3: (nz, ny, nx)}[d]
    return out.reshape(shape)


def rate_pins(dt, d: int):
    name = np.dtype(dt).name
    rates = (2, 8, 32) if name == "float32" else (1, 4, 16, 64)
    return list(zip(rates, EMAX[name][d - 1]))


def expected_bytes(rate: float, n: int) -> int:
    """testzfp.cpp:124-128: compressed size equals rate * n / 8 bytes."""
    return int(math.floor(rate * n / 8 + 0.5))
