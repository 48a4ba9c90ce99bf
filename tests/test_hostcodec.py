"""The kernels' per-thread code (gzfp_block.cuh / gzfp_array.cuh), built
for the host, against the oracle and the golden fixtures.  CPU only; the
same source runs on the GPU in the `gpu` tests."""
from __future__ import annotations

import numpy as np

from tests import cases, golden_io


def hc_compress(lib, orc, a, rate):
    nx, ny, nz = orc.dims3(a.shape)
    n = orc.stream_bytes(a.shape, a.dtype, rate)
    out = np.zeros(max(n // 8, 1), np.uint64)
    got = lib.hc_compress(orc.type_code(a.dtype), nx, ny, nz, float(rate), a.ctypes.data,
                          out.ctypes.data, out.nbytes)
    assert got == n
    return out[: n // 8]


def hc_decompress(lib, orc, s, shape, dtype, rate):
    out = np.zeros(shape, dtype)
    nx, ny, nz = orc.dims3(shape)
    assert lib.hc_decompress(orc.type_code(dtype), nx, ny, nz, float(rate), s.ctypes.data,
                             s.nbytes, out.ctypes.data)
    return out


def test_random_cases(hostcodec, orc):
    rng = np.random.default_rng(99)
    for _ in range(500):
        a, rate = cases.random_case(rng)
        s = orc.compress(a, rate)
        assert np.array_equal(hc_compress(hostcodec, orc, a, rate), s), (a.shape, a.dtype, rate)
        d = orc.decompress(s, a.shape, a.dtype, rate)
        h = hc_decompress(hostcodec, orc, s, a.shape, a.dtype, rate)
        assert np.array_equal(d.view(np.uint8), h.view(np.uint8)), (a.shape, a.dtype, rate)


def test_edge_cases(hostcodec, orc):
    for a, rate in cases.edge_cases():
        s = orc.compress(a, rate)
        assert np.array_equal(hc_compress(hostcodec, orc, a, rate), s), (a.shape, a.dtype, rate)
        h = hc_decompress(hostcodec, orc, s, a.shape, a.dtype, rate)
        d = orc.decompress(s, a.shape, a.dtype, rate)
        assert np.array_equal(d.view(np.uint8), h.view(np.uint8))


def test_arbitrary_streams(hostcodec, orc):
    rng = np.random.default_rng(11)
    for shape in ((64,), (13, 9), (8, 7, 6)):
        for dt in (np.float32, np.float64):
            for rate in (1, 2.5, 8, 16, 33):
                n = orc.stream_bytes(shape, dt, rate) // 8
                w = rng.integers(0, 2 ** 63, n, dtype=np.int64).astype(np.uint64) << np.uint64(1)
                w |= rng.integers(0, 2, n, dtype=np.int64).astype(np.uint64)
                d = orc.decompress(w, shape, dt, rate)
                h = hc_decompress(hostcodec, orc, w, shape, dt, rate)
                assert np.array_equal(d.view(np.uint8), h.view(np.uint8)), (shape, dt, rate)


def test_golden(hostcodec, orc):
    for c in golden_io.load_all():
        a = c["input"]
        assert np.array_equal(hc_compress(hostcodec, orc, a, c["rate"]), c["stream"]), c["name"]
        h = hc_decompress(hostcodec, orc, c["stream"], a.shape, a.dtype, c["rate"])
        assert np.array_equal(h.view(np.uint8), c["output"].view(np.uint8)), c["name"]


def test_full_planes_on_noise(hostcodec, orc):
    """White noise makes every coefficient significant within a few planes,
    so blocks code many 64-bit verbatim planes, some starting exactly on a
    word boundary of the stream."""
    rng = np.random.default_rng(5)
    for shape, dt in (((40, 40, 40), np.float64), ((36, 44, 40), np.float32),
                      ((200, 204), np.float64), ((40000,), np.float64)):
        a = rng.standard_normal(shape).astype(dt)
        for rate in (24, 32, 41.5, 64):
            s = orc.compress(a, rate)
            assert np.array_equal(hc_compress(hostcodec, orc, a, rate), s), (shape, dt, rate)
            d = orc.decompress(s, a.shape, a.dtype, rate)
            h = hc_decompress(hostcodec, orc, s, a.shape, a.dtype, rate)
            assert np.array_equal(d.view(np.uint8), h.view(np.uint8)), (shape, dt, rate)


def test_integer_fields(hostcodec, orc):
    """int32 / int64 arrays of every dimensionality, ragged shapes and rates,
    including values across the whole type range (the lifting wraps)."""
    rng = np.random.default_rng(23)
    for i in range(300):
        a, rate = cases.int_case(rng, wide=(i % 10 == 9))
        if orc.stream_bytes(a.shape, a.dtype, rate) == 0:
            continue  # a rate of 0 bits per block is not a stream
        s = orc.compress(a, rate)
        assert np.array_equal(hc_compress(hostcodec, orc, a, rate), s), (a.shape, a.dtype, rate)
        d = orc.decompress(s, a.shape, a.dtype, rate)
        h = hc_decompress(hostcodec, orc, s, a.shape, a.dtype, rate)
        assert np.array_equal(d, h), (a.shape, a.dtype, rate)


def test_block_offsets_general_modes(hostcodec, orc):
    """The kernels' block-length parse (what the device index walks), run on
    the host over oracle streams of zfp's fixed-precision and
    fixed-accuracy modes: every block's start bit equals the oracle
    compressor's, for all four scalar types and 1D / 2D / 3D."""
    rng = np.random.default_rng(31)
    shapes = ((1000,), (37, 29), (13, 11, 10))
    for dt in (np.float32, np.float64, np.int32, np.int64):
        for shape in shapes:
            a = np.cumsum(rng.standard_normal(int(np.prod(shape)))).reshape(shape)
            a = (a * 5000).astype(dt) if np.dtype(dt).kind == "i" else a.astype(dt)
            modes = [orc.mode_precision(dt, p) for p in (5, 16, 40)]
            if np.dtype(dt).kind == "f":
                modes += [orc.mode_accuracy(dt, t) for t in (1e-1, 1e-4, 1e-9)]
            for params in modes:
                s, offs = orc.compress_params(a, params, with_offsets=True)
                s = np.ascontiguousarray(s)
                nx, ny, nz = orc.dims3(shape)
                got = np.zeros(offs.size, np.uint64)
                end = hostcodec.hc_block_offsets(orc.type_code(dt), nx, ny, nz, *params,
                                                 s.ctypes.data, s.nbytes, got.ctypes.data)
                assert np.array_equal(got, offs), (dt, shape, params)
                assert end <= s.nbytes * 8, (dt, shape, params)


def test_general_modes_against_oracle(hostcodec, orc):
    """The mode kernels' per-block code (encode_block_mode /
    decode_block_mode), run on the host block after block: the stream of
    zfp's fixed-precision and fixed-accuracy modes and its decoded array are
    the oracle's bit for bit, for all four scalar types and 1D / 2D / 3D,
    edge blocks included."""
    rng = np.random.default_rng(32)
    shapes = ((997,), (37, 29), (13, 11, 10))
    for dt in (np.float32, np.float64, np.int32, np.int64):
        for shape in shapes:
            a = np.cumsum(rng.standard_normal(int(np.prod(shape)))).reshape(shape)
            a = (a * 5000).astype(dt) if np.dtype(dt).kind == "i" else a.astype(dt)
            modes = [orc.mode_precision(dt, p) for p in (3, 16, 40)]
            if np.dtype(dt).kind == "f":
                modes += [orc.mode_accuracy(dt, t) for t in (1e-1, 1e-4, 1e-9)]
            nx, ny, nz = orc.dims3(shape)
            t = orc.type_code(dt)
            for params in modes:
                s = orc.compress_params(a, params)
                cap = int(orc.port().gzo_bound_params(t, nx, ny, nz, *params)) + 16
                buf = np.zeros(cap // 8 + 1, np.uint64)
                bits = hostcodec.hc_compress_params(t, nx, ny, nz, *params, a.ctypes.data,
                                                    buf.ctypes.data, buf.nbytes)
                assert (bits + 63) // 64 == s.size, (dt, shape, params, bits, s.size)
                assert np.array_equal(buf[: s.size], s), (dt, shape, params)
                s = np.ascontiguousarray(s)
                out = np.zeros(shape, dt)
                used = hostcodec.hc_decompress_params(t, nx, ny, nz, *params, s.ctypes.data,
                                                      s.nbytes, out.ctypes.data)
                assert used == bits, (dt, shape, params)
                ref = orc.decompress_params(s, shape, dt, params)
                assert np.array_equal(out.view(np.uint8), ref.view(np.uint8)), (dt, shape, params)


def test_aligned_writer(hostcodec, orc):
    """The encoder's aligned writer (what the GPU kernels use for blocks of
    whole 64-bit words: every word stored, none merged), run on the host
    into a buffer of ones: the stream is the oracle's, so every word is
    written in full."""
    rng = np.random.default_rng(33)
    for dt in (np.float32, np.float64, np.int32, np.int64):
        for shape, rates in (((1003,), (16, 32, 48)), ((37, 29), (4, 8, 12)),
                             ((13, 11, 10), (1, 2, 8, 16))):
            a = np.cumsum(rng.standard_normal(int(np.prod(shape)))).reshape(shape)
            a = (a * 5000).astype(dt) if np.dtype(dt).kind == "i" else a.astype(dt)
            nx, ny, nz = orc.dims3(shape)
            for rate in rates:
                s = orc.compress(a, rate)
                out = np.zeros(s.size + 1, np.uint64)
                n = hostcodec.hc_compress_aligned(orc.type_code(dt), nx, ny, nz, float(rate),
                                                  a.ctypes.data, out.ctypes.data, out.nbytes)
                assert n == s.nbytes, (dt, shape, rate, n, s.nbytes)
                assert np.array_equal(out[: s.size], s), (dt, shape, rate)


def test_strided_views(hostcodec, orc):
    """Strided fields (zfp_field sx/sy/sz): transposed, reversed and stepped
    views, and sub-arrays, through the kernels' per-block code on the host:
    the stream is the oracle's strided stream, and decoding into a strided
    view writes exactly the oracle's values there and nothing else."""
    rng = np.random.default_rng(34)
    for dt in (np.float32, np.float64, np.int32, np.int64):
        base3 = np.cumsum(rng.standard_normal(23 * 19 * 17)).reshape(23, 19, 17)
        base2 = np.cumsum(rng.standard_normal(41 * 37)).reshape(41, 37)
        base1 = np.cumsum(rng.standard_normal(301))
        if np.dtype(dt).kind == "i":
            base3, base2, base1 = base3 * 5000, base2 * 5000, base1 * 5000
        b3, b2, b1 = base3.astype(dt), base2.astype(dt), base1.astype(dt)
        views = [b3.transpose(2, 0, 1), b3[::-1, :, ::2], b3[3:20, 1::3, ::-1],
                 b2.T, b2[::-2, 5:30], b1[::-3], b1[200:7:-1]]
        for v in views:
            for rate in (5.5, 16.0):
                s = orc.compress_view(v, rate)
                (nx, ny, nz), (sx, sy, sz), addr = orc.view_geometry(v)
                t = orc.type_code(dt)
                out = np.zeros(s.size + 1, np.uint64)
                n = hostcodec.hc_compress_strided(t, nx, ny, nz, sx, sy, sz, rate, addr,
                                                  out.ctypes.data, out.nbytes)
                assert n == s.nbytes and np.array_equal(out[: s.size], s), (dt, v.shape, rate)
                # decode into the same view of two copies of its buffer
                base = b3 if v.ndim == 3 else b2 if v.ndim == 2 else b1
                mine, theirs = base.copy(), base.copy()
                off = addr - base.__array_interface__["data"][0]  # bytes to value (0, 0, 0)
                s = np.ascontiguousarray(s)
                m_addr = mine.__array_interface__["data"][0] + off
                got = hostcodec.hc_decompress_strided(t, nx, ny, nz, sx, sy, sz, rate,
                                                      s.ctypes.data, s.nbytes, m_addr)
                assert got == s.nbytes
                tv = np.ndarray(v.shape, dt, theirs, off, v.strides)
                orc.decompress_into(s, tv, rate)
                assert np.array_equal(mine.view(np.uint8), theirs.view(np.uint8)), (dt, v.shape, rate)
