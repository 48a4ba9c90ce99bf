"""CUDA codec parity: the kernels, called through the C ABI, against the
oracle on the same seeded inputs -- bit-exact streams and bit-exact
decompressed arrays -- and against the reference's golden fixtures."""
from __future__ import annotations

import numpy as np
import pytest

from tests import cases, golden_io, zfp_pins

pytestmark = pytest.mark.gpu


def to_dev(a: np.ndarray, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def gpu_compress(gz, a: np.ndarray, rate: float, cuda) -> np.ndarray:
    w = gz.compress_tensor(to_dev(a, cuda), rate)
    return w.cpu().numpy().view(np.uint64)


def gpu_decompress(gz, words: np.ndarray, shape, dtype, rate: float, cuda) -> np.ndarray:
    import torch
    tw = torch.from_numpy(np.ascontiguousarray(words).view(np.int64)).to(cuda)
    tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
           np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64}[np.dtype(dtype)]
    return gz.decompress_tensor(tw, shape, tdt, rate).cpu().numpy()


def same_bits(x: np.ndarray, y: np.ndarray) -> bool:
    return x.shape == y.shape and np.array_equal(x.view(np.uint8), y.view(np.uint8))


def test_random_cases(gz, orc, cuda):
    rng = np.random.default_rng(4242)
    for _ in range(300):
        a, rate = cases.random_case(rng)
        s = orc.compress(a, rate)
        assert np.array_equal(gpu_compress(gz, a, rate, cuda), s), (a.shape, a.dtype, rate)
        assert same_bits(gpu_decompress(gz, s, a.shape, a.dtype, rate, cuda),
                         orc.decompress(s, a.shape, a.dtype, rate)), (a.shape, a.dtype, rate)


def test_integer_fields(gz, orc, cuda):
    """int32 / int64 fields (cuZFP's integer path): every dimensionality,
    ragged shapes, whole-range values, against the oracle."""
    rng = np.random.default_rng(4343)
    for i in range(200):
        a, rate = cases.int_case(rng, wide=(i % 8 == 7))
        if orc.stream_bytes(a.shape, a.dtype, rate) == 0:
            continue
        s = orc.compress(a, rate)
        assert np.array_equal(gpu_compress(gz, a, rate, cuda), s), (a.shape, a.dtype, rate)
        assert same_bits(gpu_decompress(gz, s, a.shape, a.dtype, rate, cuda),
                         orc.decompress(s, a.shape, a.dtype, rate)), (a.shape, a.dtype, rate)


def test_integer_host_buffers(gz, orc):
    """Host integer arrays through cuZFP's pointer rules and the Python
    mirror of its structs."""
    rng = np.random.default_rng(4444)
    for dt, rate in ((np.int32, 32.0), (np.int64, 64.0)):
        a = rng.integers(-1000, 1000, (37, 41, 23)).astype(dt)
        t = gz.zfp_type.int32 if dt == np.int32 else gz.zfp_type.int64
        zfp = gz.zfp_stream()
        gz.stream_set_rate(zfp, rate, t, 3)
        buf = np.zeros(gz.zfp_stream_maximum_size(zfp, gz.zfp_field_3d(None, t, 23, 41, 37)) // 8,
                       np.uint64)
        zfp.stream = buf
        n = gz.compress(zfp, gz.zfp_field_3d(a, t, 23, 41, 37))
        s = orc.compress(a, rate)
        assert np.array_equal(buf[: n // 8], s)
        out = np.zeros_like(a)
        gz.decompress(zfp, gz.zfp_field_3d(out, t, 23, 41, 37))
        assert np.array_equal(out, orc.decompress(s, a.shape, a.dtype, rate))


def test_edge_cases(gz, orc, cuda):
    for a, rate in cases.edge_cases():
        s = orc.compress(a, rate)
        assert np.array_equal(gpu_compress(gz, a, rate, cuda), s), (a.shape, a.dtype, rate)
        assert same_bits(gpu_decompress(gz, s, a.shape, a.dtype, rate, cuda),
                         orc.decompress(s, a.shape, a.dtype, rate))


def test_arbitrary_streams(gz, orc, cuda):
    """Decoding random words exercises budget cut-offs in every plane."""
    rng = np.random.default_rng(17)
    for shape in ((64,), (13, 9), (8, 7, 6), (21, 22, 23)):
        for dt in (np.float32, np.float64):
            for rate in (1, 2.5, 8, 16, 33):
                n = orc.stream_bytes(shape, dt, rate) // 8
                w = rng.integers(0, 2 ** 63, n, dtype=np.int64).astype(np.uint64) << np.uint64(1)
                w |= rng.integers(0, 2, n, dtype=np.int64).astype(np.uint64)
                assert same_bits(gpu_decompress(gz, w, shape, dt, rate, cuda),
                                 orc.decompress(w, shape, dt, rate)), (shape, dt, rate)


def test_1d_plane_tables(gz, orc, cuda):
    """1D blocks code and decode through the 4-value plane tables: every
    length remainder, all four scalar types, budgets from 2 to 256 bits per
    block (word-aligned or not), and random words decoded at each budget."""
    rng = np.random.default_rng(4646)
    rates = (0.5, 1, 2.25, 3, 4, 7, 8, 12, 13.5, 16, 24, 31, 32, 48, 64)
    for i, rate in enumerate(rates):
        for dt in (np.float32, np.float64, np.int32, np.int64):
            n = int(rng.integers(1, 3000)) + i % 4
            if np.dtype(dt).kind == "f":
                a = (np.cumsum(rng.standard_normal(n)) * 10.0 ** rng.integers(-20, 20)).astype(dt)
            else:
                bits = 8 * np.dtype(dt).itemsize
                a = np.clip(np.cumsum(rng.integers(-1000, 1000, n)), -(2 ** (bits - 3)),
                            2 ** (bits - 3)).astype(dt)
            if orc.stream_bytes(a.shape, a.dtype, rate) == 0:
                continue
            s = orc.compress(a, rate)
            assert np.array_equal(gpu_compress(gz, a, rate, cuda), s), (n, dt, rate)
            assert same_bits(gpu_decompress(gz, s, a.shape, a.dtype, rate, cuda),
                             orc.decompress(s, a.shape, a.dtype, rate)), (n, dt, rate)
            if np.dtype(dt).kind == "f":
                w = rng.integers(0, 2 ** 63, s.size, dtype=np.int64).astype(np.uint64)
                w = (w << np.uint64(1)) | rng.integers(0, 2, s.size).astype(np.uint64)
                assert same_bits(gpu_decompress(gz, w, a.shape, a.dtype, rate, cuda),
                                 orc.decompress(w, a.shape, a.dtype, rate)), ("random", n, dt, rate)


def test_golden_small(gz, cuda):
    for c in golden_io.load_all():
        a = c["input"]
        assert np.array_equal(gpu_compress(gz, a, c["rate"], cuda), c["stream"]), c["name"]
        assert same_bits(gpu_decompress(gz, c["stream"], a.shape, a.dtype, c["rate"], cuda),
                         c["output"]), c["name"]


def test_golden_manifest(gz, cuda):
    for sp in golden_io.manifest():
        a = golden_io.generate(sp)
        assert golden_io.sha(a) == sp["input_sha256"], sp["name"]
        s = gpu_compress(gz, a, sp["rate"], cuda)
        assert golden_io.sha(s) == sp["stream_sha256"], sp["name"]
        d = gpu_decompress(gz, s, a.shape, a.dtype, sp["rate"], cuda)
        assert golden_io.sha(d) == sp["output_sha256"], sp["name"]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_testzfp_pins(gz, cuda, dt, d):
    """Fixed-rate size and max-error pins of zfp-0.5.0/tests/testzfp.cpp."""
    f = zfp_pins.field(dt, d)
    for rate, tol in zfp_pins.rate_pins(dt, d):
        s = gpu_compress(gz, f, rate, cuda)
        zfp = gz.zfp_stream()
        actual = gz.stream_set_rate(zfp, rate, gz.zfp_type.float if dt == np.float32
                                    else gz.zfp_type.double, d)
        assert s.nbytes == zfp_pins.expected_bytes(actual, f.size)
        g = gpu_decompress(gz, s, f.shape, f.dtype, rate, cuda)
        assert float(np.max(np.abs(f - g))) <= tol


@pytest.mark.parametrize("rate", [12.0, 7.3])
def test_host_and_pinned_pointers(gz, orc, cuda, rate):
    """cuZFP's host-pointer path: arrays and streams in host memory.  On a
    coherent host link pinned buffers are coded in place by the kernels
    (rate 12: whole-word blocks), or staged through device memory (rate
    7.3: blocks that share words, compression only); pageable buffers are
    always staged."""
    import torch
    rng = np.random.default_rng(3)
    a = rng.standard_normal((19, 23, 29)).astype(np.float64)
    s_ref = orc.compress(a, rate)
    for pinned in (False, True):
        src = torch.from_numpy(a)
        if pinned:
            src = src.pin_memory()
        zfp = gz.zfp_stream()
        gz.stream_set_rate(zfp, rate, gz.zfp_type.double, 3)
        buf = torch.zeros(gz.zfp_stream_maximum_size(zfp, gz.zfp_field_3d(None, gz.zfp_type.double,
                                                                          29, 23, 19)) // 8,
                          dtype=torch.int64)
        if pinned:
            buf = buf.pin_memory()
        zfp.stream = buf
        n = gz.compress(zfp, gz.zfp_field_3d(src, gz.zfp_type.double, 29, 23, 19))
        assert n == s_ref.nbytes
        assert np.array_equal(buf.numpy().view(np.uint64)[: n // 8], s_ref)
        out = torch.zeros(a.shape, dtype=torch.float64)
        if pinned:
            out = out.pin_memory()
        gz.decompress(zfp, gz.zfp_field_3d(out, gz.zfp_type.double, 29, 23, 19))
        assert same_bits(out.numpy(), orc.decompress(s_ref, a.shape, a.dtype, rate))


def test_mixed_pointers(gz, orc, cuda):
    """Device array with a host stream, and the reverse."""
    import torch
    a = np.linspace(-3, 7, 40 * 41, dtype=np.float32).reshape(40, 41)
    rate = 9.0
    s_ref = orc.compress(a, rate)
    zfp = gz.zfp_stream()
    gz.stream_set_rate(zfp, rate, gz.zfp_type.float, 2)
    host_buf = np.zeros(s_ref.size, np.uint64)
    zfp.stream = host_buf
    gz.compress(zfp, gz.zfp_field_2d(to_dev(a, cuda), gz.zfp_type.float, 41, 40))
    assert np.array_equal(host_buf, s_ref)
    dev_out = torch.zeros((40, 41), dtype=torch.float32, device=cuda)
    gz.decompress(zfp, gz.zfp_field_2d(dev_out, gz.zfp_type.float, 41, 40))
    assert same_bits(dev_out.cpu().numpy(), orc.decompress(s_ref, a.shape, a.dtype, rate))


@pytest.mark.parametrize("shape,dtype,rate", [
    ((203, 257, 301), np.float32, 7.3),   # 467-bit blocks: slabs of 16 block layers
    ((2999, 3001), np.float64, 4.0),      # word-sized blocks, ragged last slab
    (((1 << 24) + 3,), np.float32, 12.0),  # 48-bit blocks, 4 blocks per 3 words
])
def test_staged_slabs(gz, cuda, shape, dtype, rate):
    """Host buffers larger than one staging slab give the stream and array of
    the all-device call (which the oracle pins), for pinned and pageable
    host memory and for mixed pointers: pageable memory, and compression at
    rates whose blocks share words, go through the slab pipeline; pinned
    memory on a coherent host link is otherwise coded in place."""
    import torch
    rng = np.random.default_rng(17)
    a = np.cumsum(rng.standard_normal(int(np.prod(shape)))).astype(dtype).reshape(shape)
    x = torch.from_numpy(a).to(cuda)
    w_dev = gz.compress_tensor(x, rate)
    y_dev = gz.decompress_tensor(w_dev, shape, x.dtype, rate)
    torch.cuda.synchronize()
    w_ref = w_dev.cpu()
    y_ref = y_dev.cpu().numpy()
    t = gz.zfp_type.float if dtype == np.float32 else gz.zfp_type.double
    dims = gz._dims_of(shape)

    def field(data):
        return gz.zfp_field(type=t, nx=dims[0], ny=dims[1], nz=dims[2], data=data)

    for pinned in (True, False):
        src = torch.from_numpy(a)
        buf = torch.zeros_like(w_ref)
        out = torch.zeros(shape, dtype=x.dtype)
        if pinned:
            src, buf, out = src.pin_memory(), buf.pin_memory(), out.pin_memory()
        zfp = gz.zfp_stream(stream=buf)
        gz.stream_set_rate(zfp, rate, t, len(shape))
        assert gz.compress(zfp, field(src)) == buf.numel() * 8
        assert torch.equal(buf, w_ref), pinned
        gz.decompress(zfp, field(out))
        assert same_bits(out.numpy(), y_ref), pinned
    # device array <-> host stream, host stream -> device array
    buf = torch.zeros_like(w_ref).pin_memory()
    zfp = gz.zfp_stream(stream=buf)
    gz.stream_set_rate(zfp, rate, t, len(shape))
    gz.compress(zfp, field(x))
    assert torch.equal(buf, w_ref)
    y = torch.zeros_like(x)
    gz.decompress(zfp, field(y))
    torch.cuda.synchronize()
    assert same_bits(y.cpu().numpy(), y_ref)
    # host array -> device stream
    w = torch.zeros_like(w_dev)
    zfp = gz.zfp_stream(stream=w)
    gz.stream_set_rate(zfp, rate, t, len(shape))
    gz.compress(zfp, field(torch.from_numpy(a).pin_memory()))
    torch.cuda.synchronize()
    assert torch.equal(w, w_dev)


def test_user_stream_async(gz, orc, cuda):
    """Device buffers on a caller's stream: the call is asynchronous and the
    result is complete once that stream is synchronised."""
    import torch
    rng = np.random.default_rng(8)
    a = rng.standard_normal((64, 64, 64)).astype(np.float32)
    s_ref = orc.compress(a, 16.0)
    st = torch.cuda.Stream()
    x = to_dev(a, cuda)
    torch.cuda.synchronize()
    with torch.cuda.stream(st):
        w = gz.compress_tensor(x, 16.0, cuda_stream=st)
        y = gz.decompress_tensor(w, a.shape, torch.float32, 16.0, cuda_stream=st)
    st.synchronize()
    assert np.array_equal(w.cpu().numpy().view(np.uint64), s_ref)
    assert same_bits(y.cpu().numpy(), orc.decompress(s_ref, a.shape, a.dtype, 16.0))


def test_errors(gz, cuda):
    import torch
    x = torch.zeros((4, 4, 4), dtype=torch.float64, device=cuda)
    small = torch.zeros(4, dtype=torch.int64, device=cuda)
    with pytest.raises(gz.GzfpError) as e:
        gz.compress_tensor(x, 16.0, out=small)
    assert e.value.status == gz.GZFP_ERR_CAPACITY
    with pytest.raises(gz.GzfpError):
        gz.compress_tensor(torch.zeros(4, dtype=torch.int16, device=cuda), 8.0)
    with pytest.raises(gz.GzfpError):  # 0 bits per integer block
        gz.compress_tensor(torch.zeros(4, dtype=torch.int32, device=cuda), 0.0)
    # the context stays usable after rejected calls
    w = gz.compress_tensor(x, 16.0)
    assert int(w.abs().sum()) == 0
