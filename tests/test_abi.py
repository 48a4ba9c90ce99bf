"""The C ABI library without a GPU: it loads, exports every function that
include/*.h declares, and its size / rate helpers and argument checks agree
with the reference.  No call here reaches a CUDA kernel."""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions() -> list[str]:
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        if 'extern "C"' not in src:
            continue
        body = src.split('extern "C"', 1)[1]
        names += re.findall(r"\b(gzfp_\w+)\s*\(", body)
    return sorted(set(names))


def test_library_exports_declared_symbols(gz):
    lib = ctypes.CDLL(gz.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n


def test_version_and_status_strings(gz):
    assert gz.version() >= 10000
    lib = gz._lib
    for st in range(5):
        assert lib.gzfp_status_string(st)


def test_rate_to_maxbits_matches_reference(gz, ref):
    for t in (1, 2, 3, 4):
        for dims in (1, 2, 3):
            for rate in (0, 0.1, 0.5, 1, 2, 2.25, 3.3, 4, 7.99, 8, 12, 16, 17.7, 24, 32, 64):
                assert gz._lib.gzfp_rate_to_maxbits(t, dims, rate) == \
                    ref.ref().zref_set_rate_bits(t, dims, rate), (t, dims, rate)


def test_maximum_size_matches_reference(gz, ref):
    for t in (1, 2, 3, 4):
        for shape in ((1,), (17,), (5, 9), (64, 64), (3, 4, 5), (33, 17, 9)):
            nx, ny, nz = ref.dims3(shape)
            for rate in (1, 4, 8, 16, 32, 64, 100):
                mb = ref.ref().zref_set_rate_bits(t, len(shape), rate)
                assert gz._lib.gzfp_maximum_size(t, nx, ny, nz, mb) == \
                    ref.ref().zref_maximum_size(t, nx, ny, nz, rate), (t, shape, rate)


def test_stream_size_matches_oracle(gz, orc):
    for t, dt in ((3, np.float32), (4, np.float64)):
        for shape in ((1,), (1023,), (5, 9), (3, 4, 5), (512, 512, 512)):
            nx, ny, nz = orc.dims3(shape)
            for rate in (1, 4, 12, 16, 24, 32):
                mb = gz._lib.gzfp_rate_to_maxbits(t, len(shape), rate)
                assert gz.stream_size(t, nx, ny, nz, mb) == orc.stream_bytes(shape, dt, rate)


def _compress_status(gz, t, nx, ny, nz, rate, data=1, stream=1, cap=1 << 30):
    out = ctypes.c_size_t(0)
    return gz._lib.gzfp_compress(t, nx, ny, nz, rate, data, stream, cap, ctypes.byref(out), None)


def test_argument_errors_without_device(gz):
    """Checks that fail before any CUDA call."""
    assert _compress_status(gz, 9, 4, 4, 4, 8.0) == gz.GZFP_ERR_ARG
    assert _compress_status(gz, 0, 4, 4, 4, 8.0) == gz.GZFP_ERR_ARG   # zfp_type_none
    assert _compress_status(gz, 1, 4, 4, 4, 0.0) == gz.GZFP_ERR_ARG   # int32: 0 bits per block
    assert _compress_status(gz, 2, 4, 4, 4, 0.001) == gz.GZFP_ERR_ARG  # int64: rounds to 0 bits
    assert _compress_status(gz, 3, 0, 4, 4, 8.0) == gz.GZFP_ERR_ARG
    assert _compress_status(gz, 3, 4, 0, 4, 8.0) == gz.GZFP_ERR_ARG
    assert _compress_status(gz, 3, 4, 4, 4, -1.0) == gz.GZFP_ERR_ARG
    assert _compress_status(gz, 3, 4, 4, 4, float("nan")) == gz.GZFP_ERR_ARG
    assert _compress_status(gz, 3, 4, 4, 4, 8.0, data=0) == gz.GZFP_ERR_ARG
    assert _compress_status(gz, 4, 8, 8, 8, 16.0, cap=1016) == gz.GZFP_ERR_CAPACITY
    assert gz._lib.gzfp_last_error()
    st = gz._lib.gzfp_decompress(3, 16, 16, 0, 8.0, 1, 8, 1, None)
    assert st == gz.GZFP_ERR_ARG  # stream shorter than the compressed size
    st = gz._lib.gzfp_compress_bits(3, 4, 4, 4, 8, 1, 1, 1 << 20, None, None)
    assert st == gz.GZFP_ERR_ARG  # fewer bits than the block header


def test_python_mirror_errors(gz):
    zfp = gz.zfp_stream()
    with pytest.raises(gz.GzfpError):
        gz.stream_set_rate(zfp, 8.0, gz.zfp_type.float, 4)
    gz.stream_set_rate(zfp, 8.0, gz.zfp_type.float, 3)
    assert zfp.maxbits == zfp.minbits == 512
    f = gz.zfp_field_3d(None, gz.zfp_type.float, 4, 4, 4)
    zfp.minbits = 0  # not fixed rate: zfp's general mode, but no data
    with pytest.raises(gz.GzfpError) as e:
        gz.compress(zfp, f)
    assert e.value.status == gz.GZFP_ERR_ARG
    f.sx = 2  # strided fields take the fixed-rate path only
    with pytest.raises(gz.GzfpError) as e:
        gz.compress(zfp, f)
    assert e.value.status == gz.GZFP_ERR_UNSUPPORTED
    f.sx = 0
    gz.stream_set_rate(zfp, 8.0, gz.zfp_type.float, 3)
    f.sx = 2
    with pytest.raises(gz.GzfpError) as e:  # strided, but no data
        gz.compress(zfp, f)
    assert e.value.status == gz.GZFP_ERR_ARG
    assert gz.zfp_field_dimensionality(gz.zfp_field_2d(None, gz.zfp_type.double, 3, 5)) == 2
    assert abs(gz.stream_set_rate(zfp, 2.0, gz.zfp_type.float, 1) - 2.25) < 1e-12


def test_header_write_matches_oracle(gz, orc):
    """gzfp_write_header's bits are the first bits of the oracle's headed
    stream (zfp_write_header with ZFP_HEADER_FULL), for every scalar type,
    dimensionality and both mode forms; gzfp_read_header gives them back."""
    from tests import golden_io
    dts = {1: np.int32, 2: np.int64, 3: np.float32, 4: np.float64}
    n = 0
    for t, dt in dts.items():
        for shape in ((1,), (203,), (5, 9), (16777216, 3), (3, 4, 5), (65536, 2, 3)):
            for rate in (0.5, 4, 16, 32, 100, 500):
                nx, ny, nz = orc.dims3(shape)
                mb = gz._lib.gzfp_rate_to_maxbits(t, len(shape), rate)
                hb = orc.port().gzo_header_bits(t, nx, ny, nz, float(rate))
                if mb == 0 or mb < {1: 1, 2: 1, 3: 9, 4: 12}[t]:
                    continue
                buf = ctypes.create_string_buffer(24)
                bits = ctypes.c_size_t(0)
                st = gz._lib.gzfp_write_header(t, nx, ny, nz, mb, buf, 24, ctypes.byref(bits))
                if hb == 0:  # maxbits beyond the 64-bit mode form
                    assert st == gz.GZFP_ERR_ARG and mb > 32768, (t, shape, rate)
                    continue
                assert st == 0 and bits.value == hb, (t, shape, rate)
                # the oracle's reader and the C ABI's read the same field back
                h = orc.read_header(np.frombuffer(buf.raw, np.uint8))
                assert h["bits"] == hb and h["maxbits"] == mb and h["shape"] == tuple(shape)
                assert h["dtype"] == np.dtype(dt)
                r = gz.read_header(buf.raw)
                assert r["bits"] == hb and r["maxbits"] == mb and r["shape"] == tuple(shape)
                n += 1
    assert n > 100
    for c in golden_io.headed_cases():
        h = gz.read_header(c["stream"])
        assert h["shape"] == c["input"].shape and h["dtype"] == c["input"].dtype.name
        nx, ny, nz = gz._dims_of(c["input"].shape)
        raw, bits = gz.write_header(h["type"], nx, ny, nz, h["maxbits"])
        sb = np.unpackbits(c["stream"].view(np.uint8), bitorder="little")[:bits]
        assert np.array_equal(np.unpackbits(np.frombuffer(raw, np.uint8), bitorder="little")[:bits], sb)


def test_header_errors(gz):
    lib = gz._lib
    buf = ctypes.create_string_buffer(24)
    bits = ctypes.c_size_t(0)
    w = lambda *a: lib.gzfp_write_header(*a, buf, 24, ctypes.byref(bits))  # noqa: E731
    assert w(4, 1 << 24, 5, 0, 64) == 0
    assert w(4, (1 << 24) + 1, 5, 0, 64) == gz.GZFP_ERR_ARG    # 2D axis beyond 24 bits
    assert w(3, 8, 8, (1 << 16) + 1, 64) == gz.GZFP_ERR_ARG    # 3D axis beyond 16 bits
    assert w(4, 8, 8, 8, 32769) == gz.GZFP_ERR_ARG             # beyond the long mode form
    assert w(3, 8, 8, 8, 8) == gz.GZFP_ERR_ARG                 # under the block header
    assert w(9, 8, 8, 8, 64) == gz.GZFP_ERR_ARG
    small = ctypes.create_string_buffer(12)
    assert lib.gzfp_write_header(3, 8, 0, 0, 64, small, 12, ctypes.byref(bits)) == \
        gz.GZFP_ERR_CAPACITY                                   # float: 148 bits, 19 bytes
    assert lib.gzfp_write_header(4, 8, 0, 0, 64, small, 12, ctypes.byref(bits)) == 0
    assert bits.value == 96
    with pytest.raises(gz.GzfpError) as e:
        gz.read_header(b"zfq\x05" + bytes(20))
    assert e.value.status == gz.GZFP_ERR_ARG
    with pytest.raises(gz.GzfpError) as e:
        gz.read_header(small.raw[:11])  # shorter than a header
    assert e.value.status == gz.GZFP_ERR_ARG


@pytest.mark.parametrize("idx", range(7))
def test_header_modes_abi(gz, idx):
    """zfp's other modes are reported as unsupported."""
    from tests.test_oracle import HEADER_MODES, _header_bits, _magic, _meta_3d_double
    mode, ok, maxbits = HEADER_MODES[idx]
    w = _header_bits(_magic() + [_meta_3d_double(40, 30, 20), mode])
    if ok:
        h = gz.read_header(w)
        assert h["maxbits"] == maxbits and h["shape"] == (20, 30, 40) and h["dtype"] == "float64"
    else:
        with pytest.raises(gz.GzfpError) as e:
            gz.read_header(w)
        assert e.value.status == gz.GZFP_ERR_UNSUPPORTED


def test_mode_setters_match_oracle(gz, orc):
    """gzfp_mode_precision / _accuracy / _rate give zfp's parameters (the
    oracle's restatement, itself pinned to the reference)."""
    for t, dt in ((1, np.int32), (2, np.int64), (3, np.float32), (4, np.float64)):
        for prec in (0, 1, 7, 32, 40, 64, 99):
            assert gz.mode_precision(t, prec).as_tuple() == orc.mode_precision(dt, prec)
        for tol in (0.0, 1e-300, 1e-9, 0.25, 1.0, 7.5, 1e12):
            assert gz.mode_accuracy(t, tol).as_tuple() == orc.mode_accuracy(dt, tol)
        m = gz.mode_rate(t, 3, 16.0)
        assert m.minbits == m.maxbits == 1024 and m.minexp == -1074


def test_mode_maximum_size_matches_oracle(gz, orc):
    for t, dt in ((3, np.float32), (4, np.float64), (1, np.int32), (2, np.int64)):
        for shape in ((1,), (203,), (9, 13), (5, 6, 7), (64, 64, 64)):
            nx, ny, nz = orc.dims3(shape)
            for pr in ((0, 4171, 20, -1074), (0, 4171, 64, -30), (100, 300, 40, -30),
                       (64, 64, 64, -1074)):
                got = gz.mode_maximum_size(t, nx, ny, nz, gz.Mode(*pr))
                assert got == orc.port().gzo_bound_params(t, nx, ny, nz, *pr), (t, shape, pr)


def test_mode_argument_errors(gz):
    bad = [gz.Mode(10, 5, 64, -1074), gz.Mode(0, 4171, 0, -1074), gz.Mode(0, 4171, 65, -1074)]
    for m in bad:
        assert gz.mode_maximum_size(4, 8, 8, 8, m) == 0
    assert gz.mode_maximum_size(3, 8, 8, 8, gz.Mode(0, 8, 32, -1074)) == 0  # under the block header
    with pytest.raises(gz.GzfpError):
        gz.mode_accuracy(4, float("nan"))


def test_header_mode_write_read(gz, orc):
    """gzfp_write_header_mode writes the oracle's header bits for every mode
    form, and gzfp_read_header_mode reads back the parameters zfp would."""
    n = 0
    for t, dt in ((3, np.float32), (4, np.float64), (1, np.int32), (2, np.int64)):
        for shape in ((203,), (9, 13), (5, 6, 7)):
            nx, ny, nz = orc.dims3(shape)
            modes = [gz.mode_precision(t, p) for p in (3, 24, 64)]
            modes += [gz.mode_accuracy(t, tol) for tol in (1e-8, 0.5)]
            modes += [gz.Mode(100, 300, 40, -30), gz.Mode(200, 200, 64, -1074),
                      gz.Mode(0, 4171, 16, -20), gz.mode_rate(t, len(shape), 9.0)]
            for m in modes:
                if m.maxbits < {3: 9, 4: 12}.get(t, 1):
                    continue
                raw, bits = gz.write_header_mode(t, nx, ny, nz, m)
                a = np.zeros(shape, dt)
                s = orc.compress_params_headed(a, m.as_tuple())
                sb = np.unpackbits(s.view(np.uint8), bitorder="little")[:bits]
                hb = np.unpackbits(np.frombuffer(raw, np.uint8), bitorder="little")[:bits]
                assert np.array_equal(hb, sb), (t, shape, m.as_tuple())
                h = gz.read_header_mode(raw)
                ho = orc.read_header_params(s)
                assert h["bits"] == bits == ho["bits"] and h["shape"] == shape
                assert h["mode"].as_tuple() == ho["params"], (m.as_tuple(), ho)
                n += 1
    assert n > 80
