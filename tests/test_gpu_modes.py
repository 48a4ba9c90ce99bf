"""zfp's general coding modes on the GPU through the C ABI: fixed
precision, fixed accuracy and other parameter sets give the reference's
streams (golden fixtures) and the oracle's, block start bits included;
decoding works from returned offsets and from the serial block walk."""
from __future__ import annotations

import numpy as np
import pytest

from tests import golden_io

pytestmark = pytest.mark.gpu

TYPES = {"float32": 3, "float64": 4, "int32": 1, "int64": 2}


def _field(rng, dt, shape):
    a = np.cumsum(rng.standard_normal(shape), axis=-1)
    return (a * 3000).astype(dt) if dt.startswith("int") else a.astype(dt)


def test_golden_mode_streams(gz, cuda):
    import torch
    for c in golden_io.mode_cases():
        a = c["input"]
        m = gz.Mode(*c["params"])
        x = torch.from_numpy(a).to(cuda)
        w, offs = gz.compress_mode(x, m, with_offsets=True)
        assert np.array_equal(w.cpu().numpy().view(np.uint64), c["stream"]), c["name"]
        for o in (offs, None):  # from the returned offsets, and from the walk
            d = gz.decompress_mode(w, a.shape, x.dtype, m, offsets=o)
            torch.cuda.synchronize()
            assert np.array_equal(d.cpu().numpy(), c["output"]), c["name"]
        # host buffers
        hw = gz.compress_mode(a, m)
        assert np.array_equal(hw, c["stream"]), c["name"]
        assert np.array_equal(gz.decompress_mode(c["stream"], a.shape, a.dtype, m), c["output"])


@pytest.mark.parametrize("dt", list(TYPES))
def test_modes_against_oracle(gz, orc, cuda, dt):
    import torch
    rng = np.random.default_rng(121)
    t = TYPES[dt]
    for shape in ((1,), (203,), (37, 29), (9, 10, 11), (16, 20), (12, 8, 16)):
        a = _field(rng, dt, shape)
        modes = [gz.mode_precision(t, p) for p in (2, 9, 24, 64)]
        modes += [gz.mode_accuracy(t, tol) for tol in (1e-9, 1e-3, 0.5, 1000.0)]
        modes += [gz.Mode(100, 300, 40, -30), gz.Mode(0, 100, 64, -1074),
                  gz.Mode(300, 300, 20, -1074), gz.Mode(500, 4171, 64, -60)]
        for m in modes:
            if m.maxbits < {3: 9, 4: 12}.get(t, 1):
                continue
            s, so = orc.compress_params(a, m.as_tuple(), with_offsets=True)
            x = torch.from_numpy(a).to(cuda)
            w, offs = gz.compress_mode(x, m, with_offsets=True)
            torch.cuda.synchronize()
            assert np.array_equal(w.cpu().numpy().view(np.uint64), s), (shape, m.as_tuple())
            assert np.array_equal(offs.cpu().numpy().view(np.uint64), so), (shape, m.as_tuple())
            exp = orc.decompress_params(s, shape, a.dtype, m.as_tuple())
            for o in (offs, None):
                d = gz.decompress_mode(w, shape, x.dtype, m, offsets=o)
                torch.cuda.synchronize()
                assert np.array_equal(d.cpu().numpy(), exp), (shape, m.as_tuple())
            walk = gz.index_blocks(w, shape, x.dtype, m)
            torch.cuda.synchronize()
            assert np.array_equal(walk.cpu().numpy().view(np.uint64), so)


def test_fixed_rate_parameters_take_the_fixed_rate_path(gz, cuda):
    import torch
    rng = np.random.default_rng(122)
    a = _field(rng, "float64", (20, 24, 28))
    x = torch.from_numpy(a).to(cuda)
    m = gz.mode_rate(gz.zfp_type.double, 3, 12.0)
    w, offs = gz.compress_mode(x, m, with_offsets=True)
    plain = gz.compress_tensor(x, 12.0)
    torch.cuda.synchronize()
    assert torch.equal(w, plain)
    nb = 5 * 6 * 7
    assert torch.equal(offs.cpu(), torch.arange(nb, dtype=torch.int64) * m.maxbits)
    d = gz.decompress_mode(w, a.shape, x.dtype, m)
    assert torch.equal(d, gz.decompress_tensor(plain, a.shape, x.dtype, 12.0))


def test_larger_field_accuracy(gz, orc, cuda):
    """A 96^3 double field at a fixed accuracy: stream, offsets and the
    decoded field equal the oracle's, and the error stays within the
    tolerance."""
    import torch
    from cuzfp_gb300 import synth
    a = synth.smooth_noisy_3d(96, 9, np.float64)
    m = gz.mode_accuracy(gz.zfp_type.double, 1e-5)
    x = torch.from_numpy(a).to(cuda)
    w, offs = gz.compress_mode(x, m, with_offsets=True)
    s, so = orc.compress_params(a, m.as_tuple(), with_offsets=True)
    assert np.array_equal(w.cpu().numpy().view(np.uint64), s)
    assert np.array_equal(offs.cpu().numpy().view(np.uint64), so)
    d = gz.decompress_mode(w, a.shape, x.dtype, m, offsets=offs)
    torch.cuda.synchronize()
    out = d.cpu().numpy()
    assert np.array_equal(out, orc.decompress_params(s, a.shape, a.dtype, m.as_tuple()))
    assert np.max(np.abs(out - a)) <= 1e-5


def test_mode_errors(gz, cuda):
    import torch
    x = torch.randn(16, 16, 16, dtype=torch.float64, device=cuda)
    m = gz.mode_precision(gz.zfp_type.double, 40)
    tiny = torch.empty(4, dtype=torch.int64, device=cuda)
    import ctypes
    got = ctypes.c_size_t(0)
    st = gz._lib.gzfp_compress_mode(4, 16, 16, 16, ctypes.byref(m), x.data_ptr(), tiny.data_ptr(),
                                    32, ctypes.byref(got), None, None)
    assert st == gz.GZFP_ERR_CAPACITY and got.value > 32  # the size it needs
    w = gz.compress_mode(x, m)
    with pytest.raises(gz.GzfpError) as e:  # stream cut short: the walk runs past it
        gz.decompress_mode(w[: w.numel() // 2], x.shape, x.dtype, m)
    assert e.value.status == gz.GZFP_ERR_ARG


@pytest.mark.parametrize("dt", list(TYPES))
def test_headed_modes(gz, orc, cuda, dt):
    """A header of the mode, then the blocks: the oracle's stream (itself
    pinned to zfp_write_header + zfp_compress); gzfp_decompress_headed
    decodes it from the header alone."""
    import torch
    rng = np.random.default_rng(123)
    t = TYPES[dt]
    for shape in ((203,), (37, 29), (9, 10, 11)):
        a = _field(rng, dt, shape)
        for m in (gz.mode_precision(t, 20), gz.mode_accuracy(t, 1e-4), gz.Mode(100, 300, 40, -30),
                  gz.mode_rate(t, len(shape), 10.0)):
            s = orc.compress_params_headed(a, m.as_tuple())
            x = torch.from_numpy(a).to(cuda)
            w, offs = gz.compress_mode_headed(x, m, with_offsets=True)
            torch.cuda.synchronize()
            assert np.array_equal(w.cpu().numpy().view(np.uint64), s), (shape, m.as_tuple())
            h = gz.read_header_mode(w)
            assert int(offs[0]) == h["bits"]
            d = gz.decompress_headed(w)
            torch.cuda.synchronize()
            exp = orc.decompress_params(orc.compress_params(a, m.as_tuple()), shape, a.dtype,
                                        m.as_tuple())
            assert np.array_equal(d.cpu().numpy(), exp), (shape, m.as_tuple())
            assert np.array_equal(gz.decompress_headed(s), exp)  # host stream


def test_random_params(gz, orc, cuda):
    """Random stream parameters and shapes, every scalar type: the GPU's
    streams, block start bits and decoded arrays are the oracle's."""
    import torch
    from tests.test_oracle import _random_params
    rng = np.random.default_rng(142)
    for k in range(80):
        dt = ("float32", "float64", "int32", "int64")[k % 4]
        d = 1 + int(rng.integers(0, 3))
        shape = tuple(int(v) for v in rng.integers(1, 30, d))
        a = _field(rng, dt, shape)
        pr = _random_params(rng, np.dtype(dt).type)
        m = gz.Mode(*pr)
        s, so = orc.compress_params(a, pr, with_offsets=True)
        x = torch.from_numpy(a).to(cuda)
        w, offs = gz.compress_mode(x, m, with_offsets=True)
        torch.cuda.synchronize()
        assert np.array_equal(w.cpu().numpy().view(np.uint64), s), (dt, shape, pr)
        assert np.array_equal(offs.cpu().numpy().view(np.uint64), so), (dt, shape, pr)
        d_gpu = gz.decompress_mode(w, shape, x.dtype, m, offsets=offs)
        torch.cuda.synchronize()
        assert np.array_equal(d_gpu.cpu().numpy(), orc.decompress_params(s, shape, a.dtype, pr))


def test_mirror_compress_in_general_mode(gz, orc, cuda):
    """The cuZFP-style compress / decompress with zfp_stream_set_accuracy or
    _precision take the general mode: compress_mode's stream, decoded by
    walking its blocks."""
    import torch
    rng = np.random.default_rng(124)
    a = _field(rng, "float32", (24, 20, 36))
    x = torch.from_numpy(a).to(cuda)
    for setter, v in ((gz.zfp_stream_set_accuracy, 1e-3), (gz.zfp_stream_set_precision, 18)):
        zfp = gz.zfp_stream()
        setter(zfp, v, gz.zfp_type.float)
        f = gz.zfp_field_3d(x, gz.zfp_type.float, 36, 20, 24)
        cap = gz.zfp_stream_maximum_size(zfp, f)
        zfp.stream = torch.zeros(cap // 8, dtype=torch.int64, device=cuda)
        n = gz.compress(zfp, f)
        exp = orc.compress_params(a, (zfp.minbits, zfp.maxbits, zfp.maxprec, zfp.minexp))
        assert n == exp.nbytes
        assert np.array_equal(zfp.stream[: n // 8].cpu().numpy().view(np.uint64), exp)
        out = torch.empty_like(x)
        gz.decompress(zfp, gz.zfp_field_3d(out, gz.zfp_type.float, 36, 20, 24))
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(),
                              orc.decompress_params(exp, a.shape, a.dtype,
                                                    (zfp.minbits, zfp.maxbits, zfp.maxprec,
                                                     zfp.minexp)))


@pytest.mark.parametrize("case", ["3d_f64_acc", "3d_f64_prec", "3d_f32_acc", "2d_f64_acc",
                                  "1d_f32_prec", "3d_i64_prec"])
def test_parallel_index(gz, orc, cuda, case):
    """Streams of thousands of blocks are indexed by the parallel walkers:
    the start bits equal the compressor's, and decompressing without them
    (the index runs inside the call) gives the same field, plain and headed."""
    import torch
    from cuzfp_gb300 import synth
    if case == "3d_f64_acc":
        a = synth.sinusoids((128, 128, 128), 16, 32, seed=1, dtype=np.float64)
        m = gz.mode_accuracy(gz.zfp_type.double, 1e-6)
    elif case == "3d_f64_prec":
        a = synth.sinusoids((112, 120, 128), 16, 32, seed=2, dtype=np.float64)
        m = gz.mode_precision(gz.zfp_type.double, 16)
    elif case == "3d_f32_acc":
        a = synth.smooth_noisy_3d(96, 3, np.float32)
        m = gz.mode_accuracy(gz.zfp_type.float, 1e-4)
    elif case == "2d_f64_acc":
        a = synth.sinusoids((510, 517), 8, 64, seed=4, dtype=np.float64)
        m = gz.mode_accuracy(gz.zfp_type.double, 1e-6)
    elif case == "1d_f32_prec":
        a = synth.random_walk((1 << 16) - 5, seed=5, dtype=np.float32)
        m = gz.mode_precision(gz.zfp_type.float, 12)
    else:
        a = (synth.sinusoids((80, 81, 82), 16, 32, seed=6) * 1e9).astype(np.int64)
        m = gz.mode_precision(gz.zfp_type.int64, 32)
    x = torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    w, offs = gz.compress_mode(x, m, with_offsets=True)
    assert offs.numel() >= 4096
    idx = gz.index_blocks(w, a.shape, x.dtype, m)
    torch.cuda.synchronize()
    assert torch.equal(idx, offs)
    d0 = gz.decompress_mode(w, a.shape, x.dtype, m, offsets=offs)
    d1 = gz.decompress_mode(w, a.shape, x.dtype, m)
    torch.cuda.synchronize()
    it = {np.float32: torch.int32, np.float64: torch.int64, np.int64: torch.int64}[a.dtype.type]
    assert torch.equal(d0.view(it), d1.view(it))
    s = orc.compress_params(a, m.as_tuple())
    assert np.array_equal(w.cpu().numpy().view(np.uint64), s)
    hw = gz.compress_mode_headed(x, m)
    hd = gz.decompress_headed(hw)
    torch.cuda.synchronize()
    assert torch.equal(hd.reshape(d0.shape).view(it), d0.view(it))
