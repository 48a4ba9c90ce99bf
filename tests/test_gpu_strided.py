"""Strided fields (zfp_field sx/sy/sz) on the GPU through the C ABI: the
stream of a strided view is the oracle's (zfp's strided compression), and
decoding into a view writes exactly its values."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch_views(t):
    return [t[3:20, :, 5:9], t[::2, 1::3, 2:], t.transpose(0, 2), t.permute(1, 0, 2)[::2],
            t[:, 7, :], t[5, ::2, :], t[2, 3, ::3], t[1:, 2::2, ::3]]


@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "int64"])
def test_device_views(gz, orc, cuda, dt):
    import torch
    rng = np.random.default_rng(51)
    a = np.cumsum(rng.standard_normal((30, 26, 22)), axis=2)
    a = (a * 1000).astype(dt) if dt.startswith("int") else a.astype(dt)
    t = torch.from_numpy(a).to(cuda)
    for tv in _torch_views(t):
        nv = tv.cpu().numpy()  # same values, contiguous copy
        for rate in (4.0, 12.5, 32.0):
            if orc.stream_bytes(nv.shape, nv.dtype, rate) == 0:
                continue
            w = gz.compress_tensor(tv, rate)
            s = orc.compress(np.ascontiguousarray(nv), rate)
            assert np.array_equal(w.cpu().numpy().view(np.uint64), s), (tv.shape, tv.stride(), rate)
            # decode into a strided view of a sentinel-filled tensor
            buf = torch.full_like(t, 7)
            out = buf.as_strided(tv.shape, tv.stride(), tv.storage_offset())
            gz.decompress_tensor(w, tv.shape, tv.dtype, rate, out=out)
            torch.cuda.synchronize()
            exp = orc.decompress(s, nv.shape, nv.dtype, rate)
            assert np.array_equal(out.cpu().numpy(), exp), (tv.shape, rate)
            mask = torch.ones_like(buf, dtype=torch.bool)
            mask.as_strided(tv.shape, tv.stride(), tv.storage_offset()).fill_(False)
            assert bool((buf[mask] == 7).all())


def _c_compress_strided(gz, typ, shape, strides, maxbits, addr, words, cap):
    nx, ny, nz = gz._dims_of(shape)
    sx, sy, sz = (list(strides) + [0, 0])[:3]
    out = ctypes.c_size_t(0)
    return gz._lib.gzfp_compress_strided(int(typ), nx, ny, nz, sx, sy, sz, maxbits, addr, words,
                                         cap, ctypes.byref(out), None)


def test_negative_strides_device_and_host(gz, orc, cuda):
    """Reversed axes (negative strides) through the C ABI, on device memory
    and on host memory (staged as the span the strides reach)."""
    import torch
    rng = np.random.default_rng(52)
    a = np.cumsum(rng.standard_normal((21, 18, 15)), axis=1)
    for dt, typ in ((np.float32, gz.zfp_type.float), (np.float64, gz.zfp_type.double)):
        h = a.astype(dt)
        v = h[::-1, ::2, ::-3]  # negative and positive strides
        st = [s // h.itemsize for s in v.strides[::-1]]
        rate = 10.0
        mb = gz._lib.gzfp_rate_to_maxbits(int(typ), 3, rate)
        s_ref = orc.compress(np.ascontiguousarray(v), rate)
        # device: the view's first element inside a device copy of the base
        t = torch.from_numpy(h).to(cuda)
        off = (v.__array_interface__["data"][0] - h.__array_interface__["data"][0])
        w = torch.zeros(s_ref.size, dtype=torch.int64, device=cuda)
        assert _c_compress_strided(gz, typ, v.shape, st, mb, t.data_ptr() + off, w.data_ptr(),
                                   w.numel() * 8) == 0
        torch.cuda.synchronize()
        assert np.array_equal(w.cpu().numpy().view(np.uint64), s_ref)
        # host: numpy view straight through the Python mirror
        zfp = gz.zfp_stream()
        gz.stream_set_rate(zfp, rate, typ, 3)
        buf = np.zeros(s_ref.size, np.uint64)
        zfp.stream = buf
        nx, ny, nz = gz._dims_of(v.shape)
        f = gz.zfp_field(type=typ, nx=nx, ny=ny, nz=nz, data=v)
        assert gz.compress(zfp, f) == s_ref.nbytes
        assert np.array_equal(buf, s_ref)
        # decode into a host view of a sentinel buffer: values, and the gaps kept
        hb = np.full_like(h, 7)
        hv = hb[::-1, ::2, ::-3]
        gz.decompress(zfp, gz.zfp_field(type=typ, nx=nx, ny=ny, nz=nz, data=hv))
        assert np.array_equal(hv, orc.decompress(s_ref, v.shape, v.dtype, rate))
        mask = np.ones(h.shape, bool)
        mask[::-1, ::2, ::-3] = False
        assert np.all(hb[mask] == 7)


def test_field_strides_set_explicitly(gz, orc, cuda):
    """zfp's own way: a contiguous buffer described with sx/sy/sz (here, a
    sub-array of a larger device array)."""
    import torch
    rng = np.random.default_rng(53)
    big = np.cumsum(rng.standard_normal((24, 40, 36)), axis=0).astype(np.float32)
    sub = big[4:17, 3:31, 5:27]
    t = torch.from_numpy(big).to(cuda)
    zfp = gz.zfp_stream()
    gz.stream_set_rate(zfp, 16.0, gz.zfp_type.float, 3)
    s_ref = orc.compress(np.ascontiguousarray(sub), 16.0)
    w = torch.zeros(s_ref.size, dtype=torch.int64, device=cuda)
    zfp.stream = w
    off = (sub.__array_interface__["data"][0] - big.__array_interface__["data"][0])
    f = gz.zfp_field(type=gz.zfp_type.float, nx=22, ny=28, nz=13, sx=1, sy=36, sz=36 * 40,
                     data=t.data_ptr() + off)
    gz.compress(zfp, f)
    torch.cuda.synchronize()
    assert np.array_equal(w.cpu().numpy().view(np.uint64), s_ref)
