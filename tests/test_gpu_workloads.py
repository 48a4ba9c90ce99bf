"""Parity at the measured workloads' full sizes.

The whole array is compressed and decompressed on the GPU, and the whole
stream and the whole decoded array are compared bit for bit with the
oracle's (its multithreaded CPU restatement of zfp 0.5.0) on the same
input, as the reference's own fuzzer compares whole streams and outputs
(src/utils/test.py:74-92).  Smaller instances of the same workloads are
compared in full too.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def run_workload(gz, orc, x, rate):
    """Compress and decompress the device array x; compare the whole stream
    and the whole output with the oracle's."""
    import torch
    w = gz.compress_tensor(x, rate)
    dims = x.dim()
    t = gz.zfp_type.float if x.dtype == torch.float32 else gz.zfp_type.double
    zfp = gz.zfp_stream()
    gz.stream_set_rate(zfp, rate, t, dims)
    shape = tuple(x.shape)
    nx, ny, nz = (tuple(reversed(shape)) + (0, 0))[:3]
    assert w.numel() * 8 == gz.stream_size(t, nx, ny, nz, zfp.maxbits)
    dec = gz.decompress_tensor(w, shape, x.dtype, rate)
    torch.cuda.synchronize()
    host = x.cpu().numpy()
    words = w.cpu().numpy().view(np.uint64)
    del w
    s = orc.compress(host, rate, THREADS)
    assert words.shape == s.shape
    bad = np.flatnonzero(words != s)
    assert bad.size == 0, f"{bad.size} stream words differ, first at word {bad[:4]}"
    del words
    dech = dec.cpu().numpy()
    del dec
    d = orc.decompress(s, shape, host.dtype, rate, THREADS)
    it = np.uint32 if host.dtype == np.float32 else np.uint64
    bad = np.flatnonzero(dech.view(it).ravel() != d.view(it).ravel())
    assert bad.size == 0, f"{bad.size} values differ, first at {bad[:4]}"


def test_smooth_noisy_64cube_f32_full(gz, orc, cuda):
    """64^3 float32, rate 16: whole stream and output against the oracle."""
    import torch
    from cuzfp_gb300 import synth
    a = synth.smooth_noisy_3d(64, seed=0, dtype=np.float32)
    w = gz.compress_tensor(torch.from_numpy(a).to(cuda), 16.0)
    s = orc.compress(a, 16.0)
    assert np.array_equal(w.cpu().numpy().view(np.uint64), s)
    d = gz.decompress_tensor(w, a.shape, torch.float32, 16.0).cpu().numpy()
    assert np.array_equal(d.view(np.uint8), orc.decompress(s, a.shape, a.dtype, 16.0).view(np.uint8))


@pytest.mark.parametrize("rate", [8.0, 16.0, 32.0])
def test_sinusoids_3d_f64_reduced_full(gz, orc, cuda, rate):
    """A 129 x 130 x 131 instance of the 3D float64 workload, compared in full."""
    import torch
    from cuzfp_gb300 import synth
    a = synth.sinusoids((129, 130, 131), 16, 32, seed=5, dtype=np.float64)
    w = gz.compress_tensor(torch.from_numpy(a).to(cuda), rate)
    s = orc.compress(a, rate, 8)
    assert np.array_equal(w.cpu().numpy().view(np.uint64), s)
    d = gz.decompress_tensor(w, a.shape, torch.float64, rate).cpu().numpy()
    assert np.array_equal(d.view(np.uint8), orc.decompress(s, a.shape, a.dtype, rate, 8).view(np.uint8))


@pytest.mark.parametrize("rate", [8.0, 16.0, 32.0])
def test_sinusoids_512cube_f64(gz, orc, cuda, rate):
    """The 1 GiB 3D float64 workload at full size."""
    import torch
    from cuzfp_gb300 import synth
    x = synth.sinusoids_device((512, 512, 512), 16, 32, seed=0, dtype=torch.float64, device=cuda)
    run_workload(gz, orc, x, rate)


@pytest.mark.parametrize("rate", [4.0, 12.0, 24.0])
def test_random_walk_1d_f32_full_size(gz, orc, cuda, rate):
    """2^28 - 3 float32 values (partial last block), rates 16/48/96 bits per
    block, which are not word multiples, so neighbouring blocks share words."""
    import torch
    from cuzfp_gb300 import synth
    x = synth.random_walk_device((1 << 28) - 3, seed=2, dtype=torch.float32, device=cuda)
    run_workload(gz, orc, x, rate)


@pytest.mark.parametrize("rate", [4.0, 12.0, 24.0])
def test_sinusoids_2d_full_size(gz, orc, cuda, rate):
    """2D float32 16381 x 16383 and float64 8191 x 8190, partial edge blocks."""
    import torch
    from cuzfp_gb300 import synth
    for shape, dt, seed in (((16383, 16381), torch.float32, 3), ((8190, 8191), torch.float64, 4)):
        x = synth.sinusoids_device(shape, 8, 64, seed=seed, dtype=dt, device=cuda)
        run_workload(gz, orc, x, rate)
        del x


@pytest.mark.parametrize("rate", [4.0, 12.0, 24.0])
def test_reduced_1d_2d_full(gz, orc, cuda, rate):
    """Smaller instances of the 1D / 2D workloads, compared in full."""
    import torch
    from cuzfp_gb300 import synth
    for a in (synth.random_walk((1 << 20) - 3, seed=9, dtype=np.float32),
              synth.sinusoids((1021, 1023), 8, 64, seed=3, dtype=np.float32),
              synth.sinusoids((510, 511), 8, 64, seed=4, dtype=np.float64)):
        w = gz.compress_tensor(torch.from_numpy(a).to(cuda), rate)
        s = orc.compress(a, rate, 8)
        assert np.array_equal(w.cpu().numpy().view(np.uint64), s), (a.shape, a.dtype)
        tdt = torch.float32 if a.dtype == np.float32 else torch.float64
        d = gz.decompress_tensor(w, a.shape, tdt, rate).cpu().numpy()
        assert np.array_equal(d.view(np.uint8),
                              orc.decompress(s, a.shape, a.dtype, rate, 8).view(np.uint8))
