"""Parity at the measured workloads' full sizes.

The whole array is compressed and decompressed on the GPU; the oracle then
checks block-aligned samples (bricks in 2D/3D, windows in 1D) that it can
code on its own, because a fixed-rate block's bits depend only on that
block: the GPU stream's bits for the sample must equal the oracle's stream
of the sub-array, and the GPU's decoded values there must equal the oracle's
decoding.  Smaller instances of the same workloads are compared in full.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits_of(words: np.ndarray, start: int, count: int) -> np.ndarray:
    """Bits [start, start+count) of an LSB-first uint64 word stream."""
    w0 = start // 64
    w1 = (start + count + 63) // 64
    b = np.unpackbits(words[w0:w1].view(np.uint8), bitorder="little")
    off = start - 64 * w0
    return b[off:off + count]


def gpu_field_compress(gz, x, rate):
    w = gz.compress_tensor(x, rate)
    return w


def check_region(gz, orc, host_full, words_np, dec_full, region, rate, block_index, maxbits):
    """Compare the GPU stream bits and decoded values of `region` (a tuple of
    slices, block aligned) with the oracle's coding of that sub-array."""
    sub = np.ascontiguousarray(host_full[region])
    s = orc.compress(sub, rate)
    blocks = block_index(region)
    for i, b in enumerate(blocks):
        got = bits_of(words_np, b * maxbits, maxbits)
        exp = bits_of(s, i * maxbits, maxbits)
        assert np.array_equal(got, exp), (region, i, b)
    d = orc.decompress(s, sub.shape, sub.dtype, rate)
    assert np.array_equal(d.view(np.uint8), np.ascontiguousarray(dec_full[region]).view(np.uint8))


def block_indexer(shape):
    nb = [(n + 3) // 4 for n in shape]  # C order: (z, y, x) blocks

    def index(region):
        ranges = [range(sl.start // 4, (min(sl.stop, n) + 3) // 4) for sl, n in zip(region, shape)]
        out = []
        if len(shape) == 1:
            return [bx for bx in ranges[0]]
        if len(shape) == 2:
            return [bx + nb[1] * by for by in ranges[0] for bx in ranges[1]]
        return [bx + nb[2] * (by + nb[1] * bz) for bz in ranges[0] for by in ranges[1]
                for bx in ranges[2]]
    return index


def sample_regions(shape, rng, count, edge=16):
    """Block-aligned regions, including ones that touch the far edges."""
    regions = []
    for c in range(count):
        sl = []
        for n in shape:
            nb = (n + 3) // 4
            if c == 0:
                b0 = 0
            elif c == 1:
                b0 = max(0, nb - edge // 4)
            else:
                b0 = int(rng.integers(0, max(1, nb - edge // 4 + 1)))
            sl.append(slice(4 * b0, min(n, 4 * b0 + edge)))
        regions.append(tuple(sl))
    return regions


def run_workload(gz, orc, x, rate, rng, nregions=6, edge=16):
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
    dech = dec.cpu().numpy()
    idx = block_indexer(shape)
    for region in sample_regions(shape, rng, nregions, edge):
        check_region(gz, orc, host, words, dech, region, rate, idx, zfp.maxbits)
    return host, dech


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
    run_workload(gz, orc, x, rate, np.random.default_rng(int(rate)), nregions=8)


@pytest.mark.parametrize("rate", [4.0, 12.0, 24.0])
def test_random_walk_1d_f32_full_size(gz, orc, cuda, rate):
    """2^28 - 3 float32 values (partial last block), rates 16/48/96 bits per
    block, which are not word multiples: sampled windows start on word
    boundaries, and the last one ends at the array's end."""
    import torch
    from cuzfp_gb300 import synth
    x = synth.random_walk_device((1 << 28) - 3, seed=2, dtype=torch.float32, device=cuda)
    run_workload(gz, orc, x, rate, np.random.default_rng(7), nregions=6, edge=4096)


@pytest.mark.parametrize("rate", [4.0, 12.0, 24.0])
def test_sinusoids_2d_full_size(gz, orc, cuda, rate):
    """2D float32 16381 x 16383 and float64 8191 x 8190, partial edge blocks."""
    import torch
    from cuzfp_gb300 import synth
    for shape, dt, seed in (((16383, 16381), torch.float32, 3), ((8190, 8191), torch.float64, 4)):
        x = synth.sinusoids_device(shape, 8, 64, seed=seed, dtype=dt, device=cuda)
        run_workload(gz, orc, x, rate, np.random.default_rng(seed), nregions=6, edge=64)
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
