"""Headed streams on the GPU: gzfp_compress_headed writes zfp's full header
(zfp_write_header with ZFP_HEADER_FULL) and the blocks right after it, bit
for bit the reference's stream; gzfp_decompress_headed takes the field's
type and shape from the header."""
from __future__ import annotations

import numpy as np
import pytest

from tests import golden_io

pytestmark = pytest.mark.gpu


def test_golden_device_and_host(gz, orc, cuda):
    import torch
    for c in golden_io.headed_cases():
        a = c["input"]
        # device buffers
        t = torch.from_numpy(a).to(cuda)
        w = gz.compress_headed(t, c["rate"])
        torch.cuda.synchronize()
        assert np.array_equal(w.cpu().numpy().view(np.uint64), c["stream"]), c["name"]
        sw = torch.from_numpy(c["stream"].view(np.int64)).to(cuda)
        out = gz.decompress_headed(sw)
        torch.cuda.synchronize()
        assert out.shape == a.shape and np.array_equal(out.cpu().numpy(), c["output"]), c["name"]
        # host buffers
        hw = gz.compress_headed(a, c["rate"])
        assert np.array_equal(hw, c["stream"]), c["name"]
        assert np.array_equal(gz.decompress_headed(c["stream"]), c["output"]), c["name"]


@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "int64"])
def test_random_against_oracle(gz, orc, cuda, dt):
    import torch
    rng = np.random.default_rng(81)
    for shape in ((1000,), (1,), (77, 45), (33, 18, 29), (64, 64, 64)):
        a = np.cumsum(rng.standard_normal(shape), axis=-1)
        a = (a * 3000).astype(dt) if dt.startswith("int") else a.astype(dt)
        for rate in (1.0, 7.25, 16.0, 40.0):
            if orc.stream_bytes(a.shape, a.dtype, rate) == 0:
                continue
            s = orc.compress_headed(a, rate)
            w = gz.compress_headed(torch.from_numpy(a).to(cuda), rate)
            torch.cuda.synchronize()
            assert np.array_equal(w.cpu().numpy().view(np.uint64), s), (shape, rate)
            got = gz.decompress_headed(w)
            torch.cuda.synchronize()
            assert np.array_equal(got.cpu().numpy(), orc.decompress_headed(s)), (shape, rate)


def test_large_field_round_trip(gz, orc, cuda):
    """A field larger than L2 with a header: decode(encode(x)) is the
    oracle's decode of the oracle-checked plain stream, and the blocks after
    the header equal the plain stream's."""
    import torch
    from cuzfp_gb300 import synth
    a = synth.smooth_noisy_3d(256, 5, np.float64)
    t = torch.from_numpy(a).to(cuda)
    w = gz.compress_headed(t, 16.0)
    plain = gz.compress_tensor(t, 16.0)
    torch.cuda.synchronize()
    h = gz.read_header(w)
    assert h["bits"] == 96 and h["maxbits"] == 1024 and h["shape"] == a.shape
    wb = w.cpu().numpy().view(np.uint64)
    pb = plain.cpu().numpy().view(np.uint64)
    # shift the headed words down by the 96 header bits and compare
    shifted = (wb[1:-1] >> np.uint64(32)) | (wb[2:] << np.uint64(32))
    assert np.array_equal(shifted[: pb.size], pb)
    out = gz.decompress_headed(w)
    ref = gz.decompress_tensor(plain, a.shape, t.dtype, 16.0)
    torch.cuda.synchronize()
    assert torch.equal(out, ref)


def test_errors(gz, cuda):
    import torch
    a = torch.zeros(16, 16, dtype=torch.float32, device=cuda)
    w = gz.compress_headed(a, 8.0)
    small = torch.empty(15, 16, dtype=torch.float32, device=cuda)
    with pytest.raises(gz.GzfpError) as e:
        gz.decompress_headed(w, out=small)
    assert e.value.status == gz.GZFP_ERR_CAPACITY
    with pytest.raises(gz.GzfpError) as e:
        gz.decompress_headed(w[:3])  # header only, no blocks
    assert e.value.status == gz.GZFP_ERR_ARG
    with pytest.raises(gz.GzfpError) as e:
        gz.compress_headed(a, 8.0, out=torch.empty(3, dtype=torch.int64, device=cuda))
    assert e.value.status == gz.GZFP_ERR_CAPACITY
