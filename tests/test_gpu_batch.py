"""Batched path (grid and persistent kernels): every array of a mixed batch gets exactly the
stream (and decoded array) that the plain per-array path and the oracle
give; graph plans replay bit-identically; the autotuner returns a shape
that runs."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def mixed_batch(rng, count=40, ints=True):
    """Arrays of every dimensionality and scalar type (integers too unless
    `ints` is false), ragged shapes, rates whose blocks are and are not
    whole 64-bit words."""
    arrs, rates = [], []
    types = (np.float32, np.float64, np.int32, np.int64) if ints else (np.float32, np.float64)
    for i in range(count):
        dims = 1 + i % 3
        dt = types[int(rng.integers(0, len(types)))]
        if dims == 1:
            shape = (int(rng.integers(1, 3000)),)
        elif dims == 2:
            shape = tuple(int(v) for v in rng.integers(1, 90, 2))
        else:
            shape = tuple(int(v) for v in rng.integers(1, 40, 3))
        a = np.cumsum(rng.standard_normal(int(np.prod(shape)))).reshape(shape)
        a = (a * 5000).astype(dt) if np.dtype(dt).kind == "i" else a.astype(dt)
        arrs.append(a)
        rates.append(float(rng.choice([1, 2.5, 4, 8, 12, 16, 21.3, 32])))
    return arrs, rates


def test_batch_matches_plain_and_oracle(gz, orc, cuda):
    import torch
    rng = np.random.default_rng(77)
    arrs, rates = mixed_batch(rng)
    fields = [torch.from_numpy(a).to(cuda) for a in arrs]
    for cfg in (None, gz.BatchConfig(256, 0, 4, 0), gz.BatchConfig(64, 0, 2, 0),
                gz.BatchConfig(64, 2, 4, 0), gz.BatchConfig(256, 1, 2, 1),
                gz.BatchConfig(128, 16, 1, 1)):
        streams = gz.compress_batch(fields, rates, config=cfg)
        outs = [torch.empty_like(f) for f in fields]
        gz.decompress_batch(streams, outs, rates, config=cfg)
        torch.cuda.synchronize()
        for a, r, s, o in zip(arrs, rates, streams, outs):
            ref = orc.compress(a, r)
            assert np.array_equal(s.cpu().numpy().view(np.uint64), ref), (a.shape, a.dtype, r, cfg)
            dec = orc.decompress(ref, a.shape, a.dtype, r)
            assert np.array_equal(o.cpu().numpy().view(np.uint8), dec.view(np.uint8)), (a.shape, r)


def test_batch_plan_replays(gz, cuda):
    import torch
    rng = np.random.default_rng(78)
    arrs, rates = mixed_batch(rng, 24)
    fields = [torch.from_numpy(a).to(cuda) for a in arrs]
    plain = [gz.compress_tensor(f, r) for f, r in zip(fields, rates)]
    streams = gz.batch_stream_buffers(fields, rates)
    plan = gz.BatchPlan(fields, streams, rates)
    for _ in range(2):
        for s in streams:
            s.fill_(-1)
        plan.launch()
        torch.cuda.synchronize()
        for p, s in zip(plain, streams):
            assert torch.equal(p, s)
    outs = [torch.empty_like(f) for f in fields]
    dplan = gz.BatchPlan(outs, streams, rates, decompress=True)
    dplan.launch()
    torch.cuda.synchronize()
    for f, r, o in zip(fields, rates, outs):
        exp = gz.decompress_tensor(gz.compress_tensor(f, r), f.shape, f.dtype, r)
        bits = torch.int64 if exp.element_size() == 8 else torch.int32
        assert torch.equal(exp.view(bits), o.view(bits))
    plan.close()
    dplan.close()


def test_batch_autotune(gz, cuda):
    import torch
    rng = np.random.default_rng(79)
    arrs, rates = mixed_batch(rng, 12)
    fields = [torch.from_numpy(a).to(cuda) for a in arrs]
    streams = gz.batch_stream_buffers(fields, rates)
    cfg, ms = gz.autotune_batch(fields, streams, rates, repeats=1)
    assert cfg.threads in (64, 128, 256) and ms > 0
    gz.compress_batch(fields, rates, streams=streams, config=cfg)
    torch.cuda.synchronize()
    for f, r, s in zip(fields, rates, streams):
        assert torch.equal(gz.compress_tensor(f, r), s)


def test_batch_errors(gz, cuda):
    import torch
    f = torch.zeros((8, 8, 8), dtype=torch.float64, device=cuda)
    small = torch.zeros(3, dtype=torch.int64, device=cuda)
    with pytest.raises(gz.GzfpError) as e:
        gz.compress_batch([f], [16.0], streams=[small])
    assert e.value.status == gz.GZFP_ERR_CAPACITY
    with pytest.raises(gz.GzfpError):
        gz.compress_batch([f], [16.0], config=gz.BatchConfig(96, 1, 1, 0))
    with pytest.raises(gz.GzfpError):
        gz.compress_batch([f], [16.0], config=gz.BatchConfig(128, -1, 1, 0))
