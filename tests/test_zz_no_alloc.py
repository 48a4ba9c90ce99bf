"""gzfp_batch_run_noalloc through the C ABI: two calls in a row give the
streams and decoded arrays of the allocating batch entry points, allocate
no device memory, and reject batches larger than the fixed work list.

The file name sorts last so that the suite also runs it after every other
GPU test (the work list then starts from whatever earlier calls left)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ITEMS = 1024


def _bind(gz):
    fn = gz._lib.gzfp_batch_run_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(gz.BatchItem), ctypes.c_int, ctypes.c_int,
                   ctypes.POINTER(gz.BatchConfig), ctypes.c_void_p]
    return fn


def _batch(rng, count):
    arrs, rates = [], []
    for i in range(count):
        dims = 1 + i % 3
        dt = (np.float32, np.float64, np.int32, np.int64)[int(rng.integers(0, 4))]
        if dims == 1:
            shape = (int(rng.integers(1, 5000)),)
        elif dims == 2:
            shape = tuple(int(v) for v in rng.integers(1, 120, 2))
        else:
            shape = tuple(int(v) for v in rng.integers(1, 50, 3))
        a = np.cumsum(rng.standard_normal(int(np.prod(shape)))).reshape(shape)
        a = (a * 5000).astype(dt) if np.dtype(dt).kind == "i" else a.astype(dt)
        arrs.append(a)
        rates.append(float(rng.choice([1, 3, 4, 8, 13.5, 16, 32])))
    return arrs, rates


def _bits(t):
    import torch
    return t.view(torch.int64 if t.element_size() == 8 else torch.int32)


def test_noalloc_matches_batch_entry_points(gz, cuda):
    import torch
    run = _bind(gz)
    cfgs = [None, gz.BatchConfig(64, 3, 2, 0), gz.BatchConfig(256, 0, 4, 0)]
    for call, (seed, count) in enumerate(((11, 30), (12, 17))):
        rng = np.random.default_rng(seed)
        arrs, rates = _batch(rng, count)
        fields = [torch.from_numpy(a).to(cuda) for a in arrs]
        cfg = cfgs[call]
        cref = ctypes.byref(cfg) if cfg is not None else None
        # the allocating entry points: the expected bits
        exp_s = gz.compress_batch(fields, rates, config=cfg)
        exp_o = [torch.empty_like(f) for f in fields]
        gz.decompress_batch(exp_s, exp_o, rates, config=cfg)
        got_s = gz.batch_stream_buffers(fields, rates)
        for s in got_s:
            s.fill_(-1)  # anything the kernel leaves unwritten shows
        got_o = [torch.full_like(f, float("nan") if f.is_floating_point() else -7)
                 for f in fields]
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        items = gz.batch_items(fields, got_s, rates)
        assert run(items, len(items), 0, cref, None) == 0, gz._lib.gzfp_batch_last_error()
        items = gz.batch_items(got_o, got_s, rates)
        assert run(items, len(items), 1, cref, None) == 0
        torch.cuda.synchronize()
        for i, (a, b) in enumerate(zip(exp_s, got_s)):
            assert torch.equal(a, b), (call, i, arrs[i].shape, arrs[i].dtype, rates[i])
        for i, (a, b) in enumerate(zip(exp_o, got_o)):
            assert torch.equal(_bits(a), _bits(b)), (call, i, arrs[i].shape, rates[i])
        if call == 1:
            # the work list is static: the second call takes no device memory
            assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_rejects_oversized_batches(gz, cuda):
    import torch
    run = _bind(gz)
    f = torch.zeros((4, 4, 4), dtype=torch.float32, device=cuda)
    w = torch.zeros(64, dtype=torch.int64, device=cuda)
    items = gz.batch_items([f] * (MAX_ITEMS + 1), [w] * (MAX_ITEMS + 1), [8.0] * (MAX_ITEMS + 1))
    assert run(items, len(items), 0, None, None) == gz.GZFP_ERR_CAPACITY
    assert b"1024 arrays" in gz._lib.gzfp_batch_last_error()
    # too many chunks: 2^19 chunks of 64 blocks = 2^25 blocks; a 1D float
    # array of 2^27 + 4 values has 2^25 + 1 blocks.  The buffers are full
    # size, so nothing would run out of bounds even if the check were missing.
    n = (1 << 27) + 4
    big_f = torch.zeros(n, dtype=torch.float32, device=cuda)
    big_w = torch.zeros(n // 4, dtype=torch.int64, device=cuda)
    one = gz.batch_items([big_f], [big_w], [16.0])
    assert one[0].maxbits == 64
    cfg = gz.BatchConfig(64, 1, 1, 0)
    assert run(one, 1, 0, ctypes.byref(cfg), None) == gz.GZFP_ERR_CAPACITY
    assert b"chunks" in gz._lib.gzfp_batch_last_error()


def test_noalloc_rejects_stream_capture(gz, cuda):
    """A call on a capturing stream is refused before any work is queued
    (a captured pageable upload from the shared host array would replay
    whatever a later call left there); the capture itself still ends
    cleanly."""
    import torch
    run = _bind(gz)
    f = torch.zeros((16, 16, 16), dtype=torch.float32, device=cuda)
    w = gz.batch_stream_buffers([f], [8.0])
    items = gz.batch_items([f], w, [8.0])
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        st = run(items, 1, 0, None, ctypes.c_void_p(s.cuda_stream))
        f.add_(1.0)  # the capture records something of its own
    assert st == gz.GZFP_ERR_ARG
    assert b"captured" in gz._lib.gzfp_batch_last_error()
    g.replay()
    torch.cuda.synchronize()
    assert float(f[0, 0, 0]) == 1.0  # the captured add ran once, at the replay
