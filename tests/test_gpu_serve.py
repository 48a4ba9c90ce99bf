"""Request server (gzfp_serve_run): every request's output is the same bits
whether it runs alone (a plain gzfp call) or in the server's mix of
batches; admission respects the device-memory budget; continuous batching
actually forms multi-request batches and overlaps them."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(gz, cuda, rng, count, max_edge, gap):
    """Mixed compress / decompress requests with resident inputs and a
    copy_to buffer each; returns (requests, expected outputs, copy buffers)."""
    import torch
    reqs, expect, outs = [], [], []
    t = 0.0
    for i in range(count):
        dims = int(rng.integers(1, 4))
        if dims == 1:
            shape = (int(rng.integers(1, max_edge ** 3)),)
        elif dims == 2:
            shape = tuple(int(v) for v in rng.integers(1, max_edge * 5, 2))
        else:
            shape = tuple(int(v) for v in rng.integers(1, max_edge, 3))
        dt = (torch.float32, torch.float64, torch.int32, torch.int64)[int(rng.integers(0, 4))]
        rate = float(rng.choice([4, 8, 12.5, 16, 32]))
        walk = np.cumsum(rng.standard_normal(int(np.prod(shape)))).reshape(shape)
        if not dt.is_floating_point:
            walk = walk * 5000
        x = torch.from_numpy(walk).to(dt).to(cuda)
        w = gz.compress_tensor(x, rate)  # alone
        t += float(rng.exponential(gap))
        if rng.random() < 0.5:
            out = torch.full_like(w, -1)
            reqs.append(gz.serve_request(gz.GZFP_SERVE_COMPRESS, x, rate, t, copy_to=out))
            expect.append(w)
        else:
            y = gz.decompress_tensor(w, shape, dt, rate)  # alone
            out = torch.full_like(y, float("nan") if dt.is_floating_point else -7)
            reqs.append(gz.serve_request(gz.GZFP_SERVE_DECOMPRESS, w, rate, t, shape=shape,
                                         dtype=dt, copy_to=out))
            expect.append(y)
        outs.append(out)
    torch.cuda.synchronize()
    return reqs, expect, outs


def _same(a, b):
    import torch
    if a.dtype == torch.float64:
        return torch.equal(a.view(torch.int64), b.view(torch.int64))
    if a.dtype == torch.float32:
        return torch.equal(a.view(torch.int32), b.view(torch.int32))
    return torch.equal(a, b)


def test_serve_alone_equals_mix(gz, cuda):
    """Slot mode: requests coded together in batches give the bits of plain
    calls, and requests share batches."""
    import torch
    rng = np.random.default_rng(101)
    reqs, expect, outs = _requests(gz, cuda, rng, 240, 48, 20e-6)
    cfg = gz.default_serve_config()
    cfg.device_queue = 0  # slots
    cfg.budget_bytes = 1 << 30
    cfg.max_inflight = 3
    res, stats = gz.serve(reqs, cfg)
    torch.cuda.synchronize()
    for i, (r, e, o) in enumerate(zip(res, expect, outs)):
        assert r.status == 0, i
        assert r.completed >= r.admitted >= reqs[i].arrival - 1e-9, i
        assert _same(e, o), (i, reqs[i].op, reqs[i].nx, reqs[i].ny, reqs[i].nz, reqs[i].maxbits)
    assert stats.batches < len(reqs) and stats.mean_batch > 1.0  # requests shared batches
    assert 0 < stats.peak_bytes <= cfg.budget_bytes


def test_serve_budget_and_fifo(gz, cuda):
    """A budget far below the offered outputs: requests wait for memory,
    results stay identical, the arena never exceeds the budget, and a request
    that can never fit is refused without stalling the rest."""
    import torch
    rng = np.random.default_rng(102)
    reqs, expect, outs = _requests(gz, cuda, rng, 120, 40, 0.0)  # all at once
    big = torch.zeros((160, 160, 160), dtype=torch.float64, device=cuda)  # 32 MiB output
    reqs.insert(60, gz.serve_request(gz.GZFP_SERVE_COMPRESS, big, 64.0, 0.0))
    cfg = gz.default_serve_config()
    cfg.device_queue = 0  # slots
    cfg.budget_bytes = 2 << 20
    cfg.max_batch = 8
    cfg.max_inflight = 2
    res, stats = gz.serve(reqs, cfg)
    torch.cuda.synchronize()
    assert res[60].status == gz.GZFP_ERR_CAPACITY
    rest = [r for i, r in enumerate(res) if i != 60]
    assert all(r.status == 0 for r in rest)
    for e, o in zip(expect, outs):
        assert _same(e, o)
    assert stats.peak_bytes <= cfg.budget_bytes
    assert stats.batches >= len(rest) / cfg.max_batch
    # FIFO: admission times follow arrival order (all arrivals are equal here,
    # so request order)
    adm = [r.admitted for r in rest]
    assert all(a <= b for a, b in zip(adm, adm[1:]))


def test_serve_bad_config(gz, cuda):
    import torch
    x = torch.zeros((8, 8, 8), dtype=torch.float32, device=cuda)
    req = gz.serve_request(gz.GZFP_SERVE_COMPRESS, x, 8.0, 0.0)
    cfg = gz.default_serve_config()
    assert cfg.device_queue == 1  # the default mode
    cfg.device_queue = 0
    cfg.max_inflight = 0
    with pytest.raises(gz.GzfpError):
        gz.serve([req], cfg)


# ------------------------------------------------------- device-queue mode

def _requests_3d(gz, cuda, rng, count, max_edge, gap, rates=(8.0, 12.5, 16.0, 32.0)):
    """3D float / double compress and decompress requests with resident
    inputs and a copy_to buffer each."""
    import torch
    reqs, expect, outs = [], [], []
    t = 0.0
    for _ in range(count):
        shape = tuple(int(v) for v in rng.integers(1, max_edge, 3))
        dt = torch.float32 if rng.random() < 0.5 else torch.float64
        rate = float(rng.choice(rates))
        walk = np.cumsum(rng.standard_normal(int(np.prod(shape)))).reshape(shape)
        x = torch.from_numpy(walk).to(dt).to(cuda)
        w = gz.compress_tensor(x, rate)  # alone
        t += float(rng.exponential(gap))
        if rng.random() < 0.5:
            out = torch.full_like(w, -1)
            reqs.append(gz.serve_request(gz.GZFP_SERVE_COMPRESS, x, rate, t, copy_to=out))
            expect.append(w)
        else:
            y = gz.decompress_tensor(w, shape, dt, rate)  # alone
            out = torch.full_like(y, float("nan"))
            reqs.append(gz.serve_request(gz.GZFP_SERVE_DECOMPRESS, w, rate, t, shape=shape,
                                         dtype=dt, copy_to=out))
            expect.append(y)
        outs.append(out)
    torch.cuda.synchronize()
    return reqs, expect, outs


def _queue_config(gz, **kw):
    cfg = gz.default_serve_config()
    cfg.device_queue = 1
    cfg.budget_bytes = 1 << 30
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def test_serve_queue_alone_equals_mix(gz, cuda):
    """Requests published to the running scheduler give the bits of plain
    calls, and the grids it launches overlap on the device."""
    import torch
    rng = np.random.default_rng(201)
    reqs, expect, outs = _requests_3d(gz, cuda, rng, 200, 72, 15e-6)
    res, stats = gz.serve(reqs, _queue_config(gz))
    torch.cuda.synchronize()
    for i, (r, e, o) in enumerate(zip(res, expect, outs)):
        assert r.status == 0, i
        assert r.completed >= r.admitted >= reqs[i].arrival - 1e-9, i
        assert r.device_end >= r.device_start >= 0.0, i
        assert _same(e, o), (i, reqs[i].op, reqs[i].nx, reqs[i].ny, reqs[i].nz, reqs[i].maxbits)
    # device-clock spans: some request's CTAs ran while another's did
    spans = sorted((r.device_start, r.device_end) for r in res)
    ends = np.maximum.accumulate([e for _, e in spans])
    assert any(spans[i + 1][0] < ends[i] for i in range(len(spans) - 1))
    assert stats.mean_inflight > 1.0
    assert stats.schedulers >= 1 and stats.kernels == stats.schedulers + len(reqs)
    assert 0 < stats.peak_bytes <= 1 << 30


def test_serve_queue_idle_limit(gz, cuda):
    """Arrival gaps far longer than the scheduler's wait limit: it leaves
    when the limit runs out (nothing published for idle_exit_us), the server
    starts a new one for the next request, and every result is still
    exact."""
    import torch
    rng = np.random.default_rng(202)
    reqs, expect, outs = _requests_3d(gz, cuda, rng, 12, 40, 0.0)
    for i, r in enumerate(reqs):
        r.arrival = 0.005 * i  # 5 ms apart
    res, stats = gz.serve(reqs, _queue_config(gz, idle_exit_us=200))
    torch.cuda.synchronize()
    assert all(r.status == 0 for r in res)
    for e, o in zip(expect, outs):
        assert _same(e, o)
    assert stats.schedulers >= 6  # the limit ran out between requests


def test_serve_queue_budget_and_fifo(gz, cuda):
    """A budget far below the offered outputs: requests wait for memory in
    arrival order, the arena never exceeds the budget, and a request that
    can never fit is refused without stalling the rest."""
    import torch
    rng = np.random.default_rng(203)
    reqs, expect, outs = _requests_3d(gz, cuda, rng, 100, 40, 0.0)
    big = torch.zeros((160, 160, 160), dtype=torch.float64, device=cuda)  # 32 MiB output
    reqs.insert(50, gz.serve_request(gz.GZFP_SERVE_COMPRESS, big, 64.0, 0.0))
    res, stats = gz.serve(reqs, _queue_config(gz, budget_bytes=2 << 20, max_batch=8))
    torch.cuda.synchronize()
    assert res[50].status == gz.GZFP_ERR_CAPACITY
    rest = [r for i, r in enumerate(res) if i != 50]
    assert all(r.status == 0 for r in rest)
    for e, o in zip(expect, outs):
        assert _same(e, o)
    assert stats.peak_bytes <= 2 << 20
    adm = [r.admitted for r in rest]
    assert all(a <= b for a, b in zip(adm, adm[1:]))


def test_serve_queue_every_kind(gz, cuda):
    """1D, 2D and 3D arrays of all four scalar types, rates whose blocks are
    and are not whole words: the device queue gives every request the bits
    of its plain call."""
    import torch
    rng = np.random.default_rng(204)
    reqs, expect, outs = _requests(gz, cuda, rng, 240, 48, 20e-6)
    res, stats = gz.serve(reqs, _queue_config(gz))
    torch.cuda.synchronize()
    for i, (r, e, o) in enumerate(zip(res, expect, outs)):
        assert r.status == 0, i
        assert _same(e, o), (i, reqs[i].op, reqs[i].type, reqs[i].nx, reqs[i].ny, reqs[i].nz,
                             reqs[i].maxbits)
    assert stats.kernels == stats.schedulers + len(reqs)


def test_serve_queue_bad_request(gz, cuda):
    import torch
    x = torch.zeros((8, 8, 8), dtype=torch.float32, device=cuda)
    req = gz.serve_request(gz.GZFP_SERVE_COMPRESS, x, 8.0, 0.0)
    req.maxbits = 3  # below the 9 bits of a float block's header
    with pytest.raises(gz.GzfpError):
        gz.serve([req], _queue_config(gz))
