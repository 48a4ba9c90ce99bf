"""Random access to single blocks on the GPU through the C ABI
(gzfp_decode_blocks / gzfp_encode_blocks): listed blocks decode to the
oracle's tiles, rewritten slots give the oracle's stream and keep their
neighbours' bits, host and device buffers alike."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = ((203,), (37, 29), (9, 10, 11), (64,), (16, 20), (12, 8, 16))


def _case(orc, rng, dt, shape, rate):
    a = np.cumsum(rng.standard_normal(shape), axis=-1)
    a = (a * 3000).astype(dt) if orc.is_int(dt) else a.astype(dt)
    mb = int(orc.port().gzo_maxbits(orc.type_code(dt), a.ndim, float(rate)))
    return a, mb


@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "int64"])
def test_decode_listed_blocks(gz, orc, cuda, dt):
    import torch
    rng = np.random.default_rng(101)
    for shape in SHAPES:
        for rate in (3.0, 8.0, 16.5, 32.0):
            if orc.stream_bytes(shape, dt, rate) == 0:
                continue
            a, mb = _case(orc, rng, dt, shape, rate)
            s = orc.compress(a, rate)
            tiles, codes = orc.field_tiles(a)
            n = tiles.shape[0]
            idx = np.concatenate([rng.permutation(n), rng.integers(0, n, 7)])  # repeats are fine
            exp = orc.decode_blocks(s, dt, a.ndim, mb, idx, codes[idx],
                                    tiles=np.full((idx.size, 4 ** a.ndim), 5, dt))
            ws = torch.from_numpy(s.view(np.int64)).to(cuda)
            out = torch.full((idx.size, 4 ** a.ndim), 5, dtype=getattr(torch, dt), device=cuda)
            gz.decode_blocks(ws, out.dtype, a.ndim, mb, idx.astype(np.int64), codes[idx], out=out)
            torch.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy(), exp), (shape, rate)
            # host buffers
            hout = gz.decode_blocks(s, np.dtype(dt), a.ndim, mb, idx, codes[idx],
                                    out=np.full((idx.size, 4 ** a.ndim), 5, dt))
            assert np.array_equal(hout, exp), (shape, rate)


@pytest.mark.parametrize("dt", ["float32", "float64", "int32", "int64"])
def test_encode_listed_blocks(gz, orc, cuda, dt):
    """Every block written in a random order gives the whole-field stream;
    rewriting a third of the blocks of a modified field gives the modified
    field's stream, including slots that share words."""
    import torch
    from tests.test_oracle import _block_of_each_value
    rng = np.random.default_rng(102)
    for shape in SHAPES:
        for rate in (3.0, 8.0, 16.5, 32.0):
            if orc.stream_bytes(shape, dt, rate) == 0:
                continue
            a, mb = _case(orc, rng, dt, shape, rate)
            s = orc.compress(a, rate)
            tiles, codes = orc.field_tiles(a)
            n = tiles.shape[0]
            perm = rng.permutation(n)
            w = torch.zeros(s.size, dtype=torch.int64, device=cuda)
            gz.encode_blocks(torch.from_numpy(tiles[perm]).to(cuda), a.ndim, mb,
                             perm.astype(np.int64), w, codes[perm])
            torch.cuda.synchronize()
            assert np.array_equal(w.cpu().numpy().view(np.uint64), s), (shape, rate)
            # rewrite
            pick = rng.choice(n, size=max(1, n // 3), replace=False)
            b = a.copy()
            inside = np.isin(_block_of_each_value(shape), pick)
            b[inside] = (b[inside] * 3 + 1).astype(dt)
            bt, _ = orc.field_tiles(b)
            gz.encode_blocks(torch.from_numpy(bt[pick]).to(cuda), a.ndim, mb,
                             pick.astype(np.int64), w, codes[pick])
            torch.cuda.synchronize()
            assert np.array_equal(w.cpu().numpy().view(np.uint64), orc.compress(b, rate)), \
                (shape, rate)
            # host buffers: the same rewrite on a host copy of the first stream
            hw = s.copy()
            gz.encode_blocks(bt[pick], a.ndim, mb, pick, hw, codes[pick])
            assert np.array_equal(hw, orc.compress(b, rate)), (shape, rate)


def test_indices_past_the_stream_are_skipped(gz, orc, cuda):
    import torch
    rng = np.random.default_rng(103)
    a, mb = _case(orc, rng, "float64", (8, 8, 8), 16.0)
    s = orc.compress(a, 16.0)
    tiles, codes = orc.field_tiles(a)
    ws = torch.from_numpy(s.view(np.int64)).to(cuda)
    idx = np.array([1, 8, 1 << 40, 3], np.int64)  # 8 blocks in the stream
    out = torch.full((4, 64), 7.0, dtype=torch.float64, device=cuda)
    gz.decode_blocks(ws, torch.float64, 3, mb, idx, None, out=out)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    ft, _ = orc.field_tiles(orc.decompress(s, a.shape, a.dtype, 16.0))
    assert np.array_equal(o[0], ft[1]) and np.array_equal(o[3], ft[3])
    assert np.all(o[1] == 7.0) and np.all(o[2] == 7.0)
    before = ws.clone()
    gz.encode_blocks(torch.from_numpy(tiles[:4] * 2).to(cuda), 3, mb, idx, ws, None)
    torch.cuda.synchronize()
    after = ws.cpu().numpy().view(np.uint64)
    exp = s.copy()
    orc.encode_blocks(tiles[:4] * 2, 3, mb, idx, exp, None)
    assert np.array_equal(after, exp)
    assert not torch.equal(before, ws)


def test_block_errors(gz, cuda):
    import torch
    w = torch.zeros(16, dtype=torch.int64, device=cuda)
    with pytest.raises(gz.GzfpError) as e:
        gz.decode_blocks(w, torch.float32, 4, 64, [0])
    assert e.value.status == gz.GZFP_ERR_ARG
    with pytest.raises(gz.GzfpError) as e:
        gz.decode_blocks(w, torch.float32, 3, 8, [0])  # under the block header
    assert e.value.status == gz.GZFP_ERR_ARG
    with pytest.raises(gz.GzfpError) as e:
        gz.decode_blocks(w, torch.float32, 3, 64, [0, 1], shapes=[0])
    assert e.value.status == gz.GZFP_ERR_ARG
