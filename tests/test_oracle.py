"""The oracle (CPU restatement of zfp 0.5.0 fixed-rate mode) pinned against
the reference: its own zfp build, its regression checksums and fixed-rate
pins, and the committed golden streams.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from tests import cases, golden_io, zfp_pins


def test_oracle_matches_reference_random(ref):
    rng = np.random.default_rng(1234)
    checked = 0
    for _ in range(400):
        a, rate = cases.random_case(rng)
        if cases.has_saturating_blocks(a):
            continue
        s_ref = ref.ref_compress(a, rate)
        s_orc = ref.compress(a, rate)
        assert np.array_equal(s_ref, s_orc), (a.shape, a.dtype, rate)
        d_ref = ref.ref_decompress(s_ref, a.shape, a.dtype, rate)
        d_orc = ref.decompress(s_ref, a.shape, a.dtype, rate)
        assert np.array_equal(d_ref.view(np.uint8), d_orc.view(np.uint8)), (a.shape, rate)
        checked += 1
    assert checked > 300


def test_oracle_matches_reference_edges(ref):
    for a, rate in cases.edge_cases():
        if cases.has_saturating_blocks(a):
            continue
        s_ref = ref.ref_compress(a, rate)
        assert np.array_equal(s_ref, ref.compress(a, rate)), (a.shape, a.dtype, rate)
        d_ref = ref.ref_decompress(s_ref, a.shape, a.dtype, rate)
        assert np.array_equal(d_ref.view(np.uint8),
                              ref.decompress(s_ref, a.shape, a.dtype, rate).view(np.uint8))


def test_oracle_decodes_arbitrary_streams_like_reference(ref):
    """Random words are legal fixed-rate streams; both decoders must agree
    on them too (exercises budget cut-offs and the 'assumed one' rule)."""
    rng = np.random.default_rng(7)
    for dims, shape in ((1, (64,)), (2, (12, 12)), (3, (8, 8, 8))):
        for dt in (np.float32, np.float64):
            for rate in (1, 4, 9.5, 16, 40):
                n = ref.stream_bytes(shape, dt, rate) // 8
                w = rng.integers(0, 2 ** 63, n, dtype=np.int64).astype(np.uint64)
                w ^= rng.integers(0, 2, n, dtype=np.int64).astype(np.uint64) << np.uint64(63)
                d_ref = ref.ref_decompress(w, shape, dt, rate)
                d_orc = ref.decompress(w, shape, dt, rate)
                assert np.array_equal(d_ref.view(np.uint8), d_orc.view(np.uint8)), (shape, dt, rate)


def test_multithreaded_oracle_is_byte_identical(orc):
    rng = np.random.default_rng(5)
    for _ in range(20):
        a, rate = cases.random_case(rng, max_edge=(5000, 120, 30))
        s1 = orc.compress(a, rate, 1)
        for t in (2, 3, 7):
            assert np.array_equal(s1, orc.compress(a, rate, t))
            assert np.array_equal(orc.decompress(s1, a.shape, a.dtype, rate, 1).view(np.uint8),
                                  orc.decompress(s1, a.shape, a.dtype, rate, t).view(np.uint8))


def test_testzfp_fields_match_reference_fixture(ref):
    """The regenerated regression fields equal the reference's fixture."""
    fx = ref.ref_fields()
    if fx is None:
        pytest.skip("reference fields not built")
    for t, dt in enumerate((np.float32, np.float64)):
        for d in (1, 2, 3):
            assert np.array_equal(zfp_pins.field(dt, d).ravel(), fx[t][d - 1])


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_testzfp_checksums(dt, d):
    """Input checksums of Z/tests/testzfp.cpp:475-486 (Jenkins hash)."""
    f = zfp_pins.field(dt, d)
    assert zfp_pins.jenkins(f.tobytes()) == zfp_pins.CHECKSUM[np.dtype(dt).name][d - 1]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_testzfp_fixed_rate_pins(orc, dt, d):
    """Fixed-rate pins of Z/tests/testzfp.cpp:92-178 with the error table of
    :498-509: compressed size and max error."""
    f = zfp_pins.field(dt, d)
    for rate, tol in zfp_pins.rate_pins(dt, d):
        s = orc.compress(f, rate)
        # the test compares with the rate zfp_stream_set_rate reports back
        actual = orc.port().gzo_maxbits(orc.type_code(dt), d, rate) / 4 ** d
        assert s.nbytes == zfp_pins.expected_bytes(actual, f.size)
        g = orc.decompress(s, f.shape, f.dtype, rate)
        assert float(np.max(np.abs(f - g))) <= tol


def test_golden_streams(orc):
    """Committed streams and outputs made by the reference's own build."""
    n = 0
    for case in golden_io.load_all():
        s = orc.compress(case["input"], case["rate"])
        assert np.array_equal(s, case["stream"]), case["name"]
        d = orc.decompress(case["stream"], case["input"].shape, case["input"].dtype, case["rate"])
        assert np.array_equal(d.view(np.uint8), case["output"].view(np.uint8)), case["name"]
        n += 1
    assert n >= 10


def test_golden_manifest(orc):
    """Generated inputs (digest-checked) against the reference's digests."""
    from tests import golden_io
    for sp in golden_io.manifest():
        a = golden_io.generate(sp)
        assert golden_io.sha(a) == sp["input_sha256"], sp["name"]
        s = orc.compress(a, sp["rate"])
        assert s.nbytes == sp["stream_bytes"] and golden_io.sha(s) == sp["stream_sha256"], sp["name"]
        d = orc.decompress(s, a.shape, a.dtype, sp["rate"])
        assert golden_io.sha(d) == sp["output_sha256"], sp["name"]


def test_integer_oracle_matches_reference_block_api(orc, ref):
    """zfp 0.5.0 codes integer arrays only through its per-block API
    (zfp_encode_block_int32_<d> / int64), so arrays of whole blocks pin the
    restatement's integer path: streams and decoded arrays bit for bit."""
    rng = np.random.default_rng(31)
    for _ in range(150):
        a, rate = cases.int_case(rng, max_edge=(256, 32, 12), whole_blocks=True)
        if orc.stream_bytes(a.shape, a.dtype, rate) == 0:
            continue
        s = orc.compress(a, rate)
        r = orc.ref_compress(a, rate)
        assert np.array_equal(s, r), (a.shape, a.dtype, rate)
        assert np.array_equal(orc.decompress(s, a.shape, a.dtype, rate),
                              orc.ref_decompress(r, a.shape, a.dtype, rate)), (a.shape, rate)


def _views(rng):
    """Strided views of C-order arrays: slices, steps, transposes, reversals."""
    out = []
    for dt in (np.float32, np.float64, np.int32, np.int64):
        b3 = np.cumsum(rng.standard_normal((30, 26, 22)), axis=2)
        b3 = (b3 * 1000).astype(dt) if np.dtype(dt).kind == "i" else b3.astype(dt)
        b2 = b3[:, :, 0].copy()
        out += [b3[3:20, :, 5:9], b3[::2, 1::3, 2:], b3[1:, 2::2, ::3], b3[:, 7, :], b3[5, ::2, :],
                b3[2, 3, ::3], b2[::3, 1::2], b3.transpose(2, 1, 0), b3[::-1, ::-1, ::-1],
                b3.transpose(1, 0, 2)[::2], b2.T, b3[::-2, 3, :]]
    return out


def _zfp_valid(v) -> bool:
    """zfp 0.5.0 computes its strided offsets (sz - ny*sy, sy - nx*sx and the
    block steps) in unsigned arithmetic, so it reads out of bounds unless
    every stride is positive and each axis' stride covers the previous axis'
    extent -- sub-arrays and stepped slices of C-order arrays."""
    st = [s // v.itemsize for s in v.strides[::-1]]
    n = list(v.shape[::-1])
    if any(s <= 0 for s in st):
        return False
    return all(st[a] >= n[a - 1] * st[a - 1] for a in range(1, len(st)))


def _offset(v) -> int:
    """Element offset of v[0, ..., 0] in its base array."""
    base = v.base if v.base is not None else v
    return (v.__array_interface__["data"][0] - base.__array_interface__["data"][0]) // v.itemsize


def _flat_indices(v) -> np.ndarray:
    """Base-array element indices of every value of the view."""
    idx = np.zeros(v.shape, np.int64) + _offset(v)
    for ax, (n, st) in enumerate(zip(v.shape, v.strides)):
        sh = [1] * v.ndim
        sh[ax] = n
        idx = idx + (np.arange(n) * (st // v.itemsize)).reshape(sh)
    return idx.reshape(-1)


def test_strided_fields(orc):
    """zfp_field strides: the stream of a strided view is the stream of its
    contiguous copy, and decoding into a view touches only its values;
    where zfp 0.5.0's own strided path is valid the streams equal its."""
    rng = np.random.default_rng(41)
    ref_ok = orc.ref_available() or orc.build_ref()
    checked = 0
    for v in _views(rng):
        for rate in (2.0, 8.0, 13.5, 32.0):
            if orc.stream_bytes(v.shape, v.dtype, rate) == 0:
                continue
            s = orc.compress_view(v, rate)
            assert np.array_equal(s, orc.compress(np.ascontiguousarray(v), rate)), (v.shape, rate)
            if ref_ok and _zfp_valid(v) and np.dtype(v.dtype).kind == "f":  # zfp_compress: float, double
                assert np.array_equal(s, orc.ref_compress_view(v, rate)), (v.shape, v.strides, rate)
                checked += 1
            base = np.full(v.base.shape if v.base is not None else v.shape, 7, v.dtype)
            # the same view geometry over a fresh buffer
            w = np.lib.stride_tricks.as_strided(
                base.reshape(-1)[_offset(v):], shape=v.shape, strides=v.strides)
            orc.decompress_into(s, w, rate)
            assert np.array_equal(w, orc.decompress(s, v.shape, v.dtype, rate)), (v.shape, rate)
            untouched = np.ones(base.size, bool)
            untouched[_flat_indices(v)] = False
            assert np.all(base.reshape(-1)[untouched] == 7)
    if ref_ok:
        assert checked >= 20


# ----------------------------------------------------------- headed streams

def test_headed_golden_streams(orc):
    """The oracle's header + blocks equal the reference's zfp_write_header +
    zfp_compress streams in tests/golden/headed_cases.npz, and decode to the
    reference's output from the header alone."""
    cs = golden_io.headed_cases()
    assert len(cs) >= 16
    for c in cs:
        a = c["input"]
        s = orc.compress_headed(a, c["rate"])
        assert np.array_equal(s, c["stream"]), c["name"]
        h = orc.read_header(c["stream"])
        assert h["shape"] == a.shape and h["dtype"] == a.dtype, c["name"]
        assert np.array_equal(orc.decompress_headed(c["stream"]), c["output"]), c["name"]
        # the blocks are the plain stream's bits, shifted by the header
        plain = orc.compress(a, c["rate"])
        bits = np.unpackbits(s.view(np.uint8), bitorder="little")
        pbits = np.unpackbits(plain.view(np.uint8), bitorder="little")
        nb = orc.stream_bytes(a.shape, a.dtype, c["rate"]) * 8
        hb = h["bits"]
        blocks = int(np.prod([(n + 3) // 4 for n in a.shape]))
        used = blocks * h["maxbits"]
        assert np.array_equal(bits[hb:hb + used], pbits[:used]) and used <= nb, c["name"]


def test_headed_streams_match_reference(ref):
    rng = np.random.default_rng(71)
    n = 0
    for dt in (np.float32, np.float64, np.int32, np.int64):
        for shape in ((37,), (9, 13), (5, 6, 7), (64,), (16, 16), (8, 8, 8), (4, 4, 68)):
            if ref.is_int(dt) and any(s % 4 for s in shape):
                continue
            a = np.cumsum(rng.standard_normal(shape), axis=-1)
            a = (a * 1000).astype(dt) if ref.is_int(dt) else a.astype(dt)
            for rate in (1, 4, 12.5, 32, 64, 200):
                if ref.stream_bytes(a.shape, dt, rate) == 0 or ref.headed_bytes(a.shape, dt, rate) == 0:
                    continue
                s = ref.compress_headed(a, rate)
                assert np.array_equal(s, ref.ref_compress_headed(a, rate)), (dt, shape, rate)
                h, r = ref.read_header(s), ref.ref_read_header(s)
                assert h["bits"] == r["bits"] and h["maxbits"] == r["maxbits"] == r["minbits"]
                assert np.array_equal(ref.decompress_headed(s),
                                      ref.ref_decompress_headed(s, shape, dt, rate))
                n += 1
    assert n > 100


def _header_bits(fields):
    """Pack (value, nbits) fields LSB-first into three uint64 words."""
    v, pos = 0, 0
    for x, nb in fields:
        v |= (int(x) & ((1 << nb) - 1)) << pos
        pos += nb
    return np.frombuffer(v.to_bytes(24, "little"), np.uint64).copy()


def _magic():
    return [(ord("z"), 8), (ord("f"), 8), (ord("p"), 8), (5, 8)]


def _meta_3d_double(nx, ny, nz):
    m = ((((nz - 1) << 16) | (ny - 1)) << 16) | (nx - 1)
    return ((m << 4) | (2 << 2) | 3, 52)


def _long_mode(minbits, maxbits, maxprec, minexp):
    m = minexp + 16495
    m = (m << 7) | (maxprec - 1)
    m = (m << 15) | (maxbits - 1)
    m = (m << 15) | (minbits - 1)
    return ((m << 12) | 0xfff, 64)


HEADER_MODES = [
    # (mode field, accepted as fixed rate, maxbits)
    ((767, 12), True, 768),                       # 12-bit fixed rate
    ((2047 + 20, 12), False, 0),                  # fixed precision 20
    ((3251 - 30, 12), False, 0),                  # fixed accuracy 2^-30
    (_long_mode(700, 700, 64, -1074), True, 700),
    (_long_mode(600, 700, 64, -1074), False, 0),  # variable rate
    (_long_mode(700, 700, 40, -1074), False, 0),  # precision cap
    (_long_mode(700, 700, 64, -1000), False, 0),  # accuracy floor
]


@pytest.mark.parametrize("mode,ok,maxbits", HEADER_MODES)
def test_header_modes_oracle_and_reference(orc, mode, ok, maxbits):
    """Headers of zfp's other modes are recognised as not fixed rate; the
    reference reads the same parameters from them."""
    w = _header_bits(_magic() + [_meta_3d_double(40, 30, 20), mode])
    h = orc.read_header(w)
    if ok:
        assert h["bits"] in (96, 148) and h["maxbits"] == maxbits
        assert h["shape"] == (20, 30, 40) and h["dtype"] == np.float64
    else:
        assert h["bits"] == -1
    if orc.ref_available():
        r = orc.ref_read_header(w)
        assert r["bits"] == (96 if mode[1] == 12 else 148)
        assert (r["nx"], r["ny"], r["nz"], r["type"]) == (40, 30, 20, 4)
        assert (r["minbits"] == r["maxbits"] and r["maxprec"] >= 64 and r["minexp"] == -1074) == ok


def test_header_bad_magic(orc):
    w = _header_bits([(ord("z"), 8), (ord("f"), 8), (ord("q"), 8), (5, 8),
                      _meta_3d_double(4, 4, 4), (63, 12)])
    assert orc.read_header(w)["bits"] == 0
    w = _header_bits(_magic()[:3] + [(6, 8), _meta_3d_double(4, 4, 4), (63, 12)])
    assert orc.read_header(w)["bits"] == 0


# ------------------------------------------------------------- block access

def _block_case(orc, rng, dt, shape, rate):
    a = np.cumsum(rng.standard_normal(shape), axis=-1)
    a = (a * 1000).astype(dt) if orc.is_int(dt) else a.astype(dt)
    mb = int(orc.port().gzo_maxbits(orc.type_code(dt), a.ndim, float(rate)))
    return a, mb


BLOCK_SHAPES = ((37,), (9, 13), (5, 6, 7), (16,), (8, 12), (8, 8, 12))


def test_block_access_matches_reference(ref):
    """The oracle's per-block random access against the reference's own
    per-block API at the same slots: decoding in any order, encoding in any
    order for word-aligned slots and in stream order otherwise (zfp's
    stream_flush clears the rest of a slot's last word); both equal the
    whole-field codec."""
    rng = np.random.default_rng(91)
    n_cases = 0
    for dt in (np.float32, np.float64, np.int32, np.int64):
        for shape in BLOCK_SHAPES:
            if ref.is_int(dt) and any(s % 4 for s in shape):
                continue  # zfp 0.5.0 has no partial integer blocks
            for rate in (2, 8, 16.5, 32):
                if ref.stream_bytes(shape, dt, rate) == 0:
                    continue
                a, mb = _block_case(ref, rng, dt, shape, rate)
                d = a.ndim
                s = ref.compress(a, rate)
                tiles, codes = ref.field_tiles(a)
                ft, _ = ref.field_tiles(ref.decompress(s, a.shape, dt, rate))
                perm = rng.permutation(tiles.shape[0])
                got = ref.decode_blocks(s, dt, d, mb, perm, codes[perm])
                assert np.array_equal(got, ft[perm]), (dt, shape, rate)
                assert np.array_equal(ref.ref_decode_blocks(s, dt, d, mb, perm, codes[perm]),
                                      got), (dt, shape, rate)
                w = np.zeros_like(s)
                ref.encode_blocks(tiles[perm], d, mb, perm, w, codes[perm])
                assert np.array_equal(w, s), (dt, shape, rate)
                order = perm if mb % 64 == 0 else np.arange(tiles.shape[0])
                w2 = np.zeros_like(s)
                ref.ref_encode_blocks(tiles[order], d, mb, order, w2, codes[order])
                assert np.array_equal(w2, s), (dt, shape, rate)
                n_cases += 1
    assert n_cases > 40


def _block_of_each_value(shape):
    """zfp block index (x fastest) of every value of a C-ordered array."""
    nb = [(n + 3) // 4 for n in shape]
    idx = np.zeros(shape, np.int64)
    mult = 1
    for ax in range(len(shape) - 1, -1, -1):  # x (last axis) varies fastest
        sh = [1] * len(shape)
        sh[ax] = shape[ax]
        idx += (np.arange(shape[ax]) // 4).reshape(sh) * mult
        mult *= nb[ax]
    return idx


def test_block_rewrite_keeps_neighbours(orc):
    """Rewriting some blocks of a stream in place gives the stream of the
    modified field, for slots that share words with their neighbours too."""
    rng = np.random.default_rng(92)
    for dt, shape, rate in ((np.float32, (203,), 4.0), (np.float64, (21, 18), 7.0),
                            (np.float32, (9, 10, 11), 3.5), (np.int32, (40,), 12.0)):
        a, mb = _block_case(orc, rng, dt, shape, rate)
        assert mb % 64 != 0
        s = orc.compress(a, rate)
        nblocks = int(np.prod([(n + 3) // 4 for n in shape]))
        pick = rng.choice(nblocks, size=max(1, nblocks // 3), replace=False)
        b = a.copy()
        inside = np.isin(_block_of_each_value(shape), pick)
        b[inside] = (b[inside] * 3 + 1).astype(dt)  # change only the picked blocks
        tiles, codes = orc.field_tiles(b)
        changed = s.copy()
        orc.encode_blocks(tiles[pick], b.ndim, mb, pick, changed, codes[pick])
        assert np.array_equal(changed, orc.compress(b, rate)), (dt, shape)
        assert not np.array_equal(changed, s)


# ------------------------------------------- general parameters (zfp modes)

def _mode_list(orc, dt):
    ms = [orc.mode_precision(dt, p) for p in (3, 10, 24, 64)]
    ms += [orc.mode_accuracy(dt, t) for t in (1e-8, 1e-3, 0.5, 100.0)]
    ms += [(100, 300, 40, -30), (0, 64, 64, -1074), (200, 200, 64, -1074), (0, 4171, 16, -20)]
    lo = {np.float32: 9, np.float64: 12}.get(dt, 1)
    return [m for m in ms if m[1] >= lo]


def test_mode_setters_match_reference(ref):
    """zfp_stream_set_precision / _accuracy restated: the same four
    parameters for every type and a spread of arguments."""
    for dt in (np.float32, np.float64, np.int32, np.int64):
        for prec in (0, 1, 5, 12, 20, 31, 32, 40, 64, 100):
            assert ref.mode_precision(dt, prec) == ref.mode_precision(dt, prec, lib=ref.ref())
        for tol in (0, 1e-300, 1e-12, 1e-3, 0.1, 0.5, 1.0, 3.0, 1e10):
            assert ref.mode_accuracy(dt, tol) == ref.mode_accuracy(dt, tol, lib=ref.ref())


def test_general_params_match_reference(ref):
    """Fixed precision, fixed accuracy and other parameter sets: the oracle's
    variable-length streams equal zfp_compress's, and decode to
    zfp_decompress's arrays."""
    rng = np.random.default_rng(111)
    n = 0
    for dt in (np.float32, np.float64, np.int32, np.int64):
        for shape in ((37,), (9, 13), (5, 6, 7), (64,), (16, 16), (8, 8, 12)):
            if ref.is_int(dt) and any(s % 4 for s in shape):
                continue
            a = np.cumsum(rng.standard_normal(shape), axis=-1)
            a = (a * 1000).astype(dt) if ref.is_int(dt) else a.astype(dt)
            for pr in _mode_list(ref, dt):
                s, offs = ref.compress_params(a, pr, with_offsets=True)
                assert np.array_equal(s, ref.ref_compress_params(a, pr)), (dt, shape, pr)
                d, offs2 = ref.decompress_params(s, shape, dt, pr, with_offsets=True)
                assert np.array_equal(offs, offs2)
                assert np.array_equal(d, ref.ref_decompress_params(s, shape, dt, pr)), (dt, shape)
                n += 1
    assert n > 150


def test_general_params_golden(orc):
    cs = golden_io.mode_cases()
    assert len(cs) >= 12
    for c in cs:
        a = c["input"]
        s = orc.compress_params(a, c["params"])
        assert np.array_equal(s, c["stream"]), c["name"]
        assert np.array_equal(orc.decompress_params(c["stream"], a.shape, a.dtype, c["params"]),
                              c["output"]), c["name"]


def test_general_headers_match_reference(ref):
    """Headers of every mode -- the 12-bit fixed-precision and
    fixed-accuracy forms and the 64-bit form -- followed by the blocks, as
    zfp_write_header + zfp_compress write them; zfp_read_header's parameters
    read back."""
    rng = np.random.default_rng(131)
    for dt in (np.float32, np.float64):
        for shape in ((37,), (9, 13), (5, 6, 7)):
            a = np.cumsum(rng.standard_normal(shape), axis=-1).astype(dt)
            for pr in _mode_list(ref, dt):
                s = ref.compress_params_headed(a, pr)
                assert np.array_equal(s, ref.compress_params_headed(a, pr, lib=ref.ref())), pr
                h, r = ref.read_header_params(s), ref.ref_read_header(s)
                assert h["bits"] == r["bits"] and h["shape"] == shape
                assert h["params"] == (r["minbits"], r["maxbits"], r["maxprec"], r["minexp"])


def _random_params(rng, dt):
    lo = {np.float32: 9, np.float64: 12}.get(dt, 1)
    minbits = int(rng.choice([0, 0, int(rng.integers(1, 700))]))
    maxbits = int(max(lo, minbits, int(rng.integers(lo, 4500))))
    return (minbits, maxbits, int(rng.integers(1, 65)), int(rng.integers(-1100, 60)))


def test_random_params_match_reference(ref):
    """Random stream parameters (any minbits, maxbits, maxprec, minexp that
    zfp_stream_set_params accepts) on random fields: the oracle's streams
    are the reference's."""
    rng = np.random.default_rng(141)
    for k in range(120):
        dt = (np.float32, np.float64, np.int32, np.int64)[k % 4]
        d = 1 + int(rng.integers(0, 3))
        if ref.is_int(dt):
            shape = tuple(4 * int(v) for v in rng.integers(1, 6, d))
        else:
            shape = tuple(int(v) for v in rng.integers(1, 23, d))
        a = np.cumsum(rng.standard_normal(shape) * 10.0 ** rng.integers(-5, 5), axis=-1)
        a = (a * 1000).astype(dt) if ref.is_int(dt) else a.astype(dt)
        pr = _random_params(rng, dt)
        s = ref.compress_params(a, pr)
        assert np.array_equal(s, ref.ref_compress_params(a, pr)), (dt, shape, pr)
        assert np.array_equal(ref.decompress_params(s, shape, dt, pr),
                              ref.ref_decompress_params(s, shape, dt, pr)), (dt, shape, pr)
