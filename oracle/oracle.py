"""Python access to the parity checkers (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module.  It wraps:

* the CPU restatement of zfp 0.5.0 fixed-rate mode (oracle/zfp_oracle.c,
  built to oracle/_build/libzfp_oracle.so by ``make -C oracle port``), and
* when present, the reference's own zfp 0.5.0 compiled from the reference
  tree (oracle/_ref/libzfpref.so, ``make -C oracle ref``), plus its
  regression fields (oracle/_ref/libzfpfields.so).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libzfp_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libzfpref.so")
FIELDS_LIB = os.path.join(HERE, "_ref", "libzfpfields.so")
# the cuZFP checkout: GZFP_REFERENCE_ROOT, else a checkout named `reference`
# beside this repository
REF_TREE = os.environ.get("GZFP_REFERENCE_ROOT",
                          os.path.abspath(os.path.join(HERE, "..", "..", "reference")))

INT32, INT64, FLOAT, DOUBLE = 1, 2, 3, 4  # zfp_type (Z/inc/zfp.h:107-113)

_A = [ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_double]


def build_port() -> str:
    """Compile the restatement (gcc); returns the library path."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def build_ref() -> bool:
    """Compile the reference's zfp sources when the reference tree exists."""
    if not os.path.isdir(os.path.join(REF_TREE, "src", "thirdparty_builtin", "zfp-0.5.0")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", "fields", f"REF_ROOT={REF_TREE}"], check=True)
    return True


_port = None
_ref = None


def port() -> ctypes.CDLL:
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB) or (
                os.path.getmtime(PORT_LIB) < os.path.getmtime(os.path.join(HERE, "zfp_oracle.c"))):
            build_port()
        lib = ctypes.CDLL(PORT_LIB)
        lib.gzo_compress.restype = ctypes.c_size_t
        lib.gzo_compress.argtypes = _A + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                          ctypes.c_int]
        lib.gzo_decompress.restype = ctypes.c_int
        lib.gzo_decompress.argtypes = _A + [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                            ctypes.c_int]
        lib.gzo_stream_bytes.restype = ctypes.c_size_t
        lib.gzo_stream_bytes.argtypes = _A
        lib.gzo_maxbits.restype = ctypes.c_uint
        lib.gzo_maxbits.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double]
        _L = [ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_longlong,
              ctypes.c_longlong, ctypes.c_longlong, ctypes.c_double]
        lib.gzo_compress_strided.restype = ctypes.c_size_t
        lib.gzo_compress_strided.argtypes = _L + [ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_size_t, ctypes.c_int]
        lib.gzo_decompress_strided.restype = ctypes.c_int
        lib.gzo_decompress_strided.argtypes = _L + [ctypes.c_void_p, ctypes.c_size_t,
                                                    ctypes.c_void_p, ctypes.c_int]
        lib.gzo_header_bits.restype = ctypes.c_uint
        lib.gzo_header_bits.argtypes = _A
        lib.gzo_compress_headed.restype = ctypes.c_size_t
        lib.gzo_compress_headed.argtypes = _A + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        _P = ctypes.POINTER
        lib.gzo_read_header.restype = ctypes.c_long
        lib.gzo_read_header.argtypes = [ctypes.c_void_p, ctypes.c_size_t, _P(ctypes.c_int),
                                        _P(ctypes.c_uint), _P(ctypes.c_uint), _P(ctypes.c_uint),
                                        _P(ctypes.c_uint)]
        lib.gzo_decompress_headed.restype = ctypes.c_int
        lib.gzo_decompress_headed.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                              ctypes.c_size_t]
        _B = [ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        _IDX = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]  # indices, shapes, count
        lib.gzo_decode_blocks.restype = ctypes.c_int
        lib.gzo_decode_blocks.argtypes = _B + [ctypes.c_void_p, ctypes.c_size_t] + _IDX + \
            [ctypes.c_void_p]
        lib.gzo_encode_blocks.restype = ctypes.c_int
        lib.gzo_encode_blocks.argtypes = _B + [ctypes.c_void_p] + _IDX + [ctypes.c_void_p,
                                                                          ctypes.c_size_t]
        _PR = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_int]  # minbits..minexp
        _PP = [ctypes.POINTER(ctypes.c_uint)] * 3 + [ctypes.POINTER(ctypes.c_int)]
        lib.gzo_mode_precision.restype = None
        lib.gzo_mode_precision.argtypes = [ctypes.c_int, ctypes.c_uint] + _PP
        lib.gzo_mode_accuracy.restype = None
        lib.gzo_mode_accuracy.argtypes = [ctypes.c_int, ctypes.c_double] + _PP
        _F = [ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint] + _PR
        lib.gzo_bound_params.restype = ctypes.c_size_t
        lib.gzo_bound_params.argtypes = _F
        lib.gzo_compress_params.restype = ctypes.c_size_t
        lib.gzo_compress_params.argtypes = _F + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                 ctypes.c_void_p]
        lib.gzo_compress_params_headed.restype = ctypes.c_size_t
        lib.gzo_compress_params_headed.argtypes = _F + [ctypes.c_void_p, ctypes.c_void_p,
                                                        ctypes.c_size_t]
        lib.gzo_read_header_params.restype = ctypes.c_long
        lib.gzo_read_header_params.argtypes = [ctypes.c_void_p, ctypes.c_size_t,
                                               ctypes.POINTER(ctypes.c_int)] + \
            [ctypes.POINTER(ctypes.c_uint)] * 3 + _PP
        lib.gzo_decompress_params.restype = ctypes.c_int
        lib.gzo_decompress_params.argtypes = _F + [ctypes.c_void_p, ctypes.c_size_t,
                                                   ctypes.c_void_p, ctypes.c_void_p]
        _port = lib
    return _port


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_LIB)
        lib.zref_compress.restype = ctypes.c_size_t
        lib.zref_compress.argtypes = _A + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        lib.zref_decompress.restype = ctypes.c_int
        lib.zref_decompress.argtypes = _A + [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        lib.zref_maximum_size.restype = ctypes.c_size_t
        lib.zref_maximum_size.argtypes = _A
        lib.zref_set_rate_bits.restype = ctypes.c_uint
        lib.zref_set_rate_bits.argtypes = [ctypes.c_int, ctypes.c_uint, ctypes.c_double]
        _S = [ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_int,
              ctypes.c_int, ctypes.c_int, ctypes.c_double]
        lib.zref_compress_strided.restype = ctypes.c_size_t
        lib.zref_compress_strided.argtypes = _S + [ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_size_t]
        lib.zref_decompress_strided.restype = ctypes.c_int
        lib.zref_decompress_strided.argtypes = _S + [ctypes.c_void_p, ctypes.c_size_t,
                                                     ctypes.c_void_p]
        lib.zref_compress_int.restype = ctypes.c_size_t
        lib.zref_compress_int.argtypes = _A + [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        lib.zref_decompress_int.restype = ctypes.c_int
        lib.zref_decompress_int.argtypes = _A + [ctypes.c_void_p, ctypes.c_size_t,
                                                 ctypes.c_void_p]
        lib.zref_compress_headed.restype = ctypes.c_size_t
        lib.zref_compress_headed.argtypes = _A + [ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_size_t]
        _P = ctypes.POINTER
        lib.zref_read_header.restype = ctypes.c_size_t
        lib.zref_read_header.argtypes = [ctypes.c_void_p, ctypes.c_size_t, _P(ctypes.c_int),
                                         _P(ctypes.c_uint), _P(ctypes.c_uint), _P(ctypes.c_uint),
                                         _P(ctypes.c_uint), _P(ctypes.c_uint), _P(ctypes.c_uint),
                                         _P(ctypes.c_int)]
        lib.zref_decompress_headed.restype = ctypes.c_int
        lib.zref_decompress_headed.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        lib.zref_decompress_headed_int.restype = ctypes.c_int
        lib.zref_decompress_headed_int.argtypes = _A + [ctypes.c_void_p, ctypes.c_size_t,
                                                        ctypes.c_void_p]
        _B = [ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        _IDX = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        lib.zref_decode_blocks.restype = ctypes.c_int
        lib.zref_decode_blocks.argtypes = _B + [ctypes.c_void_p, ctypes.c_size_t] + _IDX + \
            [ctypes.c_void_p]
        lib.zref_encode_blocks.restype = ctypes.c_int
        lib.zref_encode_blocks.argtypes = _B + [ctypes.c_void_p] + _IDX + [ctypes.c_void_p,
                                                                           ctypes.c_size_t]
        _PR = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_int]
        _PP = [ctypes.POINTER(ctypes.c_uint)] * 3 + [ctypes.POINTER(ctypes.c_int)]
        _F = [ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint] + _PR
        lib.zref_compress_params.restype = ctypes.c_size_t
        lib.zref_compress_params.argtypes = _F + [ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_size_t]
        lib.zref_decompress_params.restype = ctypes.c_int
        lib.zref_decompress_params.argtypes = _F + [ctypes.c_void_p, ctypes.c_size_t,
                                                    ctypes.c_void_p]
        lib.zref_compress_params_headed.restype = ctypes.c_size_t
        lib.zref_compress_params_headed.argtypes = _F + [ctypes.c_void_p, ctypes.c_void_p,
                                                         ctypes.c_size_t]
        lib.zref_set_precision.restype = None
        lib.zref_set_precision.argtypes = [ctypes.c_int, ctypes.c_uint] + _PP
        lib.zref_set_accuracy.restype = None
        lib.zref_set_accuracy.argtypes = [ctypes.c_int, ctypes.c_double] + _PP
        _ref = lib
    return _ref


def type_code(dtype) -> int:
    dt = np.dtype(dtype)
    if dt == np.float32:
        return FLOAT
    if dt == np.float64:
        return DOUBLE
    if dt == np.int32:
        return INT32
    if dt == np.int64:
        return INT64
    raise ValueError(f"unsupported dtype {dt}")


def is_int(dtype) -> bool:
    return np.dtype(dtype) in (np.dtype(np.int32), np.dtype(np.int64))


def dims3(shape) -> tuple[int, int, int]:
    s = tuple(int(v) for v in shape)[::-1]
    return (s + (0, 0))[:3]


def stream_bytes(shape, dtype, rate: float) -> int:
    nx, ny, nz = dims3(shape)
    return int(port().gzo_stream_bytes(type_code(dtype), nx, ny, nz, float(rate)))


def compress(a: np.ndarray, rate: float, nthreads: int = 1) -> np.ndarray:
    """Oracle stream (uint64 words) of a C-contiguous 1-3D float array."""
    a = np.ascontiguousarray(a)
    nx, ny, nz = dims3(a.shape)
    n = stream_bytes(a.shape, a.dtype, rate)
    out = np.zeros(max(n // 8, 1), np.uint64)
    got = port().gzo_compress(type_code(a.dtype), nx, ny, nz, float(rate), a.ctypes.data,
                              out.ctypes.data, out.nbytes, int(nthreads))
    if got != n:
        raise RuntimeError("oracle compress failed")
    return out[: n // 8]


def decompress(words: np.ndarray, shape, dtype, rate: float, nthreads: int = 1) -> np.ndarray:
    words = np.ascontiguousarray(words, dtype=np.uint64)
    out = np.zeros(tuple(shape), dtype)
    nx, ny, nz = dims3(shape)
    ok = port().gzo_decompress(type_code(dtype), nx, ny, nz, float(rate), words.ctypes.data,
                               words.nbytes, out.ctypes.data, int(nthreads))
    if not ok:
        raise RuntimeError("oracle decompress failed")
    return out


def ref_compress(a: np.ndarray, rate: float) -> np.ndarray:
    """Stream produced by the reference's own zfp 0.5.0 build (integer
    arrays: its per-block integer API, whole blocks only)."""
    a = np.ascontiguousarray(a)
    nx, ny, nz = dims3(a.shape)
    t = type_code(a.dtype)
    if is_int(a.dtype):
        n = stream_bytes(a.shape, a.dtype, rate)
        buf = np.zeros(max(n // 8, 1), np.uint64)
        got = ref().zref_compress_int(t, nx, ny, nz, float(rate), a.ctypes.data,
                                      buf.ctypes.data, buf.nbytes)
        if got != n:
            raise RuntimeError("reference integer compress failed (sizes must be multiples of 4)")
        return buf[: n // 8]
    cap = int(ref().zref_maximum_size(t, nx, ny, nz, float(rate)))
    buf = np.zeros(cap // 8 + 1, np.uint64)
    n = ref().zref_compress(t, nx, ny, nz, float(rate), a.ctypes.data, buf.ctypes.data, cap)
    return buf[: n // 8]


def ref_decompress(words: np.ndarray, shape, dtype, rate: float) -> np.ndarray:
    words = np.ascontiguousarray(words, dtype=np.uint64)
    out = np.zeros(tuple(shape), dtype)
    nx, ny, nz = dims3(shape)
    if is_int(dtype):
        if not ref().zref_decompress_int(type_code(dtype), nx, ny, nz, float(rate),
                                         words.ctypes.data, words.nbytes, out.ctypes.data):
            raise RuntimeError("reference integer decompress failed")
        return out
    ref().zref_decompress(type_code(dtype), nx, ny, nz, float(rate), words.ctypes.data,
                          words.nbytes, out.ctypes.data)
    return out


def ref_fields():
    """The reference's regression input arrays (Z/tests/fields.c), as
    (float32[3, 4096], float64[3, 4096]); None when not built."""
    if not os.path.exists(FIELDS_LIB):
        return None
    lib = ctypes.CDLL(FIELDS_LIB)
    af = np.ctypeslib.as_array((ctypes.c_float * (3 * 4096)).in_dll(lib, "array_float"))
    ad = np.ctypeslib.as_array((ctypes.c_double * (3 * 4096)).in_dll(lib, "array_double"))
    return af.reshape(3, 4096).copy(), ad.reshape(3, 4096).copy()


def view_geometry(v: np.ndarray):
    """(nx, ny, nz), element strides (sx, sy, sz) and the address of element
    (0, 0, 0) of a 1-3D numpy view, possibly non-contiguous or reversed."""
    nx, ny, nz = dims3(v.shape)
    st = [int(b) // v.itemsize for b in v.strides[::-1]] + [0, 0]
    return (nx, ny, nz), tuple(st[:3]), int(v.__array_interface__["data"][0])


def compress_view(v: np.ndarray, rate: float, nthreads: int = 1) -> np.ndarray:
    """Oracle stream of a strided view (zfp_field sx/sy/sz)."""
    (nx, ny, nz), (sx, sy, sz), addr = view_geometry(v)
    n = stream_bytes(v.shape, v.dtype, rate)
    out = np.zeros(max(n // 8, 1), np.uint64)
    lib = port()
    got = lib.gzo_compress_strided(type_code(v.dtype), nx, ny, nz, sx, sy, sz, float(rate), addr,
                                   out.ctypes.data, out.nbytes, int(nthreads))
    if got != n:
        raise RuntimeError("oracle strided compress failed")
    return out[: n // 8]


def decompress_into(words: np.ndarray, v: np.ndarray, rate: float, nthreads: int = 1) -> None:
    """Decode into the strided view `v`; other values of its buffer stay."""
    words = np.ascontiguousarray(words, dtype=np.uint64)
    (nx, ny, nz), (sx, sy, sz), addr = view_geometry(v)
    if not port().gzo_decompress_strided(type_code(v.dtype), nx, ny, nz, sx, sy, sz, float(rate),
                                         words.ctypes.data, words.nbytes, addr, int(nthreads)):
        raise RuntimeError("oracle strided decompress failed")


def ref_compress_view(v: np.ndarray, rate: float) -> np.ndarray:
    (nx, ny, nz), (sx, sy, sz), addr = view_geometry(v)
    t = type_code(v.dtype)
    cap = int(ref().zref_maximum_size(t, nx, ny, nz, float(rate)))
    buf = np.zeros(cap // 8 + 1, np.uint64)
    n = ref().zref_compress_strided(t, nx, ny, nz, sx, sy, sz, float(rate), addr, buf.ctypes.data,
                                    cap)
    return buf[: n // 8]


def ref_decompress_into(words: np.ndarray, v: np.ndarray, rate: float) -> None:
    words = np.ascontiguousarray(words, dtype=np.uint64)
    (nx, ny, nz), (sx, sy, sz), addr = view_geometry(v)
    ref().zref_decompress_strided(type_code(v.dtype), nx, ny, nz, sx, sy, sz, float(rate),
                                  words.ctypes.data, words.nbytes, addr)


# ----------------------------------------------------------- headed streams
_DTYPE_OF = {INT32: np.int32, INT64: np.int64, FLOAT: np.float32, DOUBLE: np.float64}


def _shape_of(nx: int, ny: int, nz: int) -> tuple:
    return tuple(v for v in (nz, ny, nx) if v)


def headed_bytes(shape, dtype, rate: float) -> int:
    nx, ny, nz = dims3(shape)
    hb = int(port().gzo_header_bits(type_code(dtype), nx, ny, nz, float(rate)))
    mb = int(port().gzo_maxbits(type_code(dtype), len(tuple(shape)), float(rate)))
    blocks = 1
    for n in shape:
        blocks *= (int(n) + 3) // 4
    return (hb + blocks * mb + 63) // 64 * 8 if hb else 0


def compress_headed(a: np.ndarray, rate: float) -> np.ndarray:
    """Oracle stream with zfp's full header in front (uint64 words)."""
    a = np.ascontiguousarray(a)
    nx, ny, nz = dims3(a.shape)
    n = headed_bytes(a.shape, a.dtype, rate)
    out = np.zeros(max(n // 8, 1), np.uint64)
    got = port().gzo_compress_headed(type_code(a.dtype), nx, ny, nz, float(rate), a.ctypes.data,
                                     out.ctypes.data, out.nbytes)
    if not n or got != n:
        raise RuntimeError("oracle headed compress failed")
    return out[: n // 8]


def read_header(buf) -> dict:
    """Parse a header: {'bits', 'dtype', 'shape', 'maxbits'}; bits is 0 for
    no header and -1 for a stream in a mode other than fixed rate."""
    b = np.ascontiguousarray(buf).view(np.uint8)
    t, nx, ny, nz, mb = (ctypes.c_int(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(),
                         ctypes.c_uint())
    bits = port().gzo_read_header(b.ctypes.data, b.nbytes, ctypes.byref(t), ctypes.byref(nx),
                                  ctypes.byref(ny), ctypes.byref(nz), ctypes.byref(mb))
    if bits <= 0:
        return {"bits": int(bits)}
    return {"bits": int(bits), "dtype": np.dtype(_DTYPE_OF[t.value]),
            "shape": _shape_of(nx.value, ny.value, nz.value), "maxbits": int(mb.value)}


def decompress_headed(words: np.ndarray) -> np.ndarray:
    words = np.ascontiguousarray(words, dtype=np.uint64)
    h = read_header(words)
    if h["bits"] <= 0:
        raise RuntimeError("oracle: no fixed-rate zfp header")
    out = np.zeros(h["shape"], h["dtype"])
    if not port().gzo_decompress_headed(words.ctypes.data, words.nbytes, out.ctypes.data,
                                        out.nbytes):
        raise RuntimeError("oracle headed decompress failed")
    return out


def ref_compress_headed(a: np.ndarray, rate: float) -> np.ndarray:
    """zfp_write_header(ZFP_HEADER_FULL) + zfp_compress of the reference's
    own build (integer arrays: header + its per-block integer API)."""
    a = np.ascontiguousarray(a)
    nx, ny, nz = dims3(a.shape)
    t = type_code(a.dtype)
    cap = int(ref().zref_maximum_size(t, nx, ny, nz, float(rate)))
    cap = max(cap, headed_bytes(a.shape, a.dtype, rate))
    buf = np.zeros(cap // 8 + 1, np.uint64)
    n = ref().zref_compress_headed(t, nx, ny, nz, float(rate), a.ctypes.data, buf.ctypes.data,
                                   buf.nbytes)
    if not n:
        raise RuntimeError("reference headed compress failed")
    return buf[: n // 8]


def ref_read_header(buf) -> dict:
    b = np.ascontiguousarray(buf).view(np.uint8)
    c = [ctypes.c_int(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(),
         ctypes.c_uint(), ctypes.c_uint(), ctypes.c_int()]
    bits = ref().zref_read_header(b.ctypes.data, b.nbytes, *[ctypes.byref(v) for v in c])
    t, nx, ny, nz, minbits, maxbits, maxprec, minexp = [v.value for v in c]
    return {"bits": int(bits), "type": t, "nx": nx, "ny": ny, "nz": nz, "minbits": minbits,
            "maxbits": maxbits, "maxprec": maxprec, "minexp": minexp}


def ref_decompress_headed(words: np.ndarray, shape, dtype, rate: float) -> np.ndarray:
    words = np.ascontiguousarray(words, dtype=np.uint64)
    out = np.zeros(tuple(shape), dtype)
    if is_int(dtype):
        nx, ny, nz = dims3(shape)
        ok = ref().zref_decompress_headed_int(type_code(dtype), nx, ny, nz, float(rate),
                                              words.ctypes.data, words.nbytes, out.ctypes.data)
    else:
        ok = ref().zref_decompress_headed(words.ctypes.data, words.nbytes, out.ctypes.data)
    if not ok:
        raise RuntimeError("reference headed decompress failed")
    return out


# ------------------------------------------------------------- block access
def _block_args(indices, shapes):
    idx = np.ascontiguousarray(indices, dtype=np.uint64)
    shp = None if shapes is None else np.ascontiguousarray(shapes, dtype=np.uint8)
    return idx, shp, (shp.ctypes.data if shp is not None else None)


def decode_blocks(words, dtype, dims: int, maxbits: int, indices, shapes=None,
                  tiles=None, lib=None) -> np.ndarray:
    """Decode the listed blocks into tiles of 4^dims values (a partial block
    writes only its valid values of `tiles`, zeros by default)."""
    words = np.ascontiguousarray(words, dtype=np.uint64)
    idx, shp, shp_ptr = _block_args(indices, shapes)
    if tiles is None:
        tiles = np.zeros((idx.size, 4 ** dims), dtype)
    fn = port().gzo_decode_blocks if lib is None else lib.zref_decode_blocks
    if not fn(type_code(dtype), dims, maxbits, words.ctypes.data, words.nbytes, idx.ctypes.data,
              shp_ptr, idx.size, tiles.ctypes.data):
        raise RuntimeError("decode_blocks failed")
    return tiles


def encode_blocks(tiles: np.ndarray, dims: int, maxbits: int, indices, words: np.ndarray,
                  shapes=None, lib=None) -> np.ndarray:
    """Encode tile i into the slot of indices[i] of `words` (in place)."""
    tiles = np.ascontiguousarray(tiles)
    idx, shp, shp_ptr = _block_args(indices, shapes)
    fn = port().gzo_encode_blocks if lib is None else lib.zref_encode_blocks
    if not fn(type_code(tiles.dtype), dims, maxbits, tiles.ctypes.data, idx.ctypes.data, shp_ptr,
              idx.size, words.ctypes.data, words.nbytes):
        raise RuntimeError("encode_blocks failed")
    return words


def ref_decode_blocks(words, dtype, dims, maxbits, indices, shapes=None, tiles=None):
    return decode_blocks(words, dtype, dims, maxbits, indices, shapes, tiles, lib=ref())


def ref_encode_blocks(tiles, dims, maxbits, indices, words, shapes=None):
    return encode_blocks(tiles, dims, maxbits, indices, words, shapes, lib=ref())


def field_tiles(a: np.ndarray):
    """The blocks of a contiguous field as tiles (block order x fastest, as
    the stream), with zfp's partial-block shape codes; padded positions hold
    zeros."""
    shape = a.shape
    d = a.ndim
    nb = [(n + 3) // 4 for n in shape]  # per axis, slowest first
    pad = np.zeros(tuple(4 * b for b in nb), a.dtype)
    pad[tuple(slice(0, n) for n in shape)] = a
    # (bz, 4, by, 4, bx, 4) -> (bz, by, bx, 4z, 4y, 4x)
    t = pad.reshape(sum(([b, 4] for b in nb), []))
    order = list(range(0, 2 * d, 2)) + list(range(1, 2 * d, 2))
    t = np.ascontiguousarray(t.transpose(order)).reshape(-1, 4 ** d)
    codes = np.zeros(nb, np.uint8)
    for ax in range(d):  # axis ax of the array is zfp axis d-1-ax
        n = shape[ax]
        ext = np.full(nb[ax], 4, np.int64)
        ext[-1] = n - 4 * (nb[ax] - 1)
        sh = [1] * d
        sh[ax] = nb[ax]
        codes = codes + ((4 - ext).reshape(sh) << (2 * (d - 1 - ax))).astype(np.uint8)
    return t, codes.reshape(-1)


# ------------------------------------------- general parameters (zfp modes)
def _mode_out(fn, t, v):
    mn, mx, mp, me = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_int()
    fn(t, v, ctypes.byref(mn), ctypes.byref(mx), ctypes.byref(mp), ctypes.byref(me))
    return (mn.value, mx.value, mp.value, me.value)


def mode_precision(dtype, precision: int, lib=None) -> tuple:
    """(minbits, maxbits, maxprec, minexp) of zfp_stream_set_precision."""
    fn = port().gzo_mode_precision if lib is None else lib.zref_set_precision
    return _mode_out(fn, type_code(dtype), int(precision))


def mode_accuracy(dtype, tolerance: float, lib=None) -> tuple:
    """(minbits, maxbits, maxprec, minexp) of zfp_stream_set_accuracy."""
    fn = port().gzo_mode_accuracy if lib is None else lib.zref_set_accuracy
    return _mode_out(fn, type_code(dtype), float(tolerance))


def compress_params(a: np.ndarray, params: tuple, with_offsets: bool = False):
    """Oracle stream of a contiguous array under zfp's general parameters
    (minbits, maxbits, maxprec, minexp); with_offsets also returns every
    block's start bit."""
    a = np.ascontiguousarray(a)
    nx, ny, nz = dims3(a.shape)
    t = type_code(a.dtype)
    cap = int(port().gzo_bound_params(t, nx, ny, nz, *params))
    if cap == 0:
        raise RuntimeError("bad parameters")
    out = np.zeros(cap // 8 + 1, np.uint64)
    nb = int(np.prod([(n + 3) // 4 for n in a.shape]))
    offs = np.zeros(nb, np.uint64)
    n = port().gzo_compress_params(t, nx, ny, nz, *params, a.ctypes.data, out.ctypes.data,
                                   out.nbytes, offs.ctypes.data)
    if n == 0:
        raise RuntimeError("oracle compress failed")
    return (out[: n // 8], offs) if with_offsets else out[: n // 8]


def decompress_params(words, shape, dtype, params: tuple, with_offsets: bool = False):
    words = np.ascontiguousarray(words, dtype=np.uint64)
    out = np.zeros(tuple(shape), dtype)
    nx, ny, nz = dims3(shape)
    nb = int(np.prod([(n + 3) // 4 for n in shape]))
    offs = np.zeros(nb, np.uint64)
    if not port().gzo_decompress_params(type_code(dtype), nx, ny, nz, *params, words.ctypes.data,
                                        words.nbytes, out.ctypes.data, offs.ctypes.data):
        raise RuntimeError("oracle decompress failed")
    return (out, offs) if with_offsets else out


def ref_compress_params(a: np.ndarray, params: tuple) -> np.ndarray:
    a = np.ascontiguousarray(a)
    nx, ny, nz = dims3(a.shape)
    t = type_code(a.dtype)
    cap = int(port().gzo_bound_params(t, nx, ny, nz, *params)) + 64
    buf = np.zeros(cap // 8 + 1, np.uint64)
    n = ref().zref_compress_params(t, nx, ny, nz, *params, a.ctypes.data, buf.ctypes.data,
                                   buf.nbytes)
    if n == 0:
        raise RuntimeError("reference compress failed")
    return buf[: n // 8]


def ref_decompress_params(words, shape, dtype, params: tuple) -> np.ndarray:
    words = np.ascontiguousarray(words, dtype=np.uint64)
    # zfp's reader may look a word past the stream: give it zeros there
    padded = np.concatenate([words, np.zeros(72, np.uint64)])
    out = np.zeros(tuple(shape), dtype)
    nx, ny, nz = dims3(shape)
    if not ref().zref_decompress_params(type_code(dtype), nx, ny, nz, *params,
                                        padded.ctypes.data, padded.nbytes, out.ctypes.data):
        raise RuntimeError("reference decompress failed")
    return out


def compress_params_headed(a: np.ndarray, params: tuple, lib=None) -> np.ndarray:
    """The header of these parameters, then the blocks: the oracle's, or
    with lib=ref() the reference's zfp_write_header + zfp_compress."""
    a = np.ascontiguousarray(a)
    nx, ny, nz = dims3(a.shape)
    t = type_code(a.dtype)
    cap = int(port().gzo_bound_params(t, nx, ny, nz, *params)) + 64
    buf = np.zeros(cap // 8 + 1, np.uint64)
    fn = port().gzo_compress_params_headed if lib is None else lib.zref_compress_params_headed
    n = fn(t, nx, ny, nz, *params, a.ctypes.data, buf.ctypes.data, buf.nbytes)
    if n == 0:
        raise RuntimeError("headed compress failed")
    return buf[: n // 8]


def read_header_params(buf) -> dict:
    b = np.ascontiguousarray(buf).view(np.uint8)
    t = ctypes.c_int()
    u = [ctypes.c_uint() for _ in range(6)]
    e = ctypes.c_int()
    bits = port().gzo_read_header_params(b.ctypes.data, b.nbytes, ctypes.byref(t),
                                         *[ctypes.byref(v) for v in u], ctypes.byref(e))
    if bits <= 0:
        return {"bits": int(bits)}
    nx, ny, nz, mn, mx, mp = [v.value for v in u]
    return {"bits": int(bits), "dtype": np.dtype(_DTYPE_OF[t.value]),
            "shape": _shape_of(nx, ny, nz), "params": (mn, mx, mp, e.value)}
