"""GB300-native ZFP fixed-rate codec.

Python mirror of cuZFP's host interface (src/cuZFP/cuZFP.h:9-10 and
src/cuZFP/zfp_structs.h): ``zfp_stream`` / ``zfp_field`` records,
``stream_set_rate``, ``zfp_field_1d/2d/3d``, ``zfp_stream_maximum_size``,
``compress(stream, field)`` and ``decompress(stream, field)``, with the same
argument meaning.  Every call goes through the C ABI of ``libgzfp.so``
(include/gzfp.h) to the CUDA kernels; there is no CPU code path, and
importing the package fails if the library has not been built.

Differences from cuZFP, all toward zfp 0.5.0 (the reference's own CPU
codec, which cuZFP's test driver treats as ground truth):

* ``stream_set_rate`` computes bits per block as zfp_stream_set_rate with
  wra = 0 (no rounding of 3D rates up to a word multiple, which cuZFP does
  in zfp_structs.h:64-69); the two agree for every integer 3D rate.
* Partial edge blocks are padded by zfp's pad_block rule.
* Errors raise ``GzfpError`` instead of being printed.
* Strided fields (non-zero sx/sy/sz), which cuZFP silently codes as
  contiguous, are coded through their strides as zfp 0.5.0 does; so are
  non-contiguous tensors and arrays.
* Integer fields (int32 / int64) are coded as zfp 0.5.0's integer block
  codec does (no exponent, whole budget); a rate that gives 0 bits per
  block is rejected.
"""
from __future__ import annotations

import ctypes
import enum
import math
import os
from dataclasses import dataclass, field as _dc_field
from typing import Any, Optional

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgzfp.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build the CUDA codec first "
        "(python -c 'import __graft_entry__ as g; g.build()')")

_lib = ctypes.CDLL(LIB_PATH)

_U = ctypes.c_uint
_I = ctypes.c_int
_SZ = ctypes.c_size_t
_VP = ctypes.c_void_p

_lib.gzfp_version.restype = _I
_lib.gzfp_status_string.restype = ctypes.c_char_p
_lib.gzfp_status_string.argtypes = [_I]
_lib.gzfp_last_error.restype = ctypes.c_char_p
_lib.gzfp_rate_to_maxbits.restype = _U
_lib.gzfp_rate_to_maxbits.argtypes = [_I, _U, ctypes.c_double]
_lib.gzfp_stream_size.restype = _SZ
_lib.gzfp_stream_size.argtypes = [_I, _U, _U, _U, _U]
_lib.gzfp_maximum_size.restype = _SZ
_lib.gzfp_maximum_size.argtypes = [_I, _U, _U, _U, _U]
_lib.gzfp_compress.restype = _I
_lib.gzfp_compress.argtypes = [_I, _U, _U, _U, ctypes.c_double, _VP, _VP, _SZ,
                               ctypes.POINTER(_SZ), _VP]
_lib.gzfp_decompress.restype = _I
_lib.gzfp_decompress.argtypes = [_I, _U, _U, _U, ctypes.c_double, _VP, _SZ, _VP, _VP]
_lib.gzfp_compress_bits.restype = _I
_lib.gzfp_compress_bits.argtypes = [_I, _U, _U, _U, _U, _VP, _VP, _SZ, ctypes.POINTER(_SZ), _VP]
_lib.gzfp_decompress_bits.restype = _I
_lib.gzfp_decompress_bits.argtypes = [_I, _U, _U, _U, _U, _VP, _SZ, _VP, _VP]
_LL = ctypes.c_longlong
_lib.gzfp_compress_strided.restype = _I
_lib.gzfp_compress_strided.argtypes = [_I, _U, _U, _U, _LL, _LL, _LL, _U, _VP, _VP, _SZ,
                                       ctypes.POINTER(_SZ), _VP]
_P = ctypes.POINTER
_lib.gzfp_write_header.restype = _I
_lib.gzfp_write_header.argtypes = [_I, _U, _U, _U, _U, _VP, _SZ, _P(_SZ)]
_lib.gzfp_read_header.restype = _I
_lib.gzfp_read_header.argtypes = [_VP, _SZ, _P(_I), _P(_U), _P(_U), _P(_U), _P(_U), _P(_SZ)]
_lib.gzfp_read_header_mode.restype = _I
_lib.gzfp_read_header_mode.argtypes = [_VP, _SZ, _P(_I), _P(_U), _P(_U), _P(_U), _VP, _P(_SZ)]
_lib.gzfp_write_header_mode.restype = _I
_lib.gzfp_write_header_mode.argtypes = [_I, _U, _U, _U, _VP, _VP, _SZ, _P(_SZ)]
_lib.gzfp_compress_mode_headed.restype = _I
_lib.gzfp_compress_mode_headed.argtypes = [_I, _U, _U, _U, _VP, _VP, _VP, _SZ, _P(_SZ), _VP, _VP]
_lib.gzfp_compress_headed.restype = _I
_lib.gzfp_compress_headed.argtypes = [_I, _U, _U, _U, ctypes.c_double, _VP, _VP, _SZ, _P(_SZ),
                                      _VP]
_lib.gzfp_decompress_headed.restype = _I
_lib.gzfp_decompress_headed.argtypes = [_VP, _SZ, _VP, _SZ, _VP]
_lib.gzfp_decode_blocks.restype = _I
_lib.gzfp_decode_blocks.argtypes = [_I, _U, _U, _VP, _SZ, _VP, _VP, _SZ, _VP, _VP]
_lib.gzfp_encode_blocks.restype = _I
_lib.gzfp_encode_blocks.argtypes = [_I, _U, _U, _VP, _VP, _VP, _SZ, _VP, _SZ, _VP]
_lib.gzfp_decompress_strided.restype = _I
_lib.gzfp_decompress_strided.argtypes = [_I, _U, _U, _U, _LL, _LL, _LL, _U, _VP, _SZ, _VP, _VP]

# zfp constants (src/cuZFP/zfp_structs.h:9-13)
ZFP_MAX_PREC = 64
ZFP_MIN_EXP = -1074
ZFP_MAX_BITS = 4171
ZFP_MIN_BITS = 0
ZFP_HEADER_MAX_BITS = 148

GZFP_OK = 0
GZFP_ERR_ARG = 1
GZFP_ERR_UNSUPPORTED = 2
GZFP_ERR_CAPACITY = 3
GZFP_ERR_CUDA = 4


class GzfpError(RuntimeError):
    """A failed codec call; ``status`` holds the C ABI status code."""

    def __init__(self, status: int, what: str):
        detail = _lib.gzfp_last_error().decode()
        msg = f"{what}: {_lib.gzfp_status_string(status).decode()}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)
        self.status = status


def _check(status: int, what: str) -> None:
    if status != GZFP_OK:
        raise GzfpError(status, what)


class zfp_type(enum.IntEnum):
    """Scalar types, values of src/cuZFP/zfp_structs.h:31-37."""
    none = 0
    int32 = 1
    int64 = 2
    float = 3
    double = 4


zfp_type_none = zfp_type.none
zfp_type_int32 = zfp_type.int32
zfp_type_int64 = zfp_type.int64
zfp_type_float = zfp_type.float
zfp_type_double = zfp_type.double

_TYPE_SIZE = {zfp_type.int32: 4, zfp_type.int64: 8, zfp_type.float: 4, zfp_type.double: 8}


@dataclass
class zfp_stream:
    """Compressed stream parameters and buffer (src/cuZFP/zfp_structs.h:22-29).

    ``stream`` is the word buffer: a torch tensor (CUDA or CPU), a numpy
    array, or a raw address; ``capacity`` its size in bytes (taken from the
    buffer object when omitted).
    """
    minbits: int = 0
    maxbits: int = 0
    maxprec: int = ZFP_MAX_PREC
    minexp: int = ZFP_MIN_EXP
    stream: Any = None
    capacity: Optional[int] = None


@dataclass
class zfp_field:
    """Uncompressed array description (src/cuZFP/zfp_structs.h:39-44)."""
    type: zfp_type = zfp_type.none
    nx: int = 0
    ny: int = 0
    nz: int = 0
    sx: int = 0
    sy: int = 0
    sz: int = 0
    data: Any = None


def zfp_stream_open(stream: Any = None) -> zfp_stream:
    return zfp_stream(stream=stream)


def zfp_field_1d(data: Any, type: zfp_type, nx: int) -> zfp_field:
    return zfp_field(type=zfp_type(type), nx=nx, data=data)


def zfp_field_2d(data: Any, type: zfp_type, nx: int, ny: int) -> zfp_field:
    return zfp_field(type=zfp_type(type), nx=nx, ny=ny, data=data)


def zfp_field_3d(data: Any, type: zfp_type, nx: int, ny: int, nz: int) -> zfp_field:
    return zfp_field(type=zfp_type(type), nx=nx, ny=ny, nz=nz, data=data)


def zfp_field_dimensionality(f: zfp_field) -> int:
    """Number of leading non-zero sizes (zfp's convention)."""
    return 0 if not f.nx else 1 if not f.ny else 2 if not f.nz else 3


def zfp_type_size(t: zfp_type) -> int:
    return _TYPE_SIZE.get(zfp_type(t), 0)


def stream_set_rate(zfp: zfp_stream, rate: float, type: zfp_type, dims: int) -> float:
    """Fixed-rate mode: set min/maxbits for ``rate`` bits per value and return
    the rate actually used (zfp_structs.h:46-76; zfp-0.5.0/src/zfp.c:405-430)."""
    bits = _lib.gzfp_rate_to_maxbits(int(type), int(dims), float(rate))
    if bits == 0:
        raise GzfpError(GZFP_ERR_ARG, "stream_set_rate")
    zfp.minbits = zfp.maxbits = bits
    zfp.maxprec = ZFP_MAX_PREC
    zfp.minexp = ZFP_MIN_EXP
    return bits / float(1 << (2 * dims))


def zfp_stream_set_precision(zfp: zfp_stream, precision: int, type: zfp_type) -> int:
    """zfp's fixed-precision mode (zfp-0.5.0/src/zfp.c:432-441)."""
    m = mode_precision(type, precision)
    zfp.minbits, zfp.maxbits, zfp.maxprec, zfp.minexp = m.as_tuple()
    return m.maxprec


def zfp_stream_set_accuracy(zfp: zfp_stream, tolerance: float, type: zfp_type) -> float:
    """zfp's fixed-accuracy mode (zfp-0.5.0/src/zfp.c:443-458)."""
    m = mode_accuracy(type, tolerance)
    zfp.minbits, zfp.maxbits, zfp.maxprec, zfp.minexp = m.as_tuple()
    return 2.0 ** m.minexp if tolerance > 0 else 0.0


def _fixed_rate(zfp: zfp_stream, t: zfp_type) -> bool:
    """The parameters of fixed-rate coding (the fixed-rate path's)."""
    ints = zfp_type(t) in (zfp_type.int32, zfp_type.int64)
    prec = 32 if zfp_type(t) in (zfp_type.float, zfp_type.int32) else 64
    return (zfp.minbits == zfp.maxbits and zfp.maxprec >= prec
            and (ints or zfp.minexp == ZFP_MIN_EXP))


def _mode_of(zfp: zfp_stream):
    return Mode(zfp.minbits, zfp.maxbits, zfp.maxprec, zfp.minexp)


def zfp_stream_maximum_size(zfp: zfp_stream, f: zfp_field) -> int:
    """Worst-case buffer bytes (zfp_structs.h:222-251), header allowance
    included, for every mode."""
    if _fixed_rate(zfp, f.type):
        return int(_lib.gzfp_maximum_size(int(f.type), f.nx, f.ny, f.nz, zfp.maxbits))
    n = mode_maximum_size(f.type, f.nx, f.ny, f.nz, _mode_of(zfp))
    return n + 24 if n else 0


def stream_size(type: zfp_type, nx: int, ny: int, nz: int, maxbits: int) -> int:
    """Exact compressed bytes for a fixed-rate stream."""
    return int(_lib.gzfp_stream_size(int(type), nx, ny, nz, maxbits))


# ------------------------------------------------------------------ buffers

def _addr_and_size(obj: Any) -> tuple[int, Optional[int]]:
    """Device or host address of a torch tensor, numpy array or raw int."""
    if obj is None:
        return 0, None
    if isinstance(obj, int):
        return obj, None
    if hasattr(obj, "data_ptr") and hasattr(obj, "element_size"):  # torch.Tensor
        if not obj.is_contiguous():
            raise GzfpError(GZFP_ERR_ARG, "tensor must be contiguous")
        return int(obj.data_ptr()), int(obj.numel() * obj.element_size())
    if hasattr(obj, "__array_interface__"):  # numpy
        if not obj.flags["C_CONTIGUOUS"]:
            raise GzfpError(GZFP_ERR_ARG, "array must be C-contiguous")
        return int(obj.__array_interface__["data"][0]), int(obj.nbytes)
    raise GzfpError(GZFP_ERR_ARG, f"unsupported buffer type {type(obj).__name__}")


def _element_strides(obj: Any):
    """(sx, sy, sz) element strides (x fastest) of a torch tensor or numpy
    array, or None when it is contiguous."""
    if hasattr(obj, "data_ptr") and hasattr(obj, "stride"):  # torch.Tensor
        if obj.is_contiguous():
            return None
        st = list(obj.stride())[::-1]
    elif hasattr(obj, "__array_interface__"):
        if obj.flags["C_CONTIGUOUS"]:
            return None
        st = [b // obj.itemsize for b in obj.strides[::-1]]
    else:
        return None
    return tuple((st + [0, 0])[:3])


def _field_addr(obj: Any) -> int:
    """Address of element (0, 0, 0) of a tensor or array, strided or not."""
    if hasattr(obj, "data_ptr"):
        return int(obj.data_ptr())
    if hasattr(obj, "__array_interface__"):
        return int(obj.__array_interface__["data"][0])
    return _addr_and_size(obj)[0]


def _cuda_stream_handle(cuda_stream: Any) -> int:
    if cuda_stream is None:
        return 0
    if isinstance(cuda_stream, int):
        return cuda_stream
    return int(cuda_stream.cuda_stream)  # torch.cuda.Stream


def _check_strided_mode(zfp: zfp_stream, f: zfp_field, strides) -> None:
    if strides and not _fixed_rate(zfp, f.type):
        raise GzfpError(GZFP_ERR_UNSUPPORTED, "strided fields take the fixed-rate path only")


def compress(zfp: zfp_stream, f: zfp_field, cuda_stream: Any = None) -> int:
    """Compress ``f`` into ``zfp.stream``; returns the stream size in bytes.

    Mirrors cuZFP::compress (src/cuZFP/cuZFP.cu:174-210).  With device
    buffers the work is queued on ``cuda_stream`` (default: the legacy
    default stream) and the call returns at once; with a host buffer it
    returns when the result is in host memory.  Parameters other than fixed
    rate (zfp_stream_set_precision / _accuracy) take zfp's general mode,
    which returns when the stream is complete.
    """
    strides = _field_strides(f)
    _check_strided_mode(zfp, f, strides)
    if not _fixed_rate(zfp, f.type):
        src, _ = _addr_and_size(f.data)
        dst, cap = _addr_and_size(zfp.stream)
        if zfp.capacity is not None:
            cap = zfp.capacity
        if cap is None:
            cap = zfp_stream_maximum_size(zfp, f)
        out = _SZ(0)
        m = _mode_of(zfp)
        _check(_lib.gzfp_compress_mode(int(f.type), f.nx, f.ny, f.nz, ctypes.byref(m), src, dst,
                                       cap, ctypes.byref(out), None,
                                       _cuda_stream_handle(cuda_stream)), "compress")
        return int(out.value)
    src = _field_addr(f.data) if strides else _addr_and_size(f.data)[0]
    dst, cap = _addr_and_size(zfp.stream)
    if zfp.capacity is not None:
        cap = zfp.capacity
    if cap is None:
        cap = zfp_stream_maximum_size(zfp, f)
    out = _SZ(0)
    if strides:
        st = _lib.gzfp_compress_strided(int(f.type), f.nx, f.ny, f.nz, *strides, zfp.maxbits, src,
                                        dst, cap, ctypes.byref(out),
                                        _cuda_stream_handle(cuda_stream))
    else:
        st = _lib.gzfp_compress_bits(int(f.type), f.nx, f.ny, f.nz, zfp.maxbits, src, dst, cap,
                                     ctypes.byref(out), _cuda_stream_handle(cuda_stream))
    _check(st, "compress")
    return int(out.value)


def decompress(zfp: zfp_stream, f: zfp_field, cuda_stream: Any = None) -> None:
    """Decompress ``zfp.stream`` into ``f.data`` (cuZFP::decompress,
    src/cuZFP/cuZFP.cu:212-269); in zfp's general mode the blocks are found
    by walking them (see decompress_mode for decoding from known offsets)."""
    strides = _field_strides(f)
    _check_strided_mode(zfp, f, strides)
    if not _fixed_rate(zfp, f.type):
        src, size = _addr_and_size(zfp.stream)
        if zfp.capacity is not None:
            size = zfp.capacity
        if size is None:
            size = zfp_stream_maximum_size(zfp, f)
        m = _mode_of(zfp)
        _check(_lib.gzfp_decompress_mode(int(f.type), f.nx, f.ny, f.nz, ctypes.byref(m), src,
                                         size, None, _addr_and_size(f.data)[0],
                                         _cuda_stream_handle(cuda_stream)), "decompress")
        return
    src, size = _addr_and_size(zfp.stream)
    dst = _field_addr(f.data) if strides else _addr_and_size(f.data)[0]
    if zfp.capacity is not None:
        size = zfp.capacity
    if size is None:
        size = stream_size(f.type, f.nx, f.ny, f.nz, zfp.maxbits)
    if strides:
        st = _lib.gzfp_decompress_strided(int(f.type), f.nx, f.ny, f.nz, *strides, zfp.maxbits,
                                          src, size, dst, _cuda_stream_handle(cuda_stream))
    else:
        st = _lib.gzfp_decompress_bits(int(f.type), f.nx, f.ny, f.nz, zfp.maxbits, src, size, dst,
                                       _cuda_stream_handle(cuda_stream))
    _check(st, "decompress")


def _field_strides(f: zfp_field):
    """The field's strides: its sx/sy/sz when set, else those of a
    non-contiguous tensor or array; None for a contiguous field."""
    if f.sx or f.sy or f.sz:
        return (f.sx, f.sy, f.sz)
    return _element_strides(f.data) if f.data is not None else None


# ------------------------------------------------------- array conveniences

def _dims_of(shape) -> tuple[int, int, int]:
    """(nx, ny, nz) of a C-ordered array of 1..3 dimensions."""
    if not 1 <= len(shape) <= 3:
        raise GzfpError(GZFP_ERR_ARG, "arrays must have 1 to 3 dimensions")
    s = tuple(int(v) for v in shape)[::-1]
    return (s + (0, 0))[:3]


def _type_of(dtype) -> zfp_type:
    name = str(dtype)
    if name.endswith("float32"):
        return zfp_type.float
    if name.endswith("float64"):
        return zfp_type.double
    if name.endswith("int32") and not name.endswith("uint32"):
        return zfp_type.int32
    if name.endswith("int64") and not name.endswith("uint64"):
        return zfp_type.int64
    raise GzfpError(GZFP_ERR_UNSUPPORTED, f"dtype {name}")


def compress_tensor(x, rate: float, out=None, cuda_stream: Any = None):
    """Compress a CUDA tensor (float32 / float64 / int32 / int64, 1-3 dims;
    a strided view is coded through its strides, as zfp codes a strided
    field) at ``rate`` bits per value.  Returns the uint64 word tensor of the
    stream (``out`` if given) on the same device."""
    import torch
    t = _type_of(x.dtype)
    nx, ny, nz = _dims_of(x.shape)
    zfp = zfp_stream()
    stream_set_rate(zfp, rate, t, len(x.shape))
    nbytes = stream_size(t, nx, ny, nz, zfp.maxbits)
    if out is None:
        out = torch.empty(nbytes // 8, dtype=torch.int64, device=x.device)
    zfp.stream = out
    compress(zfp, zfp_field(type=t, nx=nx, ny=ny, nz=nz, data=x), cuda_stream)
    return out


def decompress_tensor(words, shape, dtype, rate: float, out=None, cuda_stream: Any = None):
    """Inverse of compress_tensor; ``out`` may be a strided view, whose other
    elements are left as they are."""
    import torch
    t = _type_of(dtype)
    nx, ny, nz = _dims_of(shape)
    zfp = zfp_stream(stream=words)
    stream_set_rate(zfp, rate, t, len(shape))
    if out is None:
        out = torch.empty(tuple(shape), dtype=dtype, device=words.device)
    decompress(zfp, zfp_field(type=t, nx=nx, ny=ny, nz=nz, data=out), cuda_stream)
    return out


# ------------------------------------------------------------ headed streams
# zfp 0.5.0's self-describing header (zfp_write_header / zfp_read_header
# with ZFP_HEADER_FULL, zfp-0.5.0/src/zfp.c:661-719) in front of the blocks.

HEADER_MAX_BITS = 148
_DTYPE_NAME = {zfp_type.int32: "int32", zfp_type.int64: "int64", zfp_type.float: "float32",
               zfp_type.double: "float64"}


def write_header(type: zfp_type, nx: int, ny: int, nz: int, maxbits: int) -> tuple[bytes, int]:
    """The header bytes of a fixed-rate stream and its length in bits."""
    buf = ctypes.create_string_buffer(24)
    bits = _SZ(0)
    _check(_lib.gzfp_write_header(int(type), nx, ny, nz, maxbits, buf, 24, ctypes.byref(bits)),
           "write_header")
    return buf.raw[: (bits.value + 7) // 8], int(bits.value)


def read_header(buf: Any) -> dict:
    """Parse the header at the start of a host buffer (bytes, numpy array)
    or a CUDA tensor: {'type', 'shape', 'dtype', 'maxbits', 'bits'}."""
    if hasattr(buf, "data_ptr") and getattr(buf, "is_cuda", False):
        buf = buf[: 3 * 8 // buf.element_size()].cpu().numpy()
    if isinstance(buf, (bytes, bytearray)):
        raw = bytes(buf)
    else:
        import numpy as np
        raw = np.ascontiguousarray(buf).view(np.uint8).tobytes()
    c = ctypes.create_string_buffer(raw, len(raw))
    t, nx, ny, nz, mb, bits = _I(0), _U(0), _U(0), _U(0), _U(0), _SZ(0)
    _check(_lib.gzfp_read_header(c, len(raw), ctypes.byref(t), ctypes.byref(nx), ctypes.byref(ny),
                                 ctypes.byref(nz), ctypes.byref(mb), ctypes.byref(bits)),
           "read_header")
    zt = zfp_type(t.value)
    return {"type": zt, "shape": tuple(v for v in (nz.value, ny.value, nx.value) if v),
            "dtype": _DTYPE_NAME[zt], "maxbits": int(mb.value), "bits": int(bits.value)}


def read_header_mode(buf: Any) -> dict:
    """Parse the header of a stream of any mode: {'type', 'shape', 'dtype',
    'mode' (a Mode), 'bits'}."""
    if hasattr(buf, "data_ptr") and getattr(buf, "is_cuda", False):
        buf = buf[: 3 * 8 // buf.element_size()].cpu().numpy()
    if isinstance(buf, (bytes, bytearray)):
        raw = bytes(buf)
    else:
        import numpy as np
        raw = np.ascontiguousarray(buf).view(np.uint8).tobytes()
    c = ctypes.create_string_buffer(raw, len(raw))
    t, nx, ny, nz, bits = _I(0), _U(0), _U(0), _U(0), _SZ(0)
    m = Mode()
    _check(_lib.gzfp_read_header_mode(c, len(raw), ctypes.byref(t), ctypes.byref(nx),
                                      ctypes.byref(ny), ctypes.byref(nz), ctypes.byref(m),
                                      ctypes.byref(bits)), "read_header_mode")
    zt = zfp_type(t.value)
    return {"type": zt, "shape": tuple(v for v in (nz.value, ny.value, nx.value) if v),
            "dtype": _DTYPE_NAME[zt], "mode": m, "bits": int(bits.value)}


def write_header_mode(type: zfp_type, nx: int, ny: int, nz: int, mode) -> tuple[bytes, int]:
    """The header bytes of a stream with these parameters, and its bits."""
    buf = ctypes.create_string_buffer(24)
    bits = _SZ(0)
    _check(_lib.gzfp_write_header_mode(int(type), nx, ny, nz, ctypes.byref(mode), buf, 24,
                                       ctypes.byref(bits)), "write_header_mode")
    return buf.raw[: (bits.value + 7) // 8], int(bits.value)


def compress_mode_headed(x, mode, with_offsets: bool = False, cuda_stream: Any = None):
    """compress_mode with zfp's full header in front (offsets count from
    the stream's first bit)."""
    t = _type_of(x.dtype)
    nx, ny, nz = _dims_of(x.shape)
    cap = mode_maximum_size(t, nx, ny, nz, mode) + 24
    nb = _nblocks(x.shape)
    if hasattr(x, "data_ptr"):
        import torch
        out = torch.empty(cap // 8, dtype=torch.int64, device=x.device)
        offs = torch.empty(nb, dtype=torch.int64, device=x.device) if with_offsets else None
    else:
        import numpy as np
        out = np.empty(cap // 8, np.uint64)
        offs = np.empty(nb, np.uint64) if with_offsets else None
    got = _SZ(0)
    _check(_lib.gzfp_compress_mode_headed(int(t), nx, ny, nz, ctypes.byref(mode),
                                          _addr_and_size(x)[0], _addr_and_size(out)[0],
                                          out.nbytes if hasattr(out, "nbytes") else cap,
                                          ctypes.byref(got),
                                          _addr_and_size(offs)[0] if offs is not None else None,
                                          _cuda_stream_handle(cuda_stream)), "compress_mode_headed")
    words = out[: got.value // 8]
    return (words, offs) if with_offsets else words


def headed_size(type: zfp_type, nx: int, ny: int, nz: int, maxbits: int) -> int:
    """Exact bytes of a headed fixed-rate stream."""
    _, hb = write_header(type, nx, ny, nz, maxbits)
    blocks = 1
    for n in (nx, ny, nz):
        blocks *= (n + 3) // 4 if n else 1
    return (hb + blocks * maxbits + 63) // 64 * 8


def compress_headed(x, rate: float, out=None, cuda_stream: Any = None):
    """Compress a contiguous CUDA tensor or numpy array (float32 / float64 /
    int32 / int64, 1-3 dims) into a stream that starts with zfp's full
    header.  Returns the uint64 words: a tensor on the same device, or a
    numpy array for host input (``out`` if given)."""
    t = _type_of(x.dtype)
    nx, ny, nz = _dims_of(x.shape)
    mb = int(_lib.gzfp_rate_to_maxbits(int(t), len(x.shape), float(rate)))
    if mb == 0:
        raise GzfpError(GZFP_ERR_ARG, "bad type or rate")
    nbytes = headed_size(t, nx, ny, nz, mb)
    if out is None:
        if hasattr(x, "data_ptr"):
            import torch
            out = torch.empty(nbytes // 8, dtype=torch.int64, device=x.device)
        else:
            import numpy as np
            out = np.empty(nbytes // 8, np.uint64)
    src, _ = _addr_and_size(x)
    dst, cap = _addr_and_size(out)
    got = _SZ(0)
    _check(_lib.gzfp_compress_headed(int(t), nx, ny, nz, float(rate), src, dst, cap,
                                     ctypes.byref(got), _cuda_stream_handle(cuda_stream)),
           "compress_headed")
    return out


def decompress_headed(words, out=None, cuda_stream: Any = None):
    """Decompress a headed stream; type and shape come from its header.  The
    result lands in ``out`` when given, else in a new tensor on the stream's
    device (numpy array for a host stream).  Streams of every mode decode."""
    h = read_header_mode(words)
    if out is None:
        if hasattr(words, "data_ptr"):
            import torch
            out = torch.empty(h["shape"], dtype=getattr(torch, h["dtype"]), device=words.device)
        else:
            import numpy as np
            out = np.empty(h["shape"], h["dtype"])
    src, size = _addr_and_size(words)
    dst, cap = _addr_and_size(out)
    _check(_lib.gzfp_decompress_headed(src, size, dst, cap, _cuda_stream_handle(cuda_stream)),
           "decompress_headed")
    return out


# -------------------------------------------------------------- block access
# Random access to single blocks of a fixed-rate stream, as zfp's compressed
# arrays fetch and write back cached blocks (zfp-0.5.0/array/zfparray3.h:
# 225-255): block i sits at bit i * maxbits; each listed block maps to a
# tile of 4^dims values (x fastest); shape codes mark partial blocks.

def _block_buffers(indices, shapes, like):
    """Indices (uint64) and shape codes (uint8) as buffers on the side of
    `like` (a CUDA tensor: device tensors; else numpy)."""
    if hasattr(like, "data_ptr") and getattr(like, "is_cuda", False):
        import torch
        idx = torch.as_tensor(indices, dtype=torch.int64, device=like.device).contiguous()
        shp = None if shapes is None else torch.as_tensor(
            shapes, dtype=torch.uint8, device=like.device).contiguous()
    else:
        import numpy as np
        idx = np.ascontiguousarray(indices, dtype=np.uint64)
        shp = None if shapes is None else np.ascontiguousarray(shapes, dtype=np.uint8)
    n = int(idx.numel() if hasattr(idx, "numel") else idx.size)
    if shp is not None and int(shp.numel() if hasattr(shp, "numel") else shp.size) != n:
        raise GzfpError(GZFP_ERR_ARG, "one shape code per index")
    return idx, shp, n


def decode_blocks(words, dtype, dims: int, maxbits: int, indices, shapes=None, out=None,
                  cuda_stream: Any = None):
    """Decode the listed blocks of ``words`` into tiles (count x 4^dims).  A
    partial block (non-zero shape code) writes only its valid values of its
    tile.  Device words give a device result; host words a numpy one."""
    t = _type_of(dtype)
    idx, shp, n = _block_buffers(indices, shapes, words)
    if out is None:
        if hasattr(words, "data_ptr"):
            import torch
            out = torch.zeros((n, 4 ** dims), dtype=dtype, device=words.device)
        else:
            import numpy as np
            out = np.zeros((n, 4 ** dims), dtype)
    src, size = _addr_and_size(words)
    dst, _ = _addr_and_size(out)
    _check(_lib.gzfp_decode_blocks(int(t), dims, maxbits, src, size, _addr_and_size(idx)[0],
                                   _addr_and_size(shp)[0], n, dst,
                                   _cuda_stream_handle(cuda_stream)), "decode_blocks")
    return out


def encode_blocks(tiles, dims: int, maxbits: int, indices, words, shapes=None,
                  cuda_stream: Any = None):
    """Encode tile i into the slot of indices[i] of ``words``, in place; the
    other bits of ``words`` are kept."""
    t = _type_of(tiles.dtype)
    idx, shp, n = _block_buffers(indices, shapes, tiles)
    src, _ = _addr_and_size(tiles)
    dst, size = _addr_and_size(words)
    _check(_lib.gzfp_encode_blocks(int(t), dims, maxbits, src, _addr_and_size(idx)[0],
                                   _addr_and_size(shp)[0], n, dst, size,
                                   _cuda_stream_handle(cuda_stream)), "encode_blocks")
    return words


# ------------------------------------------------------------ general modes
# zfp's fixed-precision and fixed-accuracy modes and any other setting of
# its four stream parameters (zfp_stream_set_precision / _accuracy /
# _params, zfp-0.5.0/src/zfp.c:432-510): blocks of their own lengths.

class Mode(ctypes.Structure):
    _fields_ = [("minbits", _U), ("maxbits", _U), ("maxprec", _U), ("minexp", _I)]

    def as_tuple(self) -> tuple:
        return (self.minbits, self.maxbits, self.maxprec, self.minexp)


_PM = ctypes.POINTER(Mode)
_lib.gzfp_mode_rate.restype = _I
_lib.gzfp_mode_rate.argtypes = [_I, _U, ctypes.c_double, _PM]
_lib.gzfp_mode_precision.restype = _I
_lib.gzfp_mode_precision.argtypes = [_I, _U, _PM]
_lib.gzfp_mode_accuracy.restype = _I
_lib.gzfp_mode_accuracy.argtypes = [_I, ctypes.c_double, _PM]
_lib.gzfp_mode_maximum_size.restype = _SZ
_lib.gzfp_mode_maximum_size.argtypes = [_I, _U, _U, _U, _PM]
_lib.gzfp_compress_mode.restype = _I
_lib.gzfp_compress_mode.argtypes = [_I, _U, _U, _U, _PM, _VP, _VP, _SZ, _P(_SZ), _VP, _VP]
_lib.gzfp_decompress_mode.restype = _I
_lib.gzfp_decompress_mode.argtypes = [_I, _U, _U, _U, _PM, _VP, _SZ, _VP, _VP, _VP]
_lib.gzfp_index_blocks.restype = _I
_lib.gzfp_index_blocks.argtypes = [_I, _U, _U, _U, _PM, _VP, _SZ, _VP, _VP]


def mode_rate(type: zfp_type, dims: int, rate: float) -> Mode:
    m = Mode()
    _check(_lib.gzfp_mode_rate(int(type), dims, float(rate), ctypes.byref(m)), "mode_rate")
    return m


def mode_precision(type: zfp_type, precision: int) -> Mode:
    m = Mode()
    _check(_lib.gzfp_mode_precision(int(type), int(precision), ctypes.byref(m)), "mode_precision")
    return m


def mode_accuracy(type: zfp_type, tolerance: float) -> Mode:
    m = Mode()
    _check(_lib.gzfp_mode_accuracy(int(type), float(tolerance), ctypes.byref(m)), "mode_accuracy")
    return m


def mode_maximum_size(type: zfp_type, nx: int, ny: int, nz: int, mode: Mode) -> int:
    return int(_lib.gzfp_mode_maximum_size(int(type), nx, ny, nz, ctypes.byref(mode)))


def _nblocks(shape) -> int:
    n = 1
    for v in shape:
        n *= (int(v) + 3) // 4
    return n


def compress_mode(x, mode: Mode, with_offsets: bool = False, cuda_stream: Any = None):
    """Compress a contiguous CUDA tensor or numpy array under `mode`; returns
    the stream words (trimmed to the stream's size) and, with_offsets, every
    block's start bit (int64, on the same side as the input)."""
    t = _type_of(x.dtype)
    nx, ny, nz = _dims_of(x.shape)
    cap = mode_maximum_size(t, nx, ny, nz, mode)
    if cap == 0:
        raise GzfpError(GZFP_ERR_ARG, "bad mode or shape")
    nb = _nblocks(x.shape)
    if hasattr(x, "data_ptr"):
        import torch
        out = torch.empty(cap // 8, dtype=torch.int64, device=x.device)
        offs = torch.empty(nb, dtype=torch.int64, device=x.device) if with_offsets else None
    else:
        import numpy as np
        out = np.empty(cap // 8, np.uint64)
        offs = np.empty(nb, np.uint64) if with_offsets else None
    got = _SZ(0)
    _check(_lib.gzfp_compress_mode(int(t), nx, ny, nz, ctypes.byref(mode), _addr_and_size(x)[0],
                                   _addr_and_size(out)[0], cap, ctypes.byref(got),
                                   _addr_and_size(offs)[0] if offs is not None else None,
                                   _cuda_stream_handle(cuda_stream)), "compress_mode")
    words = out[: got.value // 8]
    return (words, offs) if with_offsets else words


def decompress_mode(words, shape, dtype, mode: Mode, offsets=None, out=None,
                    cuda_stream: Any = None):
    """Decompress a stream written under `mode`; `offsets` (the blocks' start
    bits, as compress_mode returns them) lets every block decode at once."""
    t = _type_of(dtype)
    nx, ny, nz = _dims_of(shape)
    if out is None:
        if hasattr(words, "data_ptr"):
            import torch
            out = torch.empty(tuple(shape), dtype=dtype, device=words.device)
        else:
            import numpy as np
            out = np.empty(tuple(shape), dtype)
    src, size = _addr_and_size(words)
    _check(_lib.gzfp_decompress_mode(int(t), nx, ny, nz, ctypes.byref(mode), src, size,
                                     _addr_and_size(offsets)[0] if offsets is not None else None,
                                     _addr_and_size(out)[0], _cuda_stream_handle(cuda_stream)),
           "decompress_mode")
    return out


def index_blocks(words, shape, dtype, mode: Mode, cuda_stream: Any = None):
    """Every block's start bit in a stream written under `mode`: walkers over
    segments of the stream whose block chains are joined where they merge
    (one GPU thread walks short streams, and any stream whose chains do not
    merge)."""
    t = _type_of(dtype)
    nx, ny, nz = _dims_of(shape)
    nb = _nblocks(shape)
    if hasattr(words, "data_ptr"):
        import torch
        offs = torch.empty(nb, dtype=torch.int64, device=words.device)
    else:
        import numpy as np
        offs = np.empty(nb, np.uint64)
    src, size = _addr_and_size(words)
    _check(_lib.gzfp_index_blocks(int(t), nx, ny, nz, ctypes.byref(mode), src, size,
                                  _addr_and_size(offs)[0], _cuda_stream_handle(cuda_stream)),
           "index_blocks")
    return offs


def version() -> int:
    return int(_lib.gzfp_version())


# ------------------------------------------------------------------ batches

class BatchItem(ctypes.Structure):
    """gzfp_batch_item (include/gzfp.h)."""
    _fields_ = [("type", _I), ("nx", _U), ("ny", _U), ("nz", _U), ("maxbits", _U),
                ("field", _VP), ("stream", _VP), ("stream_capacity", _SZ)]


class BatchConfig(ctypes.Structure):
    """gzfp_batch_config: threads per CTA, resident CTAs per SM, blocks per
    thread per claimed chunk, claim-ahead flag."""
    _fields_ = [("threads", _I), ("ctas_per_sm", _I), ("blocks_per_thread", _I),
                ("claim_ahead", _I)]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


_lib.gzfp_batch_default_config.restype = None
_lib.gzfp_batch_default_config.argtypes = [ctypes.POINTER(BatchConfig)]
_lib.gzfp_batch_last_error.restype = ctypes.c_char_p
for _fn in (_lib.gzfp_batch_compress, _lib.gzfp_batch_decompress):
    _fn.restype = _I
    _fn.argtypes = [ctypes.POINTER(BatchItem), _I, ctypes.POINTER(BatchConfig), _VP]
_lib.gzfp_batch_plan_create.restype = _I
_lib.gzfp_batch_plan_create.argtypes = [ctypes.POINTER(BatchItem), _I, _I,
                                        ctypes.POINTER(BatchConfig), ctypes.POINTER(_VP)]
_lib.gzfp_batch_plan_launch.restype = _I
_lib.gzfp_batch_plan_launch.argtypes = [_VP, _VP]
_lib.gzfp_batch_plan_destroy.restype = None
_lib.gzfp_batch_plan_destroy.argtypes = [_VP]
_lib.gzfp_batch_autotune.restype = _I
_lib.gzfp_batch_autotune.argtypes = [ctypes.POINTER(BatchItem), _I, _I, _I,
                                     ctypes.POINTER(BatchConfig), ctypes.POINTER(ctypes.c_float),
                                     _VP]


class BatchError(GzfpError):
    def __init__(self, status: int, what: str):
        RuntimeError.__init__(self, f"{what}: {_lib.gzfp_status_string(status).decode()} "
                                    f"({_lib.gzfp_batch_last_error().decode()})")
        self.status = status


def _bcheck(status: int, what: str) -> None:
    if status != GZFP_OK:
        raise BatchError(status, what)


def default_batch_config() -> BatchConfig:
    c = BatchConfig()
    _lib.gzfp_batch_default_config(ctypes.byref(c))
    return c


def batch_items(fields, streams, rates):
    """ctypes array of gzfp_batch_item for CUDA tensors `fields` (float32 /
    float64 / int32 / int64, 1-3 dims), stream word tensors `streams` and
    per-array rates."""
    items = (BatchItem * len(fields))()
    for i, (f, w, r) in enumerate(zip(fields, streams, rates)):
        t = _type_of(f.dtype)
        nx, ny, nz = _dims_of(f.shape)
        items[i] = BatchItem(int(t), nx, ny, nz,
                             _lib.gzfp_rate_to_maxbits(int(t), len(f.shape), float(r)),
                             f.data_ptr(), w.data_ptr(), w.numel() * w.element_size())
    return items


def batch_stream_buffers(fields, rates):
    """Word tensors sized for each array's fixed-rate stream."""
    import torch
    out = []
    for f, r in zip(fields, rates):
        t = _type_of(f.dtype)
        nx, ny, nz = _dims_of(f.shape)
        mb = _lib.gzfp_rate_to_maxbits(int(t), len(f.shape), float(r))
        out.append(torch.empty(stream_size(t, nx, ny, nz, mb) // 8, dtype=torch.int64,
                               device=f.device))
    return out


def compress_batch(fields, rates, streams=None, config: Optional[BatchConfig] = None,
                   cuda_stream: Any = None):
    """Compress many CUDA arrays with the batched kernels; returns the
    stream word tensors (one per array)."""
    if streams is None:
        streams = batch_stream_buffers(fields, rates)
    items = batch_items(fields, streams, rates)
    _bcheck(_lib.gzfp_batch_compress(items, len(items), ctypes.byref(config) if config else None,
                                     _cuda_stream_handle(cuda_stream)), "compress_batch")
    return streams


def decompress_batch(streams, fields, rates, config: Optional[BatchConfig] = None,
                     cuda_stream: Any = None):
    """Decompress many streams into the CUDA tensors `fields` (shape and
    dtype give each array's geometry)."""
    items = batch_items(fields, streams, rates)
    _bcheck(_lib.gzfp_batch_decompress(items, len(items),
                                       ctypes.byref(config) if config else None,
                                       _cuda_stream_handle(cuda_stream)), "decompress_batch")
    return fields


class BatchPlan:
    """A batch captured in a CUDA graph; launch() replays it."""

    def __init__(self, fields, streams, rates, decompress: bool = False,
                 config: Optional[BatchConfig] = None):
        self._items = batch_items(fields, streams, rates)
        self._keep = (list(fields), list(streams))
        h = _VP()
        _bcheck(_lib.gzfp_batch_plan_create(self._items, len(self._items), int(decompress),
                                            ctypes.byref(config) if config else None,
                                            ctypes.byref(h)), "BatchPlan")
        self._h = h

    def launch(self, cuda_stream: Any = None) -> None:
        _bcheck(_lib.gzfp_batch_plan_launch(self._h, _cuda_stream_handle(cuda_stream)),
                "BatchPlan.launch")

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.gzfp_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def autotune_batch(fields, streams, rates, decompress: bool = False, repeats: int = 3,
                   cuda_stream: Any = None):
    """Time every launch shape on this batch; returns (BatchConfig, ms)."""
    items = batch_items(fields, streams, rates)
    best = BatchConfig()
    ms = ctypes.c_float(0)
    _bcheck(_lib.gzfp_batch_autotune(items, len(items), int(decompress), int(repeats),
                                     ctypes.byref(best), ctypes.byref(ms),
                                     _cuda_stream_handle(cuda_stream)), "autotune_batch")
    return best, float(ms.value)


# ------------------------------------------------------------------ serving

GZFP_SERVE_COMPRESS = 0
GZFP_SERVE_DECOMPRESS = 1


class ServeRequest(ctypes.Structure):
    """gzfp_serve_request (include/gzfp.h)."""
    _fields_ = [("op", _I), ("type", _I), ("nx", _U), ("ny", _U), ("nz", _U), ("maxbits", _U),
                ("input", _VP), ("copy_to", _VP), ("arrival", ctypes.c_double)]


class ServeResult(ctypes.Structure):
    """gzfp_serve_result: host times of admission and completion; in the
    device-queue mode also the device-clock span of the request's CTAs."""
    _fields_ = [("admitted", ctypes.c_double), ("completed", ctypes.c_double),
                ("output_bytes", _SZ), ("batch", _I), ("status", _I),
                ("device_start", ctypes.c_double), ("device_end", ctypes.c_double)]


class ServeConfig(ctypes.Structure):
    """gzfp_serve_config: device_queue = 1 (the default) selects the
    device-queue mode, 0 the slot mode; idle_exit_us is the device queue's
    scheduler wait limit."""
    _fields_ = [("budget_bytes", _SZ), ("max_batch", _I), ("max_inflight", _I),
                ("compress_cfg", BatchConfig), ("decompress_cfg", BatchConfig),
                ("device_queue", _I), ("idle_exit_us", _U)]


class ServeStats(ctypes.Structure):
    """gzfp_serve_stats: wall time to the last completion, batches and
    requests per batch (device queue: publications), peak arena use, busy
    fraction, kernels launched, requests on the device when one is
    admitted, and (device queue) scheduler launches."""
    _fields_ = [("wall", ctypes.c_double), ("batches", _I), ("mean_batch", ctypes.c_double),
                ("peak_bytes", _SZ), ("busy", ctypes.c_double), ("kernels", _I),
                ("mean_inflight", ctypes.c_double), ("schedulers", _I)]

    def as_dict(self) -> dict:
        return {f: (float(getattr(self, f)) if t is ctypes.c_double else int(getattr(self, f)))
                for f, t in self._fields_}


_lib.gzfp_serve_default_config.restype = None
_lib.gzfp_serve_default_config.argtypes = [ctypes.POINTER(ServeConfig)]
_lib.gzfp_serve_run.restype = _I
_lib.gzfp_serve_run.argtypes = [ctypes.POINTER(ServeRequest), _I, ctypes.POINTER(ServeConfig),
                                ctypes.POINTER(ServeResult), ctypes.POINTER(ServeStats)]


def default_serve_config() -> ServeConfig:
    c = ServeConfig()
    _lib.gzfp_serve_default_config(ctypes.byref(c))
    return c


def serve_request(op: int, x, rate: float, arrival: float, shape=None, dtype=None,
                  copy_to=None) -> ServeRequest:
    """A request on the resident CUDA tensor ``x``: the field to compress
    (op GZFP_SERVE_COMPRESS) or the stream words to decompress into an array
    of ``shape`` / ``dtype``."""
    if op == GZFP_SERVE_COMPRESS:
        shape, dtype = x.shape, x.dtype
    t = _type_of(dtype)
    nx, ny, nz = _dims_of(shape)
    mb = _lib.gzfp_rate_to_maxbits(int(t), len(shape), float(rate))
    req = ServeRequest(op, int(t), nx, ny, nz, mb, x.data_ptr(),
                       copy_to.data_ptr() if copy_to is not None else None, float(arrival))
    req._keep = (x, copy_to)  # the request holds raw pointers: keep the tensors alive
    return req


def serve(requests, config: Optional[ServeConfig] = None):
    """Run the request server over ``requests`` (a sequence of ServeRequest);
    returns (list of ServeResult, ServeStats)."""
    reqs = (ServeRequest * len(requests))(*requests)
    res = (ServeResult * len(requests))()
    stats = ServeStats()
    _bcheck(_lib.gzfp_serve_run(reqs, len(requests), ctypes.byref(config) if config else None,
                                res, ctypes.byref(stats)), "serve")
    return list(res), stats


__all__ = [
    "GzfpError", "zfp_type", "zfp_stream", "zfp_field", "zfp_stream_open", "zfp_field_1d",
    "zfp_field_2d", "zfp_field_3d", "zfp_field_dimensionality", "zfp_type_size",
    "stream_set_rate", "zfp_stream_maximum_size", "stream_size", "compress", "decompress",
    "compress_tensor", "decompress_tensor", "version", "LIB_PATH", "BatchItem", "BatchConfig",
    "default_batch_config", "compress_batch", "decompress_batch", "BatchPlan", "autotune_batch",
    "batch_stream_buffers", "ServeRequest", "ServeResult", "ServeConfig", "ServeStats",
    "default_serve_config", "serve_request", "serve", "GZFP_SERVE_COMPRESS",
    "GZFP_SERVE_DECOMPRESS", "HEADER_MAX_BITS", "write_header", "read_header", "headed_size",
    "compress_headed", "decompress_headed", "decode_blocks", "encode_blocks", "Mode",
    "mode_rate", "mode_precision", "mode_accuracy", "mode_maximum_size", "compress_mode",
    "decompress_mode", "index_blocks", "read_header_mode", "write_header_mode",
    "compress_mode_headed", "zfp_stream_set_precision", "zfp_stream_set_accuracy",
]
