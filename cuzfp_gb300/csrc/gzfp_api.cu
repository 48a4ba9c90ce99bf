// gzfp_api.cu -- host side of the C ABI declared in include/gzfp.h.
//
// Validates arguments, computes fixed-rate sizes, detects host vs device
// pointers (cuZFP's is_gpu_ptr, src/cuZFP/pointers.cuh:12-22, with the CUDA
// 10+ `type` field), stages host buffers through a per-device workspace and
// launches the kernels of gzfp_enc_*.cu / gzfp_dec_*.cu.  There is no CPU
// code path: every compression or decompression runs on the GPU.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "gzfp.h"
#include "gzfp_launch.h"

namespace {

thread_local char g_last_error[512];

void clear_error() { g_last_error[0] = 0; }

int fail(int status, const char* msg) {
  snprintf(g_last_error, sizeof g_last_error, "%s", msg);
  return status;
}

int cuda_fail(cudaError_t e, const char* what) {
  snprintf(g_last_error, sizeof g_last_error, "%s: %s", what, cudaGetErrorString(e));
  return GZFP_ERR_CUDA;
}

constexpr unsigned kMaxBitsLimit = 1u << 20;

bool known_type(int type) {
  return type == GZFP_TYPE_FLOAT || type == GZFP_TYPE_DOUBLE || type == GZFP_TYPE_INT32 ||
         type == GZFP_TYPE_INT64;
}

// exponent bits of a block header: none for integer fields
int ebits_of(int type) {
  return type == GZFP_TYPE_FLOAT ? 8 : type == GZFP_TYPE_DOUBLE ? 11 : 0;
}

size_t scalar_size(int type) {
  return type == GZFP_TYPE_FLOAT || type == GZFP_TYPE_INT32 ? 4 : 8;
}

// Field geometry; ny = 0 selects 1D, nz = 0 selects 2D (zfp_field_1d/2d/3d).
bool make_geom(unsigned nx, unsigned ny, unsigned nz, gzfp::Geom& g, int& dims) {
  if (nx == 0 || (nz != 0 && ny == 0)) return false;
  dims = nz ? 3 : ny ? 2 : 1;
  g = gzfp::make_geom_blocks(nx, ny ? ny : 1, nz ? nz : 1);
  return g.nblocks < (1ull << 32);  // block indices are 32-bit on the device
}

// Rows of full blocks move as one vector when every row start is aligned:
// 16 bytes for 4-byte values, 32 for 8-byte values.
uint32_t rows_vectorizable(const void* p, unsigned nx, int type) {
  const uintptr_t a = 4 * scalar_size(type);
  return (nx % 4 == 0 && (uintptr_t)p % a == 0) ? 1u : 0u;
}

bool is_device_pointer(const void* p) {
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();  // not a CUDA allocation: clear the sticky-free error
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Host-staged calls are cut into slabs of whole block layers along the
// slowest axis (z in 3D, y in 2D, x in 1D).  A slab's values are one
// contiguous run of the array and its blocks one contiguous run of the
// stream; the slab height is chosen so that every slab boundary falls on a
// 64-bit word, so each slab is coded as an independent array and its stream
// is exactly the matching word range of the whole stream.  Slabs rotate over
// kSlots device buffers, each with its own CUDA stream: the upload of one
// slab, the kernel of the previous one and the download of the one before
// that overlap, so the call runs at the speed of the host link rather than
// the sum of copies and kernels.
constexpr int kSlots = 3;
constexpr uint64_t kSlabTarget = 32ull << 20;  // field bytes per slab

struct Slot {
  void* field = nullptr;
  size_t field_cap = 0;
  void* stream = nullptr;
  size_t stream_cap = 0;
  cudaStream_t cs = nullptr;
};

// Staging state of one device, created on first use and kept for the life
// of the process.
struct Workspace {
  std::mutex mu;
  Slot slot[kSlots];
  cudaEvent_t start = nullptr;
};
constexpr int kMaxDevices = 64;
Workspace g_ws[kMaxDevices];

cudaError_t reserve(void*& p, size_t& cap, size_t need) {
  if (cap >= need) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(&p, need);
  if (e == cudaSuccess) cap = need;
  return e;
}

cudaError_t init_workspace(Workspace& ws) {
  cudaError_t e = cudaSuccess;
  if (!ws.start && (e = cudaEventCreateWithFlags(&ws.start, cudaEventDisableTiming))) return e;
  for (Slot& sl : ws.slot)
    if (!sl.cs && (e = cudaStreamCreateWithFlags(&sl.cs, cudaStreamNonBlocking))) return e;
  return e;
}

// Slab decomposition of an array: `layers` block layers of `layer_blocks`
// blocks and 4 planes of `plane_values` values each (the last layer may
// hold fewer than 4 of the axis' `extent` planes), `per_slab` layers a slab.
struct Slabs {
  int dims;
  unsigned nx, ny;
  uint64_t extent, layers, layer_blocks, plane_values, per_slab, count;
};

Slabs plan_slabs(const gzfp::Geom& g, int dims, unsigned maxbits, size_t scalar) {
  Slabs p;
  p.dims = dims;
  p.nx = g.nx;
  p.ny = g.ny;
  if (dims == 3) {
    p.extent = g.nz, p.layers = g.bz, p.layer_blocks = (uint64_t)g.bx * g.by;
    p.plane_values = (uint64_t)g.nx * g.ny;
  } else if (dims == 2) {
    p.extent = g.ny, p.layers = g.by, p.layer_blocks = g.bx, p.plane_values = g.nx;
  } else {
    p.extent = g.nx, p.layers = g.bx, p.layer_blocks = 1, p.plane_values = 1;
  }
  // slab boundaries on whole words: per_slab * layer_blocks * maxbits % 64 == 0
  const uint64_t bits = p.layer_blocks * maxbits;
  int tz = 0;
  while (tz < 6 && !((bits >> tz) & 1)) tz++;
  const uint64_t quantum = 64ull >> tz;
  const uint64_t layer_bytes = 4 * p.plane_values * scalar;
  uint64_t per = kSlabTarget / layer_bytes / quantum * quantum;
  if (per < quantum) per = quantum;
  if (per >= p.layers) per = p.layers;
  p.per_slab = per;
  p.count = (p.layers + per - 1) / per;
  return p;
}

// Slab j: first plane, plane count, first block, block count, and the
// array geometry it is coded as.
struct Slab {
  uint64_t plane0, planes, block0, blocks;
  gzfp::Geom g;
};

Slab slab_at(const Slabs& p, uint64_t j) {
  Slab s;
  const uint64_t l0 = j * p.per_slab;
  const uint64_t l1 = l0 + p.per_slab < p.layers ? l0 + p.per_slab : p.layers;
  s.plane0 = 4 * l0;
  s.planes = (4 * l1 < p.extent ? 4 * l1 : p.extent) - s.plane0;
  s.block0 = l0 * p.layer_blocks;
  s.blocks = (l1 - l0) * p.layer_blocks;
  const unsigned n = (unsigned)s.planes;
  s.g = p.dims == 3   ? gzfp::make_geom_blocks(p.nx, p.ny, n)
        : p.dims == 2 ? gzfp::make_geom_blocks(p.nx, n, 1)
                      : gzfp::make_geom_blocks(n, 1, 1);
  return s;
}

int check_common(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                 gzfp::Geom& g, int& dims) {
  if (!known_type(type)) return fail(GZFP_ERR_ARG, "unknown scalar type");
  if (!make_geom(nx, ny, nz, g, dims))
    return fail(GZFP_ERR_ARG, "bad dimensions (nx must be > 0; nz > 0 needs ny > 0; under 2^32 blocks)");
  if (maxbits < (unsigned)ebits_of(type) + 1 || maxbits > kMaxBitsLimit)
    return fail(GZFP_ERR_ARG, "bits per block out of range");
  return GZFP_OK;
}

uint64_t stream_words(const gzfp::Geom& g, unsigned maxbits) {
  return (g.nblocks * maxbits + 63) / 64;
}

}  // namespace

extern "C" {

int gzfp_version(void) { return 10000; }

const char* gzfp_status_string(int status) {
  switch (status) {
    case GZFP_OK: return "ok";
    case GZFP_ERR_ARG: return "invalid argument";
    case GZFP_ERR_UNSUPPORTED: return "unsupported field or mode";
    case GZFP_ERR_CAPACITY: return "buffer too small";
    case GZFP_ERR_CUDA: return "CUDA error";
    default: return "unknown status";
  }
}

const char* gzfp_last_error(void) { return g_last_error; }

unsigned gzfp_rate_to_maxbits(int type, unsigned dims, double rate) {
  if (!known_type(type) || dims < 1 || dims > 3) return 0;
  if (!(rate >= 0) || rate > 1e6) return 0;
  unsigned n = 1u << (2 * dims);
  unsigned bits = (unsigned)floor(n * rate + 0.5);
  // zfp raises float and double blocks to 1 + exponent bits and leaves
  // integer blocks alone (Z/src/zfp.c:409-419); 0 bits is not a stream
  unsigned lo = ebits_of(type) ? 1u + (unsigned)ebits_of(type) : 0u;
  return bits < lo ? lo : bits;
}

size_t gzfp_stream_size(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits) {
  gzfp::Geom g;
  int dims;
  if (!known_type(type) || !make_geom(nx, ny, nz, g, dims)) return 0;
  return (size_t)(stream_words(g, maxbits) * 8);
}

size_t gzfp_maximum_size(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits) {
  gzfp::Geom g;
  int dims;
  if (!known_type(type) || !make_geom(nx, ny, nz, g, dims)) return 0;
  // zfp_stream_maximum_size: min(maxbits, bits of a block coded in full),
  // raised to minbits -- which equals maxbits in fixed-rate mode -- plus the
  // 148 header bits, rounded up to a 64-bit word
  (void)dims;
  const uint64_t b = maxbits;
  return (size_t)(((148 + g.nblocks * b + 63) & ~63ull) / 8);
}

}  // extern "C"

namespace {

cudaError_t encode_launch(int type, int dims, const void* in, const gzfp::Geom& g,
                          unsigned maxbits, uint64_t* out, uint64_t nwords, cudaStream_t s) {
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return gzfp::launch_encode_f32(dims, (const float*)in, g, maxbits, out, nwords, s);
    case GZFP_TYPE_DOUBLE:
      return gzfp::launch_encode_f64(dims, (const double*)in, g, maxbits, out, nwords, s);
    case GZFP_TYPE_INT32:
      return gzfp::launch_encode_i32(dims, (const int32_t*)in, g, maxbits, out, nwords, s);
    default:
      return gzfp::launch_encode_i64(dims, (const int64_t*)in, g, maxbits, out, nwords, s);
  }
}

cudaError_t decode_launch(int type, int dims, const uint64_t* in, uint64_t nwords,
                          const gzfp::Geom& g, unsigned maxbits, void* out, cudaStream_t s) {
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return gzfp::launch_decode_f32(dims, in, nwords, g, maxbits, (float*)out, s);
    case GZFP_TYPE_DOUBLE:
      return gzfp::launch_decode_f64(dims, in, nwords, g, maxbits, (double*)out, s);
    case GZFP_TYPE_INT32:
      return gzfp::launch_decode_i32(dims, in, nwords, g, maxbits, (int32_t*)out, s);
    default:
      return gzfp::launch_decode_i64(dims, in, nwords, g, maxbits, (int64_t*)out, s);
  }
}

// One host-staged call: slabs through the workspace's slots (see Slabs).
// `field` / `words` are the caller's pointers; dev_field / dev_words say
// which of them are device memory.  Returns after the last slab has landed.
int staged(bool decode, int type, int dims, const gzfp::Geom& g, unsigned maxbits, void* field,
           bool dev_field, uint64_t* words, bool dev_words, cudaStream_t s) {
  const size_t scalar = scalar_size(type);
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (device < 0 || device >= kMaxDevices) return fail(GZFP_ERR_CUDA, "device index out of range");
  Workspace& ws = g_ws[device];
  std::lock_guard<std::mutex> lock(ws.mu);
  if ((e = init_workspace(ws))) return cuda_fail(e, "staging streams");
  const Slabs p = plan_slabs(g, dims, maxbits, scalar);
  const uint64_t slab_values = 4 * p.per_slab * p.plane_values;
  const uint64_t slab_words = (p.per_slab * p.layer_blocks * maxbits + 63) / 64;
  for (int k = 0; k < kSlots && (uint64_t)k < p.count; k++) {
    Slot& sl = ws.slot[k];
    if (!dev_field && (e = reserve(sl.field, sl.field_cap, (size_t)(slab_values * scalar))))
      return cuda_fail(e, "cudaMalloc(field staging)");
    if (!dev_words && (e = reserve(sl.stream, sl.stream_cap, (size_t)(slab_words * 8))))
      return cuda_fail(e, "cudaMalloc(stream staging)");
  }
  // work the caller queued on `s` (say, the kernel that filled a device
  // field) comes first
  if ((e = cudaEventRecord(ws.start, s))) return cuda_fail(e, "cudaEventRecord");
  for (int k = 0; k < kSlots; k++)
    if ((e = cudaStreamWaitEvent(ws.slot[k].cs, ws.start, 0)))
      return cuda_fail(e, "cudaStreamWaitEvent");
  int st = GZFP_OK;
  for (uint64_t j = 0; j < p.count && !st; j++) {
    Slot& sl = ws.slot[j % kSlots];
    const cudaStream_t cs = sl.cs;
    const Slab b = slab_at(p, j);
    const size_t fbytes = (size_t)(b.planes * p.plane_values * scalar);
    char* hf = (char*)field + b.plane0 * p.plane_values * scalar;  // this slab of the field
    const uint64_t w0 = b.block0 * maxbits / 64;                   // word-aligned by plan_slabs
    const uint64_t nw = (b.blocks * maxbits + 63) / 64;
    uint64_t* hw = words + w0;
    void* df = dev_field ? (void*)hf : sl.field;
    uint64_t* dw = dev_words ? hw : (uint64_t*)sl.stream;
    gzfp::Geom gs = b.g;
    gs.vec = rows_vectorizable(df, p.nx, type);
    if (!decode) {
      if (!dev_field && (e = cudaMemcpyAsync(df, hf, fbytes, cudaMemcpyHostToDevice, cs))) {
        st = cuda_fail(e, "cudaMemcpyAsync(field H2D)");
        break;
      }
      if (maxbits % 64 && (e = cudaMemsetAsync(dw, 0, (size_t)(nw * 8), cs))) {
        st = cuda_fail(e, "cudaMemsetAsync(stream)");  // blocks share edge words
        break;
      }
      if ((e = encode_launch(type, dims, df, gs, maxbits, dw, nw, cs))) {
        st = cuda_fail(e, "encode kernel launch");
        break;
      }
      if (!dev_words && (e = cudaMemcpyAsync(hw, dw, (size_t)(nw * 8), cudaMemcpyDeviceToHost, cs)))
        st = cuda_fail(e, "cudaMemcpyAsync(stream D2H)");
    } else {
      if (!dev_words && (e = cudaMemcpyAsync(dw, hw, (size_t)(nw * 8), cudaMemcpyHostToDevice, cs))) {
        st = cuda_fail(e, "cudaMemcpyAsync(stream H2D)");
        break;
      }
      if ((e = decode_launch(type, dims, dw, nw, gs, maxbits, df, cs))) {
        st = cuda_fail(e, "decode kernel launch");
        break;
      }
      if (!dev_field && (e = cudaMemcpyAsync(hf, df, fbytes, cudaMemcpyDeviceToHost, cs)))
        st = cuda_fail(e, "cudaMemcpyAsync(field D2H)");
    }
  }
  // nothing of this call stays in flight, on success or not
  for (int k = 0; k < kSlots; k++) {
    cudaError_t es = cudaStreamSynchronize(ws.slot[k].cs);
    if (es && !st) st = cuda_fail(es, "cudaStreamSynchronize");
  }
  return st;
}

}  // namespace

extern "C" {

int gzfp_compress_bits(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                       const void* data, void* stream, size_t capacity, size_t* out_bytes,
                       void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  int st = check_common(type, nx, ny, nz, maxbits, g, dims);
  if (st) return st;
  if (!data || !stream) return fail(GZFP_ERR_ARG, "null pointer");
  const uint64_t nwords = stream_words(g, maxbits);
  const size_t bytes = (size_t)(nwords * 8);
  if (capacity < bytes) return fail(GZFP_ERR_CAPACITY, "stream buffer smaller than the compressed size");
  if (out_bytes) *out_bytes = bytes;
  if (g.nblocks == 0) return GZFP_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const bool dev_data = is_device_pointer(data);
  const bool dev_stream = is_device_pointer(stream);
  if (!dev_data || !dev_stream)
    return staged(false, type, dims, g, maxbits, (void*)data, dev_data, (uint64_t*)stream,
                  dev_stream, s);
  cudaError_t e;
  if (maxbits % 64 != 0) {
    // blocks share boundary words, which the kernel ORs into a zeroed stream
    if ((e = cudaMemsetAsync(stream, 0, bytes, s))) return cuda_fail(e, "cudaMemsetAsync(stream)");
  }
  g.vec = rows_vectorizable(data, nx, type);
  if ((e = encode_launch(type, dims, data, g, maxbits, (uint64_t*)stream, nwords, s)))
    return cuda_fail(e, "encode kernel launch");
  return GZFP_OK;
}

int gzfp_decompress_bits(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                         const void* stream, size_t bytes, void* data, void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  int st = check_common(type, nx, ny, nz, maxbits, g, dims);
  if (st) return st;
  if (!data || !stream) return fail(GZFP_ERR_ARG, "null pointer");
  const uint64_t nwords = stream_words(g, maxbits);
  const size_t need = (size_t)(nwords * 8);
  if (bytes < need) return fail(GZFP_ERR_ARG, "stream shorter than the compressed size");
  if (g.nblocks == 0) return GZFP_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const bool dev_data = is_device_pointer(data);
  const bool dev_stream = is_device_pointer(stream);
  if (!dev_data || !dev_stream)
    return staged(true, type, dims, g, maxbits, data, dev_data, (uint64_t*)stream, dev_stream, s);
  g.vec = rows_vectorizable(data, nx, type);
  cudaError_t e = decode_launch(type, dims, (const uint64_t*)stream, nwords, g, maxbits, data, s);
  if (e) return cuda_fail(e, "decode kernel launch");
  return GZFP_OK;
}

}  // extern "C"

namespace {

// Apply zfp's stride defaults (0 = contiguous along that axis) and decide
// whether rows of full blocks can move as vectors: unit x stride and every
// row start aligned.
void set_strides(gzfp::Geom& g, int dims, int type, const void* p, long long sx, long long sy,
                 long long sz) {
  g.sx = sx ? sx : 1;
  g.sy = sy ? sy : (long long)g.nx;
  g.sz = sz ? sz : (long long)g.nx * g.ny;
  const long long a = 4 * (long long)scalar_size(type), S = (long long)scalar_size(type);
  g.vec = (g.sx == 1 && g.nx % 4 == 0 && (uintptr_t)p % a == 0 && (dims < 2 || (g.sy * S) % a == 0) &&
           (dims < 3 || (g.sz * S) % a == 0))
              ? 1u
              : 0u;
}

// The element offsets, relative to the field pointer, of the lowest and the
// highest value a strided field reaches.
void stride_span(const gzfp::Geom& g, long long& lo, long long& hi) {
  lo = hi = 0;
  const long long n[3] = {g.nx, g.ny, g.nz}, st[3] = {g.sx, g.sy, g.sz};
  for (int a = 0; a < 3; a++) {
    const long long e = (n[a] - 1) * st[a];
    lo += e < 0 ? e : 0;
    hi += e > 0 ? e : 0;
  }
}

// One call on a field with element strides (0 = contiguous along that axis),
// everything staged at once.  `base` is the stream bit of block 0: a headed
// stream's header length, whose `header` words the encoder writes in front
// of the blocks.
int strided_call(bool decode, int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                 long long sy, long long sz, unsigned maxbits, void* field, uint64_t* words,
                 size_t words_bytes, size_t* out_bytes, void* cuda_stream, uint64_t base = 0,
                 const uint64_t* header = nullptr, unsigned header_words = 0) {
  clear_error();
  gzfp::Geom g;
  int dims;
  int st = check_common(type, nx, ny, nz, maxbits, g, dims);
  if (st) return st;
  if (!field || !words) return fail(GZFP_ERR_ARG, "null pointer");
  g.base = base;
  const uint64_t nwords = (base + g.nblocks * maxbits + 63) / 64;
  // blocks share boundary words (with each other or with the header): the
  // encoder ORs those into a zeroed stream
  const bool shared_words = maxbits % 64 || base % 64;
  const size_t need = (size_t)(nwords * 8);
  if (words_bytes < need)
    return fail(decode ? GZFP_ERR_ARG : GZFP_ERR_CAPACITY,
                decode ? "stream shorter than the compressed size"
                       : "stream buffer smaller than the compressed size");
  if (out_bytes) *out_bytes = need;
  if (g.nblocks == 0) return GZFP_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const size_t S = scalar_size(type);
  const bool dev_field = is_device_pointer(field), dev_words = is_device_pointer(words);
  cudaError_t e;
  if (dev_field && dev_words) {
    set_strides(g, dims, type, field, sx, sy, sz);
    if (!decode && shared_words && (e = cudaMemsetAsync(words, 0, need, s)))
      return cuda_fail(e, "cudaMemsetAsync(stream)");
    if (!decode && header &&
        (e = cudaMemcpyAsync(words, header, header_words * 8, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "cudaMemcpyAsync(header H2D)");
    e = decode ? decode_launch(type, dims, words, nwords, g, maxbits, field, s)
               : encode_launch(type, dims, field, g, maxbits, words, nwords, s);
    return e ? cuda_fail(e, decode ? "decode kernel launch" : "encode kernel launch") : GZFP_OK;
  }
  // host memory: stage the span the strides reach, and the stream
  set_strides(g, dims, type, nullptr, sx, sy, sz);
  long long lo, hi;
  stride_span(g, lo, hi);
  const size_t span = (size_t)(hi - lo + 1) * S;
  int device = 0;
  if ((e = cudaGetDevice(&device))) return cuda_fail(e, "cudaGetDevice");
  if (device < 0 || device >= kMaxDevices) return fail(GZFP_ERR_CUDA, "device index out of range");
  Workspace& ws = g_ws[device];
  std::lock_guard<std::mutex> lock(ws.mu);
  Slot& sl = ws.slot[0];
  char* hfield = (char*)field + lo * (long long)S;  // lowest value reached
  char* dfield = (char*)field;
  if (!dev_field) {
    if ((e = reserve(sl.field, sl.field_cap, span))) return cuda_fail(e, "cudaMalloc(field staging)");
    dfield = (char*)sl.field - lo * (long long)S;  // the kernel's field pointer
  }
  uint64_t* dwords = words;
  if (!dev_words) {
    if ((e = reserve(sl.stream, sl.stream_cap, need))) return cuda_fail(e, "cudaMalloc(stream staging)");
    dwords = (uint64_t*)sl.stream;
  }
  set_strides(g, dims, type, dfield, sx, sy, sz);
  st = GZFP_OK;
  if (!dev_field && (e = cudaMemcpyAsync(sl.field, hfield, span, cudaMemcpyHostToDevice, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(field H2D)");
  if (!st && decode && !dev_words &&
      (e = cudaMemcpyAsync(dwords, words, need, cudaMemcpyHostToDevice, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(stream H2D)");
  if (!st && !decode && shared_words && (e = cudaMemsetAsync(dwords, 0, need, s)))
    st = cuda_fail(e, "cudaMemsetAsync(stream)");
  if (!st && !decode && header &&
      (e = cudaMemcpyAsync(dwords, header, header_words * 8, cudaMemcpyHostToDevice, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(header H2D)");
  if (!st) {
    e = decode ? decode_launch(type, dims, dwords, nwords, g, maxbits, dfield, s)
               : encode_launch(type, dims, dfield, g, maxbits, dwords, nwords, s);
    if (e) st = cuda_fail(e, decode ? "decode kernel launch" : "encode kernel launch");
  }
  if (!st && decode && !dev_field &&
      (e = cudaMemcpyAsync(hfield, sl.field, span, cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(field D2H)");
  if (!st && !decode && !dev_words &&
      (e = cudaMemcpyAsync(words, dwords, need, cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(stream D2H)");
  const cudaError_t es = cudaStreamSynchronize(s);  // nothing stays in flight
  if (!st && es) st = cuda_fail(es, "cudaStreamSynchronize");
  return st;
}

}  // namespace

extern "C" {

int gzfp_compress_strided(int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                          long long sy, long long sz, unsigned maxbits, const void* data,
                          void* stream, size_t capacity, size_t* out_bytes, void* cuda_stream) {
  return strided_call(false, type, nx, ny, nz, sx, sy, sz, maxbits, (void*)data,
                      (uint64_t*)stream, capacity, out_bytes, cuda_stream);
}

int gzfp_decompress_strided(int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                            long long sy, long long sz, unsigned maxbits, const void* stream,
                            size_t bytes, void* data, void* cuda_stream) {
  return strided_call(true, type, nx, ny, nz, sx, sy, sz, maxbits, data, (uint64_t*)stream, bytes,
                      nullptr, cuda_stream);
}

int gzfp_compress(int type, unsigned nx, unsigned ny, unsigned nz, double rate, const void* data,
                  void* stream, size_t capacity, size_t* out_bytes, void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  if (!make_geom(nx, ny, nz, g, dims)) return fail(GZFP_ERR_ARG, "bad dimensions");
  unsigned maxbits = gzfp_rate_to_maxbits(type, (unsigned)dims, rate);
  if (!maxbits) return fail(GZFP_ERR_ARG, "bad type or rate");
  return gzfp_compress_bits(type, nx, ny, nz, maxbits, data, stream, capacity, out_bytes,
                            cuda_stream);
}

int gzfp_decompress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                    const void* stream, size_t bytes, void* data, void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  if (!make_geom(nx, ny, nz, g, dims)) return fail(GZFP_ERR_ARG, "bad dimensions");
  unsigned maxbits = gzfp_rate_to_maxbits(type, (unsigned)dims, rate);
  if (!maxbits) return fail(GZFP_ERR_ARG, "bad type or rate");
  return gzfp_decompress_bits(type, nx, ny, nz, maxbits, stream, bytes, data, cuda_stream);
}

}  // extern "C"

// ------------------------------------------------------------ block access
namespace {

cudaError_t blocks_launch(bool decode, int type, int dims, unsigned maxbits, uint64_t* words,
                          uint64_t nwords, const unsigned long long* index, const uint8_t* shape,
                          uint64_t count, void* tiles, cudaStream_t s) {
  using namespace gzfp;
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return decode ? launch_decode_blocks<float>(dims, words, nwords, index, shape, count, maxbits,
                                                  (float*)tiles, s)
                    : launch_encode_blocks<float>(dims, (const float*)tiles, index, shape, count,
                                                  maxbits, words, nwords, s);
    case GZFP_TYPE_DOUBLE:
      return decode ? launch_decode_blocks<double>(dims, words, nwords, index, shape, count,
                                                   maxbits, (double*)tiles, s)
                    : launch_encode_blocks<double>(dims, (const double*)tiles, index, shape, count,
                                                   maxbits, words, nwords, s);
    case GZFP_TYPE_INT32:
      return decode ? launch_decode_blocks<int32_t>(dims, words, nwords, index, shape, count,
                                                    maxbits, (int32_t*)tiles, s)
                    : launch_encode_blocks<int32_t>(dims, (const int32_t*)tiles, index, shape,
                                                    count, maxbits, words, nwords, s);
    default:
      return decode ? launch_decode_blocks<int64_t>(dims, words, nwords, index, shape, count,
                                                    maxbits, (int64_t*)tiles, s)
                    : launch_encode_blocks<int64_t>(dims, (const int64_t*)tiles, index, shape,
                                                    count, maxbits, words, nwords, s);
  }
}

// Host buffers go through the workspace of the current device: tiles and
// stream in slot 0, indices and shapes in slot 1.
int blocks_call(bool decode, int type, unsigned dims, unsigned maxbits, uint64_t* words,
                size_t bytes, const unsigned long long* index, const uint8_t* shape, size_t count,
                void* tiles, void* cuda_stream) {
  clear_error();
  if (!known_type(type)) return fail(GZFP_ERR_ARG, "unknown scalar type");
  if (dims < 1 || dims > 3) return fail(GZFP_ERR_ARG, "dims must be 1, 2 or 3");
  if (maxbits < (unsigned)ebits_of(type) + 1 || maxbits > kMaxBitsLimit)
    return fail(GZFP_ERR_ARG, "bits per block out of range");
  if (count == 0) return GZFP_OK;
  if (!words || !index || !tiles) return fail(GZFP_ERR_ARG, "null pointer");
  const uint64_t nwords = bytes / 8;
  const size_t tile_bytes = count * ((size_t)1 << (2 * dims)) * scalar_size(type);
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const bool dev_words = is_device_pointer(words), dev_index = is_device_pointer(index);
  const bool dev_shape = !shape || is_device_pointer(shape), dev_tiles = is_device_pointer(tiles);
  cudaError_t e;
  if (dev_words && dev_index && dev_shape && dev_tiles) {
    e = blocks_launch(decode, type, (int)dims, maxbits, words, nwords, index, shape, count, tiles, s);
    return e ? cuda_fail(e, "block kernel launch") : GZFP_OK;
  }
  int device = 0;
  if ((e = cudaGetDevice(&device))) return cuda_fail(e, "cudaGetDevice");
  if (device < 0 || device >= kMaxDevices) return fail(GZFP_ERR_CUDA, "device index out of range");
  Workspace& ws = g_ws[device];
  std::lock_guard<std::mutex> lock(ws.mu);
  Slot &s0 = ws.slot[0], &s1 = ws.slot[1];
  uint64_t* dw = words;
  const unsigned long long* di = index;
  const uint8_t* dsh = shape;
  void* dt = tiles;
  const size_t wbytes = (size_t)nwords * 8;
  if (!dev_words && (e = reserve(s0.stream, s0.stream_cap, wbytes ? wbytes : 8)))
    return cuda_fail(e, "cudaMalloc(stream staging)");
  if (!dev_tiles && (e = reserve(s0.field, s0.field_cap, tile_bytes)))
    return cuda_fail(e, "cudaMalloc(tile staging)");
  if (!dev_index && (e = reserve(s1.field, s1.field_cap, count * 8)))
    return cuda_fail(e, "cudaMalloc(index staging)");
  if (!dev_shape && (e = reserve(s1.stream, s1.stream_cap, count)))
    return cuda_fail(e, "cudaMalloc(shape staging)");
  int st = GZFP_OK;
  auto h2d = [&](void* dst, const void* src, size_t n, const char* what) {
    if (!st && (e = cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s))) st = cuda_fail(e, what);
  };
  if (!dev_words) {
    dw = (uint64_t*)s0.stream;
    h2d(dw, words, wbytes, "cudaMemcpyAsync(stream H2D)");
  }
  if (!dev_index) {
    di = (const unsigned long long*)s1.field;
    h2d((void*)di, index, count * 8, "cudaMemcpyAsync(indices H2D)");
  }
  if (!dev_shape) {
    dsh = (const uint8_t*)s1.stream;
    h2d((void*)dsh, shape, count, "cudaMemcpyAsync(shapes H2D)");
  }
  if (!dev_tiles) {
    dt = s0.field;
    // decoding a partial block leaves the rest of its tile as it was
    h2d(dt, tiles, tile_bytes, "cudaMemcpyAsync(tiles H2D)");
  }
  if (!st && (e = blocks_launch(decode, type, (int)dims, maxbits, dw, nwords, di, dsh, count, dt, s)))
    st = cuda_fail(e, "block kernel launch");
  if (!st && decode && !dev_tiles &&
      (e = cudaMemcpyAsync(tiles, dt, tile_bytes, cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(tiles D2H)");
  if (!st && !decode && !dev_words &&
      (e = cudaMemcpyAsync(words, dw, wbytes, cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(stream D2H)");
  const cudaError_t es = cudaStreamSynchronize(s);  // nothing stays in flight
  if (!st && es) st = cuda_fail(es, "cudaStreamSynchronize");
  return st;
}

}  // namespace

extern "C" {

int gzfp_decode_blocks(int type, unsigned dims, unsigned maxbits, const void* stream,
                       size_t bytes, const unsigned long long* indices,
                       const unsigned char* shapes, size_t count, void* tiles, void* cuda_stream) {
  return blocks_call(true, type, dims, maxbits, (uint64_t*)stream, bytes, indices, shapes, count,
                     tiles, cuda_stream);
}

int gzfp_encode_blocks(int type, unsigned dims, unsigned maxbits, const void* tiles,
                       const unsigned long long* indices, const unsigned char* shapes,
                       size_t count, void* stream, size_t bytes, void* cuda_stream) {
  return blocks_call(false, type, dims, maxbits, (uint64_t*)stream, bytes, indices, shapes, count,
                     (void*)tiles, cuda_stream);
}

}  // extern "C"

// ------------------------------------------------------------ general modes
namespace {

// Device buffers of the general-mode calls on one device, grown on demand
// and kept for the life of the process.
struct ModeSpace {
  std::mutex mu;
  void* scratch = nullptr;  size_t scratch_cap = 0;   // one slot per block
  void* lengths = nullptr;  size_t lengths_cap = 0;
  void* offsets = nullptr;  size_t offsets_cap = 0;
  void* sums = nullptr;     size_t sums_cap = 0;      // scan partials + total; walk end
  void* field = nullptr;    size_t field_cap = 0;     // staged host field
  void* stream = nullptr;   size_t stream_cap = 0;    // staged host stream
};
ModeSpace g_mode[kMaxDevices];

int mode_space(ModeSpace*& ms) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (device < 0 || device >= kMaxDevices) return fail(GZFP_ERR_CUDA, "device index out of range");
  ms = &g_mode[device];
  return GZFP_OK;
}

unsigned precision_bits(int type) {
  return type == GZFP_TYPE_FLOAT || type == GZFP_TYPE_INT32 ? 32 : 64;
}

// zfp_stream_set_params' checks (zfp-0.5.0/src/zfp.c:499-510), plus room
// for the header of a floating-point block and this library's block limit
int check_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* m,
               gzfp::Geom& g, int& dims) {
  if (!m) return fail(GZFP_ERR_ARG, "null mode");
  if (!known_type(type)) return fail(GZFP_ERR_ARG, "unknown scalar type");
  if (!make_geom(nx, ny, nz, g, dims))
    return fail(GZFP_ERR_ARG, "bad dimensions (nx must be > 0; nz > 0 needs ny > 0; under 2^32 blocks)");
  if (m->minbits > m->maxbits || m->maxprec == 0 || m->maxprec > 64)
    return fail(GZFP_ERR_ARG, "bad mode (minbits > maxbits, or maxprec outside 1..64)");
  if (m->maxbits < (unsigned)ebits_of(type) + 1 || m->maxbits > kMaxBitsLimit)
    return fail(GZFP_ERR_ARG, "bits per block out of range");
  return GZFP_OK;
}

// parameters whose blocks are exactly the fixed-rate path's
bool fixed_rate_mode(int type, const gzfp_mode* m) {
  const bool ints = type == GZFP_TYPE_INT32 || type == GZFP_TYPE_INT64;
  return m->minbits == m->maxbits && m->maxprec >= precision_bits(type) &&
         (ints || m->minexp == -1074);
}

gzfp::General general_of(const gzfp_mode* m) {
  return gzfp::General{m->minbits, m->maxbits, m->maxprec, m->minexp};
}

uint32_t mode_block_bound(int type, int dims, const gzfp_mode* m) {
  return gzfp::block_bound_host(dims, (int)precision_bits(type), ebits_of(type), general_of(m));
}

cudaError_t encode_mode_launch(int type, int dims, const void* in, const gzfp::Geom& g,
                               const gzfp::General& mode, uint64_t* scratch, uint32_t slot_words,
                               uint32_t* lengths, cudaStream_t s) {
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return gzfp::launch_encode_mode<float>(dims, (const float*)in, g, mode, scratch, slot_words, lengths, s);
    case GZFP_TYPE_DOUBLE:
      return gzfp::launch_encode_mode<double>(dims, (const double*)in, g, mode, scratch, slot_words, lengths, s);
    case GZFP_TYPE_INT32:
      return gzfp::launch_encode_mode<int32_t>(dims, (const int32_t*)in, g, mode, scratch, slot_words, lengths, s);
    default:
      return gzfp::launch_encode_mode<int64_t>(dims, (const int64_t*)in, g, mode, scratch, slot_words, lengths, s);
  }
}

cudaError_t decode_mode_launch(int type, int dims, const uint64_t* in, uint64_t nwords,
                               const unsigned long long* offsets, const gzfp::Geom& g,
                               const gzfp::General& mode, void* out, cudaStream_t s) {
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return gzfp::launch_decode_mode<float>(dims, in, nwords, offsets, g, mode, (float*)out, s);
    case GZFP_TYPE_DOUBLE:
      return gzfp::launch_decode_mode<double>(dims, in, nwords, offsets, g, mode, (double*)out, s);
    case GZFP_TYPE_INT32:
      return gzfp::launch_decode_mode<int32_t>(dims, in, nwords, offsets, g, mode, (int32_t*)out, s);
    default:
      return gzfp::launch_decode_mode<int64_t>(dims, in, nwords, offsets, g, mode, (int64_t*)out, s);
  }
}

cudaError_t index_launch(int type, int dims, const uint64_t* in, uint64_t nwords, uint64_t nblocks,
                         const gzfp::General& mode, uint64_t first, unsigned long long* offsets,
                         unsigned long long* end, cudaStream_t s) {
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return gzfp::launch_index_blocks<float>(dims, in, nwords, nblocks, mode, first, offsets, end, s);
    case GZFP_TYPE_DOUBLE:
      return gzfp::launch_index_blocks<double>(dims, in, nwords, nblocks, mode, first, offsets, end, s);
    case GZFP_TYPE_INT32:
      return gzfp::launch_index_blocks<int32_t>(dims, in, nwords, nblocks, mode, first, offsets, end, s);
    default:
      return gzfp::launch_index_blocks<int64_t>(dims, in, nwords, nblocks, mode, first, offsets, end, s);
  }
}

// Walk the blocks of a device stream into ms.offsets; *end_bit = the bit
// after the last block.  Synchronises `s`.
int walk_blocks(ModeSpace& ms, int type, int dims, const uint64_t* words, uint64_t nwords,
                const gzfp::Geom& g, const gzfp::General& mode, uint64_t first, uint64_t& end_bit,
                cudaStream_t s) {
  cudaError_t e;
  if ((e = reserve(ms.offsets, ms.offsets_cap, (size_t)g.nblocks * 8)) ||
      (e = reserve(ms.sums, ms.sums_cap, 64)))
    return cuda_fail(e, "cudaMalloc(block offsets)");
  if ((e = index_launch(type, dims, words, nwords, g.nblocks, mode, first,
                        (unsigned long long*)ms.offsets, (unsigned long long*)ms.sums, s)))
    return cuda_fail(e, "block walk launch");
  unsigned long long end = 0;
  if ((e = cudaMemcpyAsync(&end, ms.sums, 8, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "block walk");
  end_bit = end;
  return GZFP_OK;
}

}  // namespace

extern "C" {

int gzfp_mode_rate(int type, unsigned dims, double rate, gzfp_mode* mode) {
  clear_error();
  if (!mode) return fail(GZFP_ERR_ARG, "null mode");
  const unsigned b = gzfp_rate_to_maxbits(type, dims, rate);
  if (!b) return fail(GZFP_ERR_ARG, "bad type, dimensionality or rate");
  *mode = gzfp_mode{b, b, precision_bits(type), -1074};
  return GZFP_OK;
}

int gzfp_mode_precision(int type, unsigned precision, gzfp_mode* mode) {
  clear_error();
  if (!mode) return fail(GZFP_ERR_ARG, "null mode");
  if (!known_type(type)) return fail(GZFP_ERR_ARG, "unknown scalar type");
  const unsigned P = precision_bits(type);
  *mode = gzfp_mode{0, 4171, precision ? (precision < P ? precision : P) : P, -1074};
  return GZFP_OK;
}

int gzfp_mode_accuracy(int type, double tolerance, gzfp_mode* mode) {
  clear_error();
  if (!mode) return fail(GZFP_ERR_ARG, "null mode");
  if (!known_type(type)) return fail(GZFP_ERR_ARG, "unknown scalar type");
  if (isnan(tolerance)) return fail(GZFP_ERR_ARG, "tolerance is NaN");
  int emin = -1074;
  if (tolerance > 0) {
    frexp(tolerance, &emin);  // tolerance = x * 2^emin with 0.5 <= x < 1
    emin--;
  }
  *mode = gzfp_mode{0, 4171, precision_bits(type), emin};
  return GZFP_OK;
}

size_t gzfp_mode_maximum_size(int type, unsigned nx, unsigned ny, unsigned nz,
                              const gzfp_mode* mode) {
  gzfp::Geom g;
  int dims;
  if (check_mode(type, nx, ny, nz, mode, g, dims)) return 0;
  return (size_t)((g.nblocks * mode_block_bound(type, dims, mode) + 63) / 64 * 8);
}

}  // extern "C"

namespace {

// A general-mode compression; with `header` (hbits bits in whole words)
// the stream starts with it and the blocks follow directly.
int compress_mode_impl(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                       const void* data, void* stream, size_t capacity, size_t* out_bytes,
                       unsigned long long* offsets, void* cuda_stream, const uint64_t* header,
                       unsigned hbits) {
  gzfp::Geom g;
  int dims;
  int st = check_mode(type, nx, ny, nz, mode, g, dims);
  if (st) return st;
  if (!data || !stream) return fail(GZFP_ERR_ARG, "null pointer");
  cudaStream_t s = (cudaStream_t)cuda_stream;
  cudaError_t e;
  if (fixed_rate_mode(type, mode)) {
    st = header ? strided_call(false, type, nx, ny, nz, 0, 0, 0, mode->maxbits, (void*)data,
                               (uint64_t*)stream, capacity, out_bytes, cuda_stream, hbits, header,
                               (hbits + 63) / 64)
                : gzfp_compress_bits(type, nx, ny, nz, mode->maxbits, data, stream, capacity,
                                     out_bytes, cuda_stream);
    if (st || !offsets) return st;
    if (is_device_pointer(offsets)) {
      if ((e = gzfp::launch_fixed_offsets(offsets, g.nblocks, hbits, mode->maxbits, s)))
        return cuda_fail(e, "offsets kernel launch");
    } else {
      for (uint64_t b = 0; b < g.nblocks; b++) offsets[b] = hbits + b * mode->maxbits;
    }
    return GZFP_OK;
  }
  if (out_bytes) *out_bytes = 0;
  if (g.nblocks == 0) return GZFP_OK;
  ModeSpace* msp;
  if ((st = mode_space(msp))) return st;
  ModeSpace& ms = *msp;
  std::lock_guard<std::mutex> lock(ms.mu);
  const size_t S = scalar_size(type);
  const gzfp::General gm = general_of(mode);
  const uint32_t slot_words = (mode_block_bound(type, dims, mode) + 63) / 64;
  const uint64_t m = gzfp::scan_sums_count(g.nblocks);
  const bool dev_data = is_device_pointer(data), dev_stream = is_device_pointer(stream);
  const bool dev_offsets = offsets && is_device_pointer(offsets);
  // one slot of slack after the last: a slot holds the most bits any block
  // can take, and the slack keeps even a longer block inside the buffer
  if ((e = reserve(ms.scratch, ms.scratch_cap, (size_t)((g.nblocks + 1) * slot_words * 8))) ||
      (e = reserve(ms.lengths, ms.lengths_cap, (size_t)g.nblocks * 4)) ||
      (e = reserve(ms.offsets, ms.offsets_cap, (size_t)g.nblocks * 8)) ||
      (e = reserve(ms.sums, ms.sums_cap, (size_t)(m + 1) * 8)))
    return cuda_fail(e, "cudaMalloc(general-mode scratch)");
  const void* din = data;
  const size_t field_bytes = (size_t)g.nx * g.ny * g.nz * S;
  if (!dev_data) {
    if ((e = reserve(ms.field, ms.field_cap, field_bytes)))
      return cuda_fail(e, "cudaMalloc(field staging)");
    if ((e = cudaMemcpyAsync(ms.field, data, field_bytes, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "cudaMemcpyAsync(field H2D)");
    din = ms.field;
  }
  gzfp::Geom gv = g;
  gv.vec = rows_vectorizable(din, nx, type);
  if ((e = encode_mode_launch(type, dims, din, gv, gm, (uint64_t*)ms.scratch, slot_words,
                              (uint32_t*)ms.lengths, s)))
    return cuda_fail(e, "encode kernel launch");
  if ((e = gzfp::launch_scan_lengths((const uint32_t*)ms.lengths, g.nblocks, hbits,
                                     (uint64_t*)ms.sums, (unsigned long long*)ms.offsets, s)))
    return cuda_fail(e, "scan kernel launch");
  unsigned long long total = 0;
  if ((e = cudaMemcpyAsync(&total, (uint64_t*)ms.sums + m, 8, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "encode");
  const size_t bytes = (size_t)((hbits + total + 63) / 64 * 8);
  if (out_bytes) *out_bytes = bytes;
  if (capacity < bytes) return fail(GZFP_ERR_CAPACITY, "stream buffer smaller than the compressed size");
  uint64_t* dstream = (uint64_t*)stream;
  if (!dev_stream) {
    if ((e = reserve(ms.stream, ms.stream_cap, bytes))) return cuda_fail(e, "cudaMalloc(stream staging)");
    dstream = (uint64_t*)ms.stream;
  }
  st = GZFP_OK;
  if ((e = cudaMemsetAsync(dstream, 0, bytes, s)) ||
      (header && (e = cudaMemcpyAsync(dstream, header, (hbits + 63) / 64 * 8,
                                      cudaMemcpyHostToDevice, s))) ||
      (e = gzfp::launch_place_blocks((const uint64_t*)ms.scratch, slot_words,
                                     (const uint32_t*)ms.lengths,
                                     (const unsigned long long*)ms.offsets, g.nblocks, dstream, s)))
    st = cuda_fail(e, "block placement");
  if (!st && !dev_stream && (e = cudaMemcpyAsync(stream, dstream, bytes, cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(stream D2H)");
  if (!st && offsets &&
      (e = cudaMemcpyAsync(offsets, ms.offsets, (size_t)g.nblocks * 8,
                           dev_offsets ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(offsets)");
  const cudaError_t es = cudaStreamSynchronize(s);  // the scratch is reused by the next call
  if (!st && es) st = cuda_fail(es, "cudaStreamSynchronize");
  return st;
}

// A general-mode decompression whose first block starts at bit `first`.
int decompress_mode_impl(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                         const void* stream, size_t bytes, const unsigned long long* offsets,
                         void* data, void* cuda_stream, uint64_t first) {
  gzfp::Geom g;
  int dims;
  int st = check_mode(type, nx, ny, nz, mode, g, dims);
  if (st) return st;
  if (!stream || !data) return fail(GZFP_ERR_ARG, "null pointer");
  if (fixed_rate_mode(type, mode))
    return first ? strided_call(true, type, nx, ny, nz, 0, 0, 0, mode->maxbits, data,
                                (uint64_t*)stream, bytes, nullptr, cuda_stream, first)
                 : gzfp_decompress_bits(type, nx, ny, nz, mode->maxbits, stream, bytes, data,
                                        cuda_stream);
  if (g.nblocks == 0) return GZFP_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  ModeSpace* msp;
  if ((st = mode_space(msp))) return st;
  ModeSpace& ms = *msp;
  std::lock_guard<std::mutex> lock(ms.mu);
  cudaError_t e;
  const uint64_t nwords = bytes / 8;
  const gzfp::General gm = general_of(mode);
  const size_t field_bytes = (size_t)g.nx * g.ny * g.nz * scalar_size(type);
  const bool dev_stream = is_device_pointer(stream), dev_data = is_device_pointer(data);
  bool staged = !dev_stream || !dev_data;
  const uint64_t* dw = (const uint64_t*)stream;
  if (!dev_stream) {
    if ((e = reserve(ms.stream, ms.stream_cap, nwords ? nwords * 8 : 8)) ||
        (e = cudaMemcpyAsync(ms.stream, stream, nwords * 8, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "stream staging");
    dw = (const uint64_t*)ms.stream;
  }
  const unsigned long long* doff = offsets;
  if (!offsets) {
    uint64_t end = 0;
    if ((st = walk_blocks(ms, type, dims, dw, nwords, g, gm, first, end, s))) return st;
    if (end > nwords * 64) return fail(GZFP_ERR_ARG, "stream shorter than its blocks");
    doff = (const unsigned long long*)ms.offsets;
  } else if (!is_device_pointer(offsets)) {
    if ((e = reserve(ms.offsets, ms.offsets_cap, (size_t)g.nblocks * 8)) ||
        (e = cudaMemcpyAsync(ms.offsets, offsets, (size_t)g.nblocks * 8, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "offsets staging");
    doff = (const unsigned long long*)ms.offsets;
    staged = true;
  }
  void* dout = data;
  if (!dev_data) {
    if ((e = reserve(ms.field, ms.field_cap, field_bytes))) return cuda_fail(e, "cudaMalloc(field staging)");
    dout = ms.field;
  }
  gzfp::Geom gv = g;
  gv.vec = rows_vectorizable(dout, nx, type);
  st = GZFP_OK;
  if ((e = decode_mode_launch(type, dims, dw, nwords, doff, gv, gm, dout, s)))
    st = cuda_fail(e, "decode kernel launch");
  if (!st && !dev_data && (e = cudaMemcpyAsync(data, dout, field_bytes, cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(field D2H)");
  if (staged || !offsets) {  // staging buffers and the walk's offsets are reused by the next call
    const cudaError_t es = cudaStreamSynchronize(s);
    if (!st && es) st = cuda_fail(es, "cudaStreamSynchronize");
  }
  return st;
}

}  // namespace

extern "C" {

int gzfp_compress_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                       const void* data, void* stream, size_t capacity, size_t* out_bytes,
                       unsigned long long* offsets, void* cuda_stream) {
  clear_error();
  return compress_mode_impl(type, nx, ny, nz, mode, data, stream, capacity, out_bytes, offsets,
                            cuda_stream, nullptr, 0);
}

int gzfp_decompress_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                         const void* stream, size_t bytes, const unsigned long long* offsets,
                         void* data, void* cuda_stream) {
  clear_error();
  return decompress_mode_impl(type, nx, ny, nz, mode, stream, bytes, offsets, data, cuda_stream,
                              0);
}

int gzfp_index_blocks(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                      const void* stream, size_t bytes, unsigned long long* offsets,
                      void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  int st = check_mode(type, nx, ny, nz, mode, g, dims);
  if (st) return st;
  if (!stream || !offsets) return fail(GZFP_ERR_ARG, "null pointer");
  if (g.nblocks == 0) return GZFP_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  ModeSpace* msp;
  if ((st = mode_space(msp))) return st;
  ModeSpace& ms = *msp;
  std::lock_guard<std::mutex> lock(ms.mu);
  cudaError_t e;
  const uint64_t nwords = bytes / 8;
  const uint64_t* dw = (const uint64_t*)stream;
  if (!is_device_pointer(stream)) {
    if ((e = reserve(ms.stream, ms.stream_cap, nwords ? nwords * 8 : 8)) ||
        (e = cudaMemcpyAsync(ms.stream, stream, nwords * 8, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "stream staging");
    dw = (const uint64_t*)ms.stream;
  }
  uint64_t end = 0;
  if ((st = walk_blocks(ms, type, dims, dw, nwords, g, general_of(mode), 0, end, s))) return st;
  if (end > nwords * 64) return fail(GZFP_ERR_ARG, "stream shorter than its blocks");
  if ((e = cudaMemcpyAsync(offsets, ms.offsets, (size_t)g.nblocks * 8,
                           is_device_pointer(offsets) ? cudaMemcpyDeviceToDevice
                                                      : cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "cudaMemcpyAsync(offsets)");
  return GZFP_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ headers
// zfp 0.5.0's full header (zfp_write_header / zfp_read_header with
// ZFP_HEADER_FULL, Z/src/zfp.c:661-719): a 32-bit magic, 52 bits of field
// metadata (zfp_field_metadata / zfp_field_set_metadata, :158-182 and
// :254-275) and the stream parameters in 12 or 64 bits (zfp_stream_mode /
// zfp_stream_set_mode, :305-345 and :461-498).
namespace {

constexpr unsigned kMagicBits = 32, kMetaBits = 52, kModeShortBits = 12, kModeLongBits = 64;
constexpr uint64_t kModeShortMax = (1u << kModeShortBits) - 2;  // ZFP_MODE_SHORT_MAX
constexpr int kMinExp = -1074;                                    // ZFP_MIN_EXP
constexpr unsigned kMaxBitsZfp = 4171;                            // ZFP_MAX_BITS
constexpr int kMinExpBias = 16495;  // minexp offset of the long mode form
constexpr unsigned kLongField = 0x8000;  // largest minbits / maxbits the long form records

// up to 192 bits, LSB first in 64-bit words (the stream's own layout)
struct HeaderWords {
  uint64_t w[3] = {0, 0, 0};
  unsigned n = 0;
  void put(uint64_t v, unsigned bits) {  // bits <= 64
    if (bits < 64) v &= (1ull << bits) - 1;
    const unsigned i = n >> 6, o = n & 63;
    w[i] |= v << o;
    if (o && o + bits > 64) w[i + 1] |= v >> (64 - o);
    n += bits;
  }
  uint64_t get(unsigned& pos, unsigned bits) const {  // bits <= 64
    const unsigned i = pos >> 6, o = pos & 63;
    uint64_t v = w[i] >> o;
    if (o && o + bits > 64) v |= w[i + 1] << (64 - o);
    pos += bits;
    return bits < 64 ? v & ((1ull << bits) - 1) : v;
  }
};

// Field sizes a header records: 48 bits of nx - 1 in 1D, 24 bits per axis
// in 2D, 16 bits per axis in 3D (zfp_field_metadata, Z/src/zfp.c:158-182).
bool header_sizes_fit(int dims, unsigned nx, unsigned ny, unsigned nz) {
  if (dims == 2) return nx <= (1u << 24) && ny <= (1u << 24);
  if (dims == 3) return nx <= (1u << 16) && ny <= (1u << 16) && nz <= (1u << 16);
  return true;
}

// zfp_stream_mode: the 12-bit forms for fixed rate (maxbits - 1), fixed
// precision (maxprec + 2047) and fixed accuracy (minexp + 3251), else the
// 64-bit form holding every parameter.
uint64_t mode_code(const gzfp_mode& m, unsigned& bits) {
  bits = kModeShortBits;
  if (m.minbits == m.maxbits && m.maxbits >= 1 && m.maxbits <= 2048 && m.maxprec >= 64 &&
      m.minexp <= kMinExp)
    return m.maxbits - 1;
  if (m.minbits == 0 && m.maxbits >= kMaxBitsZfp && m.maxprec >= 1 && m.maxprec <= 128 &&
      m.minexp <= kMinExp)
    return m.maxprec + 2047;
  if (m.minbits == 0 && m.maxbits >= kMaxBitsZfp && m.maxprec >= 64 && m.minexp >= kMinExp &&
      m.minexp <= 843)
    return (uint64_t)(m.minexp + 3251);
  bits = kModeLongBits;
  auto clamp1 = [](unsigned v, unsigned hi) { return (v < 1 ? 1 : v > hi ? hi : v) - 1; };
  const int e = m.minexp + kMinExpBias;
  uint64_t code = (uint64_t)(e < 0 ? 0 : e > 0x7fff ? 0x7fff : e);
  code = (code << 7) | clamp1(m.maxprec, 0x80);
  code = (code << 15) | clamp1(m.maxbits, kLongField);
  code = (code << 15) | clamp1(m.minbits, kLongField);
  return (code << 12) | 0xfff;
}

int build_header_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode& m,
                      HeaderWords& h) {
  gzfp::Geom g;
  int dims;
  int st = check_mode(type, nx, ny, nz, &m, g, dims);
  if (st) return st;
  if (!header_sizes_fit(dims, nx, ny, nz))
    return fail(GZFP_ERR_ARG, "field sizes beyond what a zfp header records");
  unsigned mbits;
  const uint64_t code = mode_code(m, mbits);
  // the long form clamps: refuse parameters it would record differently
  if (mbits == kModeLongBits &&
      (m.minbits > kLongField || m.maxbits > kLongField || m.minexp + kMinExpBias < 0 ||
       m.minexp + kMinExpBias > 0x7fff))
    return fail(GZFP_ERR_ARG, "parameters beyond what a zfp header records");
  h.put('z', 8);
  h.put('f', 8);
  h.put('p', 8);
  h.put(5, 8);  // ZFP_VERSION >> 4 for 0.5.0
  uint64_t meta = dims == 1   ? (uint64_t)(nx - 1)
                  : dims == 2 ? ((uint64_t)(ny - 1) << 24) | (nx - 1)
                              : ((((uint64_t)(nz - 1) << 16) | (ny - 1)) << 16) | (nx - 1);
  meta = (meta << 4) | ((uint64_t)(dims - 1) << 2) | (uint64_t)(type - 1);
  h.put(meta, kMetaBits);
  h.put(code, mbits);
  return GZFP_OK;
}

// Parse a header into the field and the stream parameters
// (zfp_stream_set_mode); checks that the parameters can code a stream.
int parse_header_mode(const HeaderWords& h, size_t avail_bits, int* type, unsigned* nx,
                      unsigned* ny, unsigned* nz, gzfp_mode* m, size_t* header_bits) {
  if (avail_bits < kMagicBits + kMetaBits + kModeShortBits)
    return fail(GZFP_ERR_ARG, "stream shorter than a zfp header");
  unsigned pos = 0;
  if (h.get(pos, 8) != 'z' || h.get(pos, 8) != 'f' || h.get(pos, 8) != 'p' || h.get(pos, 8) != 5)
    return fail(GZFP_ERR_ARG, "no zfp 0.5.0 header (magic mismatch)");
  uint64_t meta = h.get(pos, kMetaBits);
  const int t = (int)(meta & 3) + 1;
  const int dims = (int)((meta >> 2) & 3) + 1;
  meta >>= 4;
  unsigned x, y = 0, z = 0;
  if (dims == 1) {
    const uint64_t n = (meta & 0xffffffffffffull) + 1;
    if (n > 0xffffffffull) return fail(GZFP_ERR_UNSUPPORTED, "1D field of 2^32 values or more");
    x = (unsigned)n;
  } else if (dims == 2) {
    x = (unsigned)(meta & 0xffffff) + 1;
    y = (unsigned)((meta >> 24) & 0xffffff) + 1;
  } else if (dims == 3) {
    x = (unsigned)(meta & 0xffff) + 1;
    y = (unsigned)((meta >> 16) & 0xffff) + 1;
    z = (unsigned)((meta >> 32) & 0xffff) + 1;
  } else {
    return fail(GZFP_ERR_UNSUPPORTED, "4D field (not part of zfp 0.5.0)");
  }
  uint64_t code = h.get(pos, kModeShortBits);
  gzfp_mode md;
  if (code <= kModeShortMax) {
    if (code < 2048)
      md = gzfp_mode{(unsigned)code + 1, (unsigned)code + 1, 64, kMinExp};
    else if (code < 2176)
      md = gzfp_mode{0, kMaxBitsZfp, (unsigned)code - 2047, kMinExp};
    else
      md = gzfp_mode{0, kMaxBitsZfp, 64, (int)code - 3251};
  } else {
    if (avail_bits < kMagicBits + kMetaBits + kModeLongBits)
      return fail(GZFP_ERR_ARG, "stream shorter than a zfp header");
    code |= h.get(pos, kModeLongBits - kModeShortBits) << kModeShortBits;
    md.minbits = (unsigned)((code >> 12) & 0x7fff) + 1;
    md.maxbits = (unsigned)((code >> 27) & 0x7fff) + 1;
    md.maxprec = (unsigned)((code >> 42) & 0x7f) + 1;
    md.minexp = (int)((code >> 49) & 0x7fff) - kMinExpBias;
  }
  gzfp::Geom g;
  int d;
  if (check_mode(t, x, y, z, &md, g, d))
    return fail(GZFP_ERR_UNSUPPORTED, "header parameters this codec cannot decode");
  *type = t;
  *nx = x;
  *ny = y;
  *nz = z;
  *m = md;
  *header_bits = pos;
  return GZFP_OK;
}

// the header at the start of a host or device stream (for a device stream:
// a copy of its first words after the work queued on `s`)
int stream_header(const void* stream, size_t bytes, cudaStream_t s, HeaderWords& h) {
  const size_t hb = bytes < sizeof h.w ? bytes : sizeof h.w;
  if (is_device_pointer(stream)) {
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h.w, stream, hb, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_fail(e, "cudaMemcpyAsync(header D2H)");
  } else {
    memcpy(h.w, stream, hb);
  }
  return GZFP_OK;
}

}  // namespace

extern "C" {

int gzfp_write_header_mode(int type, unsigned nx, unsigned ny, unsigned nz,
                           const gzfp_mode* mode, void* header, size_t capacity,
                           size_t* header_bits) {
  clear_error();
  if (!mode || !header) return fail(GZFP_ERR_ARG, "null pointer");
  HeaderWords h;
  int st = build_header_mode(type, nx, ny, nz, *mode, h);
  if (st) return st;
  const size_t bytes = (h.n + 7) / 8;
  if (capacity < bytes) return fail(GZFP_ERR_CAPACITY, "header buffer too small");
  memcpy(header, h.w, bytes);
  if (header_bits) *header_bits = h.n;
  return GZFP_OK;
}

int gzfp_write_header(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                      void* header, size_t capacity, size_t* header_bits) {
  clear_error();
  // the parameters zfp_stream_set_rate leaves
  const gzfp_mode m{maxbits, maxbits, precision_bits(type), kMinExp};
  return gzfp_write_header_mode(type, nx, ny, nz, &m, header, capacity, header_bits);
}

int gzfp_read_header_mode(const void* header, size_t bytes, int* type, unsigned* nx,
                          unsigned* ny, unsigned* nz, gzfp_mode* mode, size_t* header_bits) {
  clear_error();
  if (!header || !type || !nx || !ny || !nz || !mode || !header_bits)
    return fail(GZFP_ERR_ARG, "null pointer");
  HeaderWords h;
  memcpy(h.w, header, bytes < sizeof h.w ? bytes : sizeof h.w);
  return parse_header_mode(h, bytes * 8, type, nx, ny, nz, mode, header_bits);
}

int gzfp_read_header(const void* header, size_t bytes, int* type, unsigned* nx, unsigned* ny,
                     unsigned* nz, unsigned* maxbits, size_t* header_bits) {
  gzfp_mode m;
  int st = gzfp_read_header_mode(header, bytes, type, nx, ny, nz, &m, header_bits);
  if (st) return st;
  if (!maxbits) return fail(GZFP_ERR_ARG, "null pointer");
  if (!fixed_rate_mode(*type, &m))
    return fail(GZFP_ERR_UNSUPPORTED, "stream in a mode other than fixed rate (see gzfp_read_header_mode)");
  *maxbits = m.maxbits;
  return GZFP_OK;
}

int gzfp_compress_headed(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                         const void* data, void* stream, size_t capacity, size_t* out_bytes,
                         void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  if (!make_geom(nx, ny, nz, g, dims)) return fail(GZFP_ERR_ARG, "bad dimensions");
  gzfp_mode m;
  int st = gzfp_mode_rate(type, (unsigned)dims, rate, &m);
  if (st) return st;
  return gzfp_compress_mode_headed(type, nx, ny, nz, &m, data, stream, capacity, out_bytes,
                                   nullptr, cuda_stream);
}

int gzfp_compress_mode_headed(int type, unsigned nx, unsigned ny, unsigned nz,
                              const gzfp_mode* mode, const void* data, void* stream,
                              size_t capacity, size_t* out_bytes, unsigned long long* offsets,
                              void* cuda_stream) {
  clear_error();
  if (!mode) return fail(GZFP_ERR_ARG, "null mode");
  HeaderWords h;
  int st = build_header_mode(type, nx, ny, nz, *mode, h);
  if (st) return st;
  return compress_mode_impl(type, nx, ny, nz, mode, data, stream, capacity, out_bytes, offsets,
                            cuda_stream, h.w, h.n);
}

int gzfp_decompress_headed(const void* stream, size_t bytes, void* data, size_t data_bytes,
                           void* cuda_stream) {
  clear_error();
  if (!stream || !data) return fail(GZFP_ERR_ARG, "null pointer");
  HeaderWords h;
  int st = stream_header(stream, bytes, (cudaStream_t)cuda_stream, h);
  if (st) return st;
  int type;
  unsigned nx, ny, nz;
  gzfp_mode m;
  size_t header_bits;
  if ((st = parse_header_mode(h, bytes * 8, &type, &nx, &ny, &nz, &m, &header_bits))) return st;
  const uint64_t values = (uint64_t)nx * (ny ? ny : 1) * (nz ? nz : 1);
  if (data_bytes < values * scalar_size(type))
    return fail(GZFP_ERR_CAPACITY, "output buffer smaller than the field in the header");
  return decompress_mode_impl(type, nx, ny, nz, &m, stream, bytes, nullptr, data, cuda_stream,
                              header_bits);
}

}  // extern "C"
