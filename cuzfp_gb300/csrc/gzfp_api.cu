// gzfp_api.cu -- host side of the C ABI declared in include/gzfp.h: the
// fixed-rate calls, host staging and strided fields.  (Block access, the
// general modes and stream headers are in gzfp_access_api.cu,
// gzfp_modes_api.cu and gzfp_header_api.cu, sharing gzfp_host.h.)
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
#include "gzfp_host.h"
#include "gzfp_launch.h"
#include "gzfp_slabs.h"

namespace gzfp_host {

thread_local char g_last_error[kErrorLen];

void clear_error() { g_last_error[0] = 0; }

int fail(int status, const char* msg) {
  snprintf(g_last_error, sizeof g_last_error, "%s", msg);
  return status;
}

int cuda_fail(cudaError_t e, const char* what) {
  snprintf(g_last_error, sizeof g_last_error, "%s: %s", what, cudaGetErrorString(e));
  return GZFP_ERR_CUDA;
}


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

// The device address of host memory that the kernels may read and write in
// place, else null: memory pinned or registered with CUDA, on a device whose
// host link is hardware-coherent (it uses the host's page tables, as a
// Grace-Blackwell part's chip-to-chip link does).  There the kernels reach
// the link's bandwidth (measured on GB300: 211 GB/s host to device and 193
// GB/s back, the copy engines' figures), so no slab pipeline is needed.
void* direct_host_alias(const void* p) {
  int dev = 0, coherent = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coherent, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
          cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (!coherent) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
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

}  // namespace gzfp_host

using namespace gzfp_host;

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
  cudaError_t e;
  if (!dev_data || !dev_stream) {
    // pinned host memory on a coherent link: the kernel codes it in place
    // (blocks of whole words only: shared words are merged with atomics,
    // which stay in device memory); the call returns when it is done
    const void* hd = dev_data ? data : direct_host_alias(data);
    void* hs = dev_stream ? stream : direct_host_alias(stream);
    if (hd && hs && maxbits % 64 == 0) {
      g.vec = rows_vectorizable(hd, nx, type);
      if ((e = encode_launch(type, dims, hd, g, maxbits, (uint64_t*)hs, nwords, s)))
        return cuda_fail(e, "encode kernel launch");
      if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "encode kernel");
      return GZFP_OK;
    }
    return staged(false, type, dims, g, maxbits, (void*)data, dev_data, (uint64_t*)stream,
                  dev_stream, s);
  }
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
  cudaError_t e;
  if (!dev_data || !dev_stream) {
    // pinned host memory on a coherent link: decoded in place (see above)
    void* hd = dev_data ? data : direct_host_alias(data);
    const void* hs = dev_stream ? stream : direct_host_alias(stream);
    if (hd && hs) {
      g.vec = rows_vectorizable(hd, nx, type);
      if ((e = decode_launch(type, dims, (const uint64_t*)hs, nwords, g, maxbits, hd, s)))
        return cuda_fail(e, "decode kernel launch");
      if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "decode kernel");
      return GZFP_OK;
    }
    return staged(true, type, dims, g, maxbits, data, dev_data, (uint64_t*)stream, dev_stream, s);
  }
  g.vec = rows_vectorizable(data, nx, type);
  e = decode_launch(type, dims, (const uint64_t*)stream, nwords, g, maxbits, data, s);
  if (e) return cuda_fail(e, "decode kernel launch");
  return GZFP_OK;
}

}  // extern "C"

namespace gzfp_host {

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
                 size_t words_bytes, size_t* out_bytes, void* cuda_stream, uint64_t base,
                 const uint64_t* header, unsigned header_words) {
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

}  // namespace gzfp_host

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

