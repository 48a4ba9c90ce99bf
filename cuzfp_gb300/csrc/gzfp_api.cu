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

int ebits_of(int type) { return type == GZFP_TYPE_FLOAT ? 8 : 11; }

// Field geometry; ny = 0 selects 1D, nz = 0 selects 2D (zfp_field_1d/2d/3d).
bool make_geom(unsigned nx, unsigned ny, unsigned nz, gzfp::Geom& g, int& dims) {
  if (nx == 0 || (nz != 0 && ny == 0)) return false;
  dims = nz ? 3 : ny ? 2 : 1;
  g = gzfp::make_geom_blocks(nx, ny ? ny : 1, nz ? nz : 1);
  return g.nblocks < (1ull << 32);  // block indices are 32-bit on the device
}

// Rows of full blocks move as one vector when every row start is aligned:
// 16 bytes for float, 32 for double.
uint32_t rows_vectorizable(const void* p, unsigned nx, int type) {
  const uintptr_t a = type == GZFP_TYPE_FLOAT ? 16 : 32;
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

// Device buffers used to stage host arrays and streams, one set per device,
// grown on demand and kept for the life of the process.
struct Workspace {
  std::mutex mu;
  void* field = nullptr;
  size_t field_cap = 0;
  void* stream = nullptr;
  size_t stream_cap = 0;
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

int check_common(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                 gzfp::Geom& g, int& dims) {
  if (type == GZFP_TYPE_INT32 || type == GZFP_TYPE_INT64)
    return fail(GZFP_ERR_UNSUPPORTED, "integer fields are not supported by this path");
  if (type != GZFP_TYPE_FLOAT && type != GZFP_TYPE_DOUBLE)
    return fail(GZFP_ERR_ARG, "unknown scalar type");
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
  if ((type != GZFP_TYPE_FLOAT && type != GZFP_TYPE_DOUBLE) || dims < 1 || dims > 3) return 0;
  if (!(rate >= 0) || rate > 1e6) return 0;
  unsigned n = 1u << (2 * dims);
  unsigned bits = (unsigned)floor(n * rate + 0.5);
  unsigned lo = 1u + (unsigned)ebits_of(type);
  return bits < lo ? lo : bits;
}

size_t gzfp_stream_size(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits) {
  gzfp::Geom g;
  int dims;
  if ((type != GZFP_TYPE_FLOAT && type != GZFP_TYPE_DOUBLE) || !make_geom(nx, ny, nz, g, dims))
    return 0;
  return (size_t)(stream_words(g, maxbits) * 8);
}

size_t gzfp_maximum_size(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits) {
  gzfp::Geom g;
  int dims;
  if ((type != GZFP_TYPE_FLOAT && type != GZFP_TYPE_DOUBLE) || !make_geom(nx, ny, nz, g, dims))
    return 0;
  // zfp_stream_maximum_size: min(maxbits, bits of a block coded in full),
  // raised to minbits -- which equals maxbits in fixed-rate mode -- plus the
  // 148 header bits, rounded up to a 64-bit word
  (void)dims;
  const uint64_t b = maxbits;
  return (size_t)(((148 + g.nblocks * b + 63) & ~63ull) / 8);
}

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
  const size_t field_bytes =
      (size_t)g.nx * g.ny * g.nz * (type == GZFP_TYPE_FLOAT ? sizeof(float) : sizeof(double));

  const bool dev_data = is_device_pointer(data);
  const bool dev_stream = is_device_pointer(stream);
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (device < 0 || device >= kMaxDevices) return fail(GZFP_ERR_CUDA, "device index out of range");
  Workspace& ws = g_ws[device];
  std::unique_lock<std::mutex> lock(ws.mu, std::defer_lock);
  if (!dev_data || !dev_stream) lock.lock();

  const void* d_data = data;
  uint64_t* d_stream = (uint64_t*)stream;
  if (!dev_data) {
    if ((e = reserve(ws.field, ws.field_cap, field_bytes))) return cuda_fail(e, "cudaMalloc(field workspace)");
    if ((e = cudaMemcpyAsync(ws.field, data, field_bytes, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "cudaMemcpyAsync(field H2D)");
    d_data = ws.field;
  }
  if (!dev_stream) {
    if ((e = reserve(ws.stream, ws.stream_cap, bytes))) return cuda_fail(e, "cudaMalloc(stream workspace)");
    d_stream = (uint64_t*)ws.stream;
  }
  if (maxbits % 64 != 0) {
    // blocks share boundary words, which the kernel ORs into a zeroed stream
    if ((e = cudaMemsetAsync(d_stream, 0, bytes, s))) return cuda_fail(e, "cudaMemsetAsync(stream)");
  }
  g.vec = rows_vectorizable(d_data, nx, type);
  if (type == GZFP_TYPE_FLOAT)
    e = gzfp::launch_encode_f32(dims, (const float*)d_data, g, maxbits, d_stream, nwords, s);
  else
    e = gzfp::launch_encode_f64(dims, (const double*)d_data, g, maxbits, d_stream, nwords, s);
  if (e) return cuda_fail(e, "encode kernel launch");
  if (!dev_stream) {
    if ((e = cudaMemcpyAsync(stream, d_stream, bytes, cudaMemcpyDeviceToHost, s)))
      return cuda_fail(e, "cudaMemcpyAsync(stream D2H)");
  }
  if (!dev_data || !dev_stream) {
    if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "cudaStreamSynchronize");
  }
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
  const size_t field_bytes =
      (size_t)g.nx * g.ny * g.nz * (type == GZFP_TYPE_FLOAT ? sizeof(float) : sizeof(double));

  const bool dev_data = is_device_pointer(data);
  const bool dev_stream = is_device_pointer(stream);
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (device < 0 || device >= kMaxDevices) return fail(GZFP_ERR_CUDA, "device index out of range");
  Workspace& ws = g_ws[device];
  std::unique_lock<std::mutex> lock(ws.mu, std::defer_lock);
  if (!dev_data || !dev_stream) lock.lock();

  const uint64_t* d_stream = (const uint64_t*)stream;
  void* d_data = data;
  if (!dev_stream) {
    if ((e = reserve(ws.stream, ws.stream_cap, need))) return cuda_fail(e, "cudaMalloc(stream workspace)");
    if ((e = cudaMemcpyAsync(ws.stream, stream, need, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "cudaMemcpyAsync(stream H2D)");
    d_stream = (const uint64_t*)ws.stream;
  }
  if (!dev_data) {
    if ((e = reserve(ws.field, ws.field_cap, field_bytes))) return cuda_fail(e, "cudaMalloc(field workspace)");
    d_data = ws.field;
  }
  g.vec = rows_vectorizable(d_data, nx, type);
  if (type == GZFP_TYPE_FLOAT)
    e = gzfp::launch_decode_f32(dims, d_stream, nwords, g, maxbits, (float*)d_data, s);
  else
    e = gzfp::launch_decode_f64(dims, d_stream, nwords, g, maxbits, (double*)d_data, s);
  if (e) return cuda_fail(e, "decode kernel launch");
  if (!dev_data) {
    if ((e = cudaMemcpyAsync(data, d_data, field_bytes, cudaMemcpyDeviceToHost, s)))
      return cuda_fail(e, "cudaMemcpyAsync(field D2H)");
  }
  if (!dev_data || !dev_stream) {
    if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "cudaStreamSynchronize");
  }
  return GZFP_OK;
}

int gzfp_compress(int type, unsigned nx, unsigned ny, unsigned nz, double rate, const void* data,
                  void* stream, size_t capacity, size_t* out_bytes, void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  if (!make_geom(nx, ny, nz, g, dims)) return fail(GZFP_ERR_ARG, "bad dimensions");
  if (type == GZFP_TYPE_INT32 || type == GZFP_TYPE_INT64)
    return fail(GZFP_ERR_UNSUPPORTED, "integer fields are not supported by this path");
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
  if (type == GZFP_TYPE_INT32 || type == GZFP_TYPE_INT64)
    return fail(GZFP_ERR_UNSUPPORTED, "integer fields are not supported by this path");
  unsigned maxbits = gzfp_rate_to_maxbits(type, (unsigned)dims, rate);
  if (!maxbits) return fail(GZFP_ERR_ARG, "bad type or rate");
  return gzfp_decompress_bits(type, nx, ny, nz, maxbits, stream, bytes, data, cuda_stream);
}

}  // extern "C"
