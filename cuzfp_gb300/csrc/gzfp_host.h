// gzfp_host.h -- internal interface between the host-side translation units
// of the C ABI (gzfp_api.cu: core calls, staging, strided fields;
// gzfp_access_api.cu: block access; gzfp_modes_api.cu: general modes;
// gzfp_header_api.cu: stream headers).  Not installed, not part of the ABI.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <mutex>

#include "gzfp.h"
#include "gzfp_array.cuh"

namespace gzfp_host {

// ---- errors: the detail of the calling thread's last failure
constexpr size_t kErrorLen = 512;
extern thread_local char g_last_error[kErrorLen];
void clear_error();
int fail(int status, const char* msg);            // records msg, returns status
int cuda_fail(cudaError_t e, const char* what);   // records the CUDA error, returns GZFP_ERR_CUDA

// ---- fields and arguments
constexpr unsigned kMaxBitsLimit = 1u << 20;  // largest bits per block taken
bool known_type(int type);
int ebits_of(int type);                       // block-header exponent bits (0 for integers)
size_t scalar_size(int type);
// geometry of nx x ny x nz (ny = 0: 1D, nz = 0: 2D), under 2^32 blocks
bool make_geom(unsigned nx, unsigned ny, unsigned nz, gzfp::Geom& g, int& dims);
uint32_t rows_vectorizable(const void* p, unsigned nx, int type);
bool is_device_pointer(const void* p);
int check_common(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                 gzfp::Geom& g, int& dims);
uint64_t stream_words(const gzfp::Geom& g, unsigned maxbits);

// ---- per-device staging workspace (host buffers)
constexpr int kSlots = 3;
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
extern Workspace g_ws[kMaxDevices];
cudaError_t reserve(void*& p, size_t& cap, size_t need);  // grow a device buffer

// ---- one call on a field with element strides (0 = contiguous), staged
// whole; `base` is the stream bit of block 0 and `header` the words written
// in front of it (headed streams)
int strided_call(bool decode, int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                 long long sy, long long sz, unsigned maxbits, void* field, uint64_t* words,
                 size_t words_bytes, size_t* out_bytes, void* cuda_stream, uint64_t base = 0,
                 const uint64_t* header = nullptr, unsigned header_words = 0);

// ---- general modes (gzfp_modes_api.cu)
unsigned precision_bits(int type);  // 32 or 64
int check_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* m,
               gzfp::Geom& g, int& dims);
bool fixed_rate_mode(int type, const gzfp_mode* m);  // the fixed-rate path's parameters
int compress_mode_impl(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                       const void* data, void* stream, size_t capacity, size_t* out_bytes,
                       unsigned long long* offsets, void* cuda_stream, const uint64_t* header,
                       unsigned hbits);
int decompress_mode_impl(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                         const void* stream, size_t bytes, const unsigned long long* offsets,
                         void* data, void* cuda_stream, uint64_t first);

}  // namespace gzfp_host
