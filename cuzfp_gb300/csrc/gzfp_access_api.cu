// gzfp_access_api.cu -- random access to single blocks (gzfp_decode_blocks /
// gzfp_encode_blocks, include/gzfp.h): argument checks, staging of host
// buffers and the launches of gzfp_blocks_*.cu.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "gzfp.h"
#include "gzfp_host.h"
#include "gzfp_launch.h"

using namespace gzfp_host;

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

