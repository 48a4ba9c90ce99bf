// gzfp_launch.h -- internal launcher interface between the host API
// (gzfp_api.cu) and the kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gzfp_array.cuh"

namespace gzfp {

// Launch the plain-path encoder / decoder for `dims` (1..3) on stream `s`.
cudaError_t launch_encode_f32(int dims, const float* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s);
cudaError_t launch_encode_f64(int dims, const double* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s);
cudaError_t launch_decode_f32(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, float* out, cudaStream_t s);
cudaError_t launch_decode_f64(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, double* out, cudaStream_t s);
cudaError_t launch_encode_i32(int dims, const int32_t* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s);
cudaError_t launch_encode_i64(int dims, const int64_t* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s);
cudaError_t launch_decode_i32(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, int32_t* out, cudaStream_t s);
cudaError_t launch_decode_i64(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, int64_t* out, cudaStream_t s);

// Random access to listed blocks, each coded from / into its own tile of
// 4^dims values (gzfp_blocks.cuh; instantiated for float, double, int32_t
// and int64_t in gzfp_blocks_*.cu).
template <typename T>
cudaError_t launch_encode_blocks(int dims, const T* tiles, const unsigned long long* index,
                                 const uint8_t* shape, uint64_t count, uint32_t maxbits,
                                 uint64_t* out, uint64_t nwords, cudaStream_t s);
template <typename T>
cudaError_t launch_decode_blocks(int dims, const uint64_t* in, uint64_t nwords,
                                 const unsigned long long* index, const uint8_t* shape,
                                 uint64_t count, uint32_t maxbits, T* tiles, cudaStream_t s);

}  // namespace gzfp
