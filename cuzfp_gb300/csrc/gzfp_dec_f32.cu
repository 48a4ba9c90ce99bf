// Decoder kernels for float fields (1D, 2D, 3D).
#include "gzfp_kernels.cuh"
#include "gzfp_launch.h"

namespace gzfp {

cudaError_t launch_decode_f32(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, float* out, cudaStream_t s) {
  if (g.nblocks == 0) return cudaSuccess;
  const dim3 grid((unsigned)((g.nblocks + kThreads - 1) / kThreads));
  switch (dims) {
    case 1: decode_kernel<1, float><<<grid, kThreads, 0, s>>>(in, nwords, g, maxbits, out); break;
    case 2: decode_kernel<2, float><<<grid, kThreads, 0, s>>>(in, nwords, g, maxbits, out); break;
    case 3: decode_kernel<3, float><<<grid, kThreads, 0, s>>>(in, nwords, g, maxbits, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace gzfp
