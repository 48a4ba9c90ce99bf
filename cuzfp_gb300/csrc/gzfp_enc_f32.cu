// Encoder kernels for float fields (1D, 2D, 3D).
#include "gzfp_kernels.cuh"
#include "gzfp_launch.h"

namespace gzfp {

cudaError_t launch_encode_f32(int dims, const float* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s) {
  if (g.nblocks == 0) return cudaSuccess;
  const dim3 grid((unsigned)((g.nblocks + kThreads - 1) / kThreads));
  switch (dims) {
    case 1: encode_kernel<1, float><<<grid, kThreads, 0, s>>>(in, g, maxbits, out, nwords); break;
    case 2: encode_kernel<2, float><<<grid, kThreads, 0, s>>>(in, g, maxbits, out, nwords); break;
    case 3: encode_kernel<3, float><<<grid, kThreads, 0, s>>>(in, g, maxbits, out, nwords); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace gzfp
