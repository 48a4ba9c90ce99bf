// Encoder kernels for float fields (1D, 2D, 3D).
#include "gzfp_kernels.cuh"
#include "gzfp_launch.h"

namespace gzfp {

cudaError_t launch_encode_f32(int dims, const float* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_encode_t<1, float>(in, g, maxbits, out, nwords, s);
    case 2: return launch_encode_t<2, float>(in, g, maxbits, out, nwords, s);
    case 3: return launch_encode_t<3, float>(in, g, maxbits, out, nwords, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gzfp
