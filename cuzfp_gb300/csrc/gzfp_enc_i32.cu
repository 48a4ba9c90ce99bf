// Encoder kernels for int32 integer fields (1D, 2D, 3D).
#include "gzfp_kernels.cuh"
#include "gzfp_launch.h"

namespace gzfp {

cudaError_t launch_encode_i32(int dims, const int32_t* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_encode_t<1, int32_t>(in, g, maxbits, out, nwords, s);
    case 2: return launch_encode_t<2, int32_t>(in, g, maxbits, out, nwords, s);
    case 3: return launch_encode_t<3, int32_t>(in, g, maxbits, out, nwords, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gzfp
