// Decoder kernels for int32 integer fields (1D, 2D, 3D).
#include "gzfp_kernels.cuh"
#include "gzfp_launch.h"

namespace gzfp {

cudaError_t launch_decode_i32(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, int32_t* out, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_decode_t<1, int32_t>(in, nwords, g, maxbits, out, s);
    case 2: return launch_decode_t<2, int32_t>(in, nwords, g, maxbits, out, s);
    case 3: return launch_decode_t<3, int32_t>(in, nwords, g, maxbits, out, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gzfp
