// Decoder kernels for int64 integer fields (1D, 2D, 3D).
#include "gzfp_kernels.cuh"
#include "gzfp_launch.h"

namespace gzfp {

cudaError_t launch_decode_i64(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, int64_t* out, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_decode_t<1, int64_t>(in, nwords, g, maxbits, out, s);
    case 2: return launch_decode_t<2, int64_t>(in, nwords, g, maxbits, out, s);
    case 3: return launch_decode_t<3, int64_t>(in, nwords, g, maxbits, out, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gzfp
