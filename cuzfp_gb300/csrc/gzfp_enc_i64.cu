// Encoder kernels for int64 integer fields (1D, 2D, 3D).
#include "gzfp_kernels.cuh"
#include "gzfp_launch.h"

namespace gzfp {

cudaError_t launch_encode_i64(int dims, const int64_t* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_encode_t<1, int64_t>(in, g, maxbits, out, nwords, s);
    case 2: return launch_encode_t<2, int64_t>(in, g, maxbits, out, nwords, s);
    case 3: return launch_encode_t<3, int64_t>(in, g, maxbits, out, nwords, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gzfp
