// Block-access kernels (listed blocks to / from 4^d tiles) for float fields.
#include "gzfp_blocks.cuh"
#include "gzfp_launch.h"

namespace gzfp {

template cudaError_t launch_encode_blocks<float>(int, const float*, const unsigned long long*,
                                              const uint8_t*, uint64_t, uint32_t, uint64_t*,
                                              uint64_t, cudaStream_t);
template cudaError_t launch_decode_blocks<float>(int, const uint64_t*, uint64_t,
                                              const unsigned long long*, const uint8_t*, uint64_t,
                                              uint32_t, float*, cudaStream_t);

}  // namespace gzfp
