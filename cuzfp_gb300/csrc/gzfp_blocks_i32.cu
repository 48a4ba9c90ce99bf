// Block-access kernels (listed blocks to / from 4^d tiles) for int32 fields.
#include "gzfp_blocks.cuh"
#include "gzfp_launch.h"

namespace gzfp {

template cudaError_t launch_encode_blocks<int32_t>(int, const int32_t*, const unsigned long long*,
                                              const uint8_t*, uint64_t, uint32_t, uint64_t*,
                                              uint64_t, cudaStream_t);
template cudaError_t launch_decode_blocks<int32_t>(int, const uint64_t*, uint64_t,
                                              const unsigned long long*, const uint8_t*, uint64_t,
                                              uint32_t, int32_t*, cudaStream_t);

}  // namespace gzfp
