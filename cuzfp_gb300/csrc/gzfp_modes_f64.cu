// General-mode kernels (fixed precision, fixed accuracy, any zfp stream
// parameters) for double fields.
#include "gzfp_launch.h"
#include "gzfp_modes.cuh"

namespace gzfp {

template cudaError_t launch_encode_mode<double>(int, const double*, const Geom&, const General&,
                                            uint64_t*, uint32_t, uint32_t*, cudaStream_t);
template cudaError_t launch_decode_mode<double>(int, const uint64_t*, uint64_t,
                                            const unsigned long long*, const Geom&,
                                            const General&, double*, cudaStream_t);
template cudaError_t launch_index_walk<double>(int, const IndexJob&, bool, cudaStream_t);
template cudaError_t launch_index_assemble<double>(int, const IndexJob&, const IndexPiece*, uint32_t,
                                            unsigned long long*, uint64_t, unsigned long long*,
                                            cudaStream_t);
template cudaError_t launch_index_blocks<double>(int, const uint64_t*, uint64_t, uint64_t,
                                             const General&, uint64_t, unsigned long long*,
                                             unsigned long long*, cudaStream_t);

}  // namespace gzfp
