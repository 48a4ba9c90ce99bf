// Persistent batch kernels with 64 threads per CTA (encode and decode).
#include "gzfp_batch_launch.h"

namespace gzfp {

cudaError_t launch_batch_64(bool decode, int grid, int bpt, bool ahead, const BatchDesc* descs,
                            const uint32_t* chunk_item, uint64_t nchunks,
                            unsigned long long* counter, cudaStream_t s) {
  return launch_batch_t<64>(decode, grid, bpt, ahead, descs, chunk_item, nchunks, counter, s);
}

int batch_occupancy_64(bool decode) { return batch_occupancy<64>(decode); }

}  // namespace gzfp
