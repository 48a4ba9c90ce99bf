// Persistent batch kernels with 256 threads per CTA (encode and decode).
#include "gzfp_batch_launch.h"

namespace gzfp {

cudaError_t launch_batch_256(bool decode, int grid, int bpt, bool ahead, const BatchDesc* descs,
                            const uint32_t* chunk_item, uint64_t nchunks,
                            unsigned long long* counter, cudaStream_t s) {
  return launch_batch_t<256>(decode, grid, bpt, ahead, descs, chunk_item, nchunks, counter, s);
}

int batch_occupancy_256(bool decode) { return batch_occupancy<256>(decode); }

}  // namespace gzfp
