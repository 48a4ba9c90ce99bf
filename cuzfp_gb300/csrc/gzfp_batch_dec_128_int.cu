// Batch kernels (grid and persistent): decode, 128 threads per CTA, one kernel per
// integer kind.
#include "gzfp_batch_launch.h"

namespace gzfp {

cudaError_t launch_batch_dec_128_int(int kind_index, int grid, int bpt, bool ahead,
                                     uint32_t staged_w, const BatchDesc* descs,
                                     const uint32_t* chunk_item, uint64_t lo, uint64_t hi,
                                     unsigned long long* counter, cudaStream_t s) {
  return launch_batch_t<128, true, true>(kind_index, grid, bpt, ahead, staged_w, descs, chunk_item,
                                         lo, hi, counter, s);
}

int batch_occupancy_dec_128_int(int kind_index, uint32_t staged_w) {
  return batch_occupancy_t<128, true, true>(kind_index, staged_w);
}

}  // namespace gzfp
