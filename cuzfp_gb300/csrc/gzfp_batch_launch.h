// gzfp_batch_launch.h -- internal interface between the batch host API
// (gzfp_batch.cu) and the batch kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include "gzfp_batch.cuh"

namespace gzfp {

// Launch the persistent batch kernel with `threads` (64, 128 or 256) per CTA
// on `grid` CTAs.  Defined in gzfp_batch_{enc,dec}_<threads>.cu.
cudaError_t launch_batch_64(bool decode, int grid, int bpt, bool ahead, const BatchDesc* descs,
                            const uint32_t* chunk_item, uint64_t nchunks,
                            unsigned long long* counter, cudaStream_t s);
cudaError_t launch_batch_128(bool decode, int grid, int bpt, bool ahead, const BatchDesc* descs,
                             const uint32_t* chunk_item, uint64_t nchunks,
                             unsigned long long* counter, cudaStream_t s);
cudaError_t launch_batch_256(bool decode, int grid, int bpt, bool ahead, const BatchDesc* descs,
                             const uint32_t* chunk_item, uint64_t nchunks,
                             unsigned long long* counter, cudaStream_t s);

// resident CTAs per SM of the batch kernel at 64 / 128 / 256 threads per CTA
int batch_occupancy_64(bool decode);
int batch_occupancy_128(bool decode);
int batch_occupancy_256(bool decode);

// Record the detail that gzfp_batch_last_error returns on this thread.
void batch_set_error(const char* msg);

}  // namespace gzfp
