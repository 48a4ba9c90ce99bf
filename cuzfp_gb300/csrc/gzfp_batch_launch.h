// gzfp_batch_launch.h -- internal interface between the batch host code
// (gzfp_batch.cu, gzfp_batch_noalloc.cu, gzfp_serve.cu) and the batch
// kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include "gzfp_batch.cuh"

namespace gzfp {

#define GZFP_BATCH_DECL(dir, nt)                                                              \
  cudaError_t launch_batch_##dir##_##nt(int kind_index, int grid, int bpt, bool ahead,        \
                                        uint32_t staged_w, const BatchDesc* descs,             \
                                        const uint32_t* chunk_item, uint64_t lo, uint64_t hi,  \
                                        unsigned long long* counter, cudaStream_t s);          \
  int batch_occupancy_##dir##_##nt(int kind_index, uint32_t staged_w);

// Launch the persistent kernel of kind `kind_index` (into kBatchKind) over
// chunks [lo, hi) with 64, 128 or 256 threads per CTA on `grid` CTAs, and
// report its resident CTAs per SM (staged_w: decode staging depth in words
// per block, 0 for none).  Defined in gzfp_batch_{enc,dec}_<threads>.cu.
GZFP_BATCH_DECL(enc, 64)
GZFP_BATCH_DECL(enc, 128)
GZFP_BATCH_DECL(enc, 256)
GZFP_BATCH_DECL(dec, 64)
GZFP_BATCH_DECL(dec, 128)
GZFP_BATCH_DECL(dec, 256)
#undef GZFP_BATCH_DECL

inline cudaError_t launch_batch(int threads, bool decode, int kind_index, int grid, int bpt,
                                bool ahead, uint32_t staged_w, const BatchDesc* descs,
                                const uint32_t* chunk_item, uint64_t lo, uint64_t hi,
                                unsigned long long* counter, cudaStream_t s) {
  auto f = decode ? (threads == 64 ? launch_batch_dec_64 : threads == 128 ? launch_batch_dec_128
                                                                           : launch_batch_dec_256)
                  : (threads == 64 ? launch_batch_enc_64 : threads == 128 ? launch_batch_enc_128
                                                                           : launch_batch_enc_256);
  return f(kind_index, grid, bpt, ahead, staged_w, descs, chunk_item, lo, hi, counter, s);
}

inline int batch_occupancy(int threads, bool decode, int kind_index, uint32_t staged_w) {
  auto f = decode ? (threads == 64 ? batch_occupancy_dec_64 : threads == 128 ? batch_occupancy_dec_128
                                                                              : batch_occupancy_dec_256)
                  : (threads == 64 ? batch_occupancy_enc_64 : threads == 128 ? batch_occupancy_enc_128
                                                                              : batch_occupancy_enc_256);
  return f(kind_index, staged_w);
}

// Record the detail that gzfp_batch_last_error returns on this thread.
void batch_set_error(const char* msg);

}  // namespace gzfp
