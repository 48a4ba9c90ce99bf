// gzfp_batch_launch.h -- internal interface between the batch host code
// (gzfp_batch.cu, gzfp_batch_noalloc.cu, gzfp_serve.cu) and the batch
// kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include "gzfp.h"
#include "gzfp_batch.cuh"

namespace gzfp {

// Scalar types a batch takes, and per type: the block header's exponent
// bits (none for integers), the alignment that lets a row of four values
// move as one vector, and the kind code (kBatchKind) of an array.
inline bool batch_type_ok(int type) {
  return type == GZFP_TYPE_FLOAT || type == GZFP_TYPE_DOUBLE || type == GZFP_TYPE_INT32 ||
         type == GZFP_TYPE_INT64;
}
inline unsigned batch_ebits(int type) {
  return type == GZFP_TYPE_FLOAT ? 8 : type == GZFP_TYPE_DOUBLE ? 11 : 0;
}
inline size_t batch_scalar_size(int type) {
  return type == GZFP_TYPE_FLOAT || type == GZFP_TYPE_INT32 ? 4 : 8;
}
inline uintptr_t batch_row_align(int type) { return 4 * batch_scalar_size(type); }
inline uint32_t batch_kind(int type, int dims) {
  const uint32_t slot = type == GZFP_TYPE_FLOAT    ? 0u
                        : type == GZFP_TYPE_DOUBLE ? 1u
                        : type == GZFP_TYPE_INT32  ? 2u
                                                   : 3u;
  return (uint32_t)dims | slot << 3;
}

#define GZFP_BATCH_DECL(dir, nt, grp)                                                         \
  cudaError_t launch_batch_##dir##_##nt##grp(int kind_index, int grid, int bpt, bool ahead,     \
                                             uint32_t staged_w, const BatchDesc* descs,        \
                                             const uint32_t* chunk_item, uint64_t lo,          \
                                             uint64_t hi, unsigned long long* counter,         \
                                             cudaStream_t s);                                  \
  int batch_occupancy_##dir##_##nt##grp(int kind_index, uint32_t staged_w);

// Launch the kernel of kind `kind_index` (into kBatchKind) over chunks
// [lo, hi) with 64, 128 or 256 threads per CTA: the persistent kernel on
// `grid` CTAs, or the grid kernel for grid == 0 (launch_batch_kind in
// gzfp_batch.cuh); and report the persistent kernel's resident CTAs per SM
// (staged_w: staging depth in words per block, 0 for none).  Defined in gzfp_batch_{enc,dec}_<threads>.cu
// (floating-point kinds) and gzfp_batch_{enc,dec}_<threads>_int.cu
// (integer kinds).
GZFP_BATCH_DECL(enc, 64, )
GZFP_BATCH_DECL(enc, 128, )
GZFP_BATCH_DECL(enc, 256, )
GZFP_BATCH_DECL(dec, 64, )
GZFP_BATCH_DECL(dec, 128, )
GZFP_BATCH_DECL(dec, 256, )
GZFP_BATCH_DECL(enc, 64, _int)
GZFP_BATCH_DECL(enc, 128, _int)
GZFP_BATCH_DECL(enc, 256, _int)
GZFP_BATCH_DECL(dec, 64, _int)
GZFP_BATCH_DECL(dec, 128, _int)
GZFP_BATCH_DECL(dec, 256, _int)
#undef GZFP_BATCH_DECL

inline cudaError_t launch_batch(int threads, bool decode, int kind_index, int grid, int bpt,
                                bool ahead, uint32_t staged_w, const BatchDesc* descs,
                                const uint32_t* chunk_item, uint64_t lo, uint64_t hi,
                                unsigned long long* counter, cudaStream_t s) {
  const bool ints = kind_index >= kBatchFloatKinds;
  decltype(&launch_batch_enc_64) f;
  if (threads == 64)
    f = decode ? (ints ? launch_batch_dec_64_int : launch_batch_dec_64)
               : (ints ? launch_batch_enc_64_int : launch_batch_enc_64);
  else if (threads == 128)
    f = decode ? (ints ? launch_batch_dec_128_int : launch_batch_dec_128)
               : (ints ? launch_batch_enc_128_int : launch_batch_enc_128);
  else
    f = decode ? (ints ? launch_batch_dec_256_int : launch_batch_dec_256)
               : (ints ? launch_batch_enc_256_int : launch_batch_enc_256);
  return f(kind_index, grid, bpt, ahead, staged_w, descs, chunk_item, lo, hi, counter, s);
}

inline int batch_occupancy(int threads, bool decode, int kind_index, uint32_t staged_w) {
  const bool ints = kind_index >= kBatchFloatKinds;
  decltype(&batch_occupancy_enc_64) f;
  if (threads == 64)
    f = decode ? (ints ? batch_occupancy_dec_64_int : batch_occupancy_dec_64)
               : (ints ? batch_occupancy_enc_64_int : batch_occupancy_enc_64);
  else if (threads == 128)
    f = decode ? (ints ? batch_occupancy_dec_128_int : batch_occupancy_dec_128)
               : (ints ? batch_occupancy_enc_128_int : batch_occupancy_enc_128);
  else
    f = decode ? (ints ? batch_occupancy_dec_256_int : batch_occupancy_dec_256)
               : (ints ? batch_occupancy_enc_256_int : batch_occupancy_enc_256);
  return f(kind_index, staged_w);
}

// Record the detail that gzfp_batch_last_error returns on this thread.
void batch_set_error(const char* msg);

}  // namespace gzfp
