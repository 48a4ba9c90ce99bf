// gzfp_launch.h -- internal launcher interface between the host API
// (gzfp_api.cu) and the kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gzfp_array.cuh"
#include "gzfp_index_host.h"

namespace gzfp {

// Launch the plain-path encoder / decoder for `dims` (1..3) on stream `s`.
cudaError_t launch_encode_f32(int dims, const float* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s);
cudaError_t launch_encode_f64(int dims, const double* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s);
cudaError_t launch_decode_f32(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, float* out, cudaStream_t s);
cudaError_t launch_decode_f64(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, double* out, cudaStream_t s);
cudaError_t launch_encode_i32(int dims, const int32_t* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s);
cudaError_t launch_encode_i64(int dims, const int64_t* in, const Geom& g, uint32_t maxbits,
                              uint64_t* out, uint64_t nwords, cudaStream_t s);
cudaError_t launch_decode_i32(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, int32_t* out, cudaStream_t s);
cudaError_t launch_decode_i64(int dims, const uint64_t* in, uint64_t nwords, const Geom& g,
                              uint32_t maxbits, int64_t* out, cudaStream_t s);

// Random access to listed blocks, each coded from / into its own tile of
// 4^dims values (gzfp_blocks.cuh; instantiated for float, double, int32_t
// and int64_t in gzfp_blocks_*.cu).
template <typename T>
cudaError_t launch_encode_blocks(int dims, const T* tiles, const unsigned long long* index,
                                 const uint8_t* shape, uint64_t count, uint32_t maxbits,
                                 uint64_t* out, uint64_t nwords, cudaStream_t s);
template <typename T>
cudaError_t launch_decode_blocks(int dims, const uint64_t* in, uint64_t nwords,
                                 const unsigned long long* index, const uint8_t* shape,
                                 uint64_t count, uint32_t maxbits, T* tiles, cudaStream_t s);

// zfp's general coding modes (gzfp_modes.cuh; instantiated for the four
// scalar types in gzfp_modes_*.cu): every block into its own scratch slot
// with its length, decoding from known start bits, and the serial walk that
// finds those start bits.  The scan and the placement of the blocks are
// type-independent (gzfp_modes_common.cu).
template <typename T>
cudaError_t launch_encode_mode(int dims, const T* in, const Geom& g, const General& mode,
                               uint64_t* scratch, uint32_t slot_words, uint32_t* lengths,
                               cudaStream_t s);
template <typename T>
cudaError_t launch_decode_mode(int dims, const uint64_t* in, uint64_t nwords,
                               const unsigned long long* offsets, const Geom& g,
                               const General& mode, T* out, cudaStream_t s);
template <typename T>
cudaError_t launch_index_blocks(int dims, const uint64_t* in, uint64_t nwords, uint64_t nblocks,
                                const General& mode, uint64_t first, unsigned long long* offsets,
                                unsigned long long* end, cudaStream_t s);
// Exclusive scan of n block lengths into start bits from `first` (sums:
// room for ceil(n / 4096) + 1 entries; sums[ceil(n / 4096)] receives the
// total length), then the placement of every block at its start bit in a
// zeroed stream.
cudaError_t launch_scan_lengths(const uint32_t* lengths, uint64_t n, uint64_t first,
                                uint64_t* sums, unsigned long long* offsets, cudaStream_t s);
uint64_t scan_sums_count(uint64_t n);
// most bits one block can take under `mode` (gzfp_modes.cuh block_bound)
uint32_t block_bound_host(int dims, int P, int ebits, const General& mode);
// offsets[b] = first + b * maxbits: the start bits of a fixed-rate stream
cudaError_t launch_fixed_offsets(unsigned long long* offsets, uint64_t n, uint64_t first,
                                 uint32_t maxbits, cudaStream_t s);
// Parallel index of a general-mode stream (gzfp_modes.cuh): walkers over
// segments of the stream, their extensions up to the chain they merge with,
// and the assembly of the true chain's pieces into the block offsets.
struct IndexJob {
  const uint64_t* in;
  uint64_t nwords;
  General mode;
  uint64_t first;                // bit of block 0
  uint64_t seg_bits;             // segment length
  uint32_t nseg, cap;            // segments, positions a segment's list holds
  uint32_t ext_cap;              // steps an extension may take
  unsigned long long* lists;     // nseg * cap block starts, in stream order
  unsigned long long* counts;    // per segment: entries in its list (cap + 1: overflow)
  unsigned long long* exits;     // per segment: the walker's first start past its end
  unsigned long long* info;      // per segment: extension steps, merge segment, merge
                                 // index, status (0 merged, 1 stream end, 2 failed)
};
template <typename T>
cudaError_t launch_index_walk(int dims, const IndexJob& j, bool extend, cudaStream_t s);
template <typename T>
cudaError_t launch_index_assemble(int dims, const IndexJob& j, const IndexPiece* pieces,
                                  uint32_t npieces, unsigned long long* offsets, uint64_t nblocks,
                                  unsigned long long* end, cudaStream_t s);

cudaError_t launch_place_blocks(const uint64_t* scratch, uint32_t slot_words,
                                const uint32_t* lengths, const unsigned long long* offsets,
                                uint64_t nblocks, uint64_t* out, cudaStream_t s);

}  // namespace gzfp
