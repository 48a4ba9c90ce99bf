// gzfp_modes.cuh -- zfp's general coding modes on the GPU: fixed precision,
// fixed accuracy and any other setting of the four stream parameters
// (zfp_stream_set_precision / _accuracy / _params, Z/src/zfp.c:432-510).
//
// Blocks then have their own lengths and follow one another in the stream
// (Z/src/template/compress.c), so a block's position is the sum of the
// lengths before it.  Compression runs in three steps: every block is coded
// into its own scratch slot and its length recorded; an exclusive scan of
// the lengths gives every block's start bit; every block's bits are then
// moved to that position.  Decompression decodes every block from its start
// bit when the offsets are known (the compressor returns them); otherwise a
// single thread first walks the blocks to find them, which is serial in the
// number of blocks.
#pragma once

#include "gzfp_kernels.cuh"

namespace gzfp {

// most bits one block can take under `mode`: zfp_stream_maximum_size's
// per-block bound (Z/src/zfp.c:368-397), raised to minbits
GZ_HD uint32_t block_bound(int dims, int P, int ebits, const General& mode) {
  const uint32_t values = 1u << (2 * dims);
  const uint32_t prec = mode.maxprec < (uint32_t)P ? mode.maxprec : (uint32_t)P;
  uint32_t b = 1 + (uint32_t)ebits + values - 1 + values * prec;
  b = b < mode.maxbits ? b : mode.maxbits;
  return b > mode.minbits ? b : mode.minbits;
}

// Step 1: block b coded into scratch words [b * slot_words, ...), its length
// in bits to lengths[b].  The slot is the block's alone, so every word is a
// plain store.
template <int D, typename T>
__global__ void __launch_bounds__(kThreads, (MinBlocks<D, T>::value))
    encode_mode_kernel(const T* __restrict__ in, Geom g, General mode,
                       uint64_t* __restrict__ scratch, uint32_t slot_words,
                       uint32_t* __restrict__ lengths) {
  typedef typename FT<T>::UInt UInt;
  constexpr int BS = 1 << (2 * D);
  extern __shared__ uint64_t smem[];
  const Plane4Tables* t4 = stage_tables<D, kThreads>(smem);
  SmemPlanes ps{smem + table_words<D>() + threadIdx.x, t4};
  const uint64_t b = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (b >= g.nblocks) return;
  uint32_t ix, iy, iz;
  block_coords(g, b, ix, iy, iz);
  UInt raw[BS];
  gather<D, T>(in, g, ix, iy, iz, raw);
  BitWriter<DevWords> w(DevWords{scratch + b * slot_words, nullptr, slot_words}, 0,
                        slot_words * 64);
  lengths[b] = encode_block_mode<D, T>(raw, mode, w, ps);
  w.finish();
}

// Steps 2 and 3 (the scan of the lengths and the placement of the blocks)
// do not depend on the scalar type: gzfp_modes_common.cu.

// Decode block b from stream bit offsets[b].
template <int D, typename T>
__global__ void __launch_bounds__(kThreads, (MinBlocks<D, T>::value))
    decode_mode_kernel(const uint64_t* __restrict__ in, uint64_t nwords,
                       const unsigned long long* __restrict__ offsets, Geom g, General mode,
                       T* __restrict__ out) {
  typedef typename FT<T>::UInt UInt;
  constexpr int BS = 1 << (2 * D);
  extern __shared__ uint64_t smem[];
  const Plane4Tables* t4 = stage_tables<D, kThreads>(smem);
  SmemPlanes ps{smem + table_words<D>() + threadIdx.x, t4};
  const uint64_t b = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (b >= g.nblocks) return;
  uint32_t ix, iy, iz;
  block_coords(g, b, ix, iy, iz);
  BitReader<DevWords> r(DevWords{nullptr, in, nwords}, offsets[b]);
  UInt raw[BS];
  decode_block_mode<D, T>(r, mode, raw, ps);
  scatter<D, T>(out, g, ix, iy, iz, raw);
}

// One thread walks the blocks of a stream from bit `first` (after a header,
// or 0): offsets[b] = start bit of block b, *end = the bit after the last
// block.  Reads past the stream's words see zeros, so a short stream ends
// the walk with an end past its size.
template <int D, typename T>
__global__ void index_blocks_kernel(const uint64_t* __restrict__ in, uint64_t nwords,
                                    uint64_t nblocks, General mode, uint64_t first,
                                    unsigned long long* __restrict__ offsets,
                                    unsigned long long* __restrict__ end) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  uint64_t pos = first;
  for (uint64_t b = 0; b < nblocks; b++) {
    offsets[b] = pos;
    BitReader<DevWords> r(DevWords{nullptr, in, nwords}, pos);
    pos += block_bits<D, T>(r, mode);
  }
  *end = pos;
}

template <int D, typename T>
cudaError_t launch_encode_mode_t(const T* in, const Geom& g, const General& mode,
                                 uint64_t* scratch, uint32_t slot_words, uint32_t* lengths,
                                 cudaStream_t s) {
  if (g.nblocks == 0) return cudaSuccess;
  const dim3 grid((unsigned)((g.nblocks + kThreads - 1) / kThreads));
  const size_t sm = smem_bytes(store_slots<D, T>(), false, 0, table_words<D>());
  auto k = encode_mode_kernel<D, T>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<grid, kThreads, sm, s>>>(in, g, mode, scratch, slot_words, lengths);
  return cudaGetLastError();
}

template <int D, typename T>
cudaError_t launch_decode_mode_t(const uint64_t* in, uint64_t nwords,
                                 const unsigned long long* offsets, const Geom& g,
                                 const General& mode, T* out, cudaStream_t s) {
  if (g.nblocks == 0) return cudaSuccess;
  const dim3 grid((unsigned)((g.nblocks + kThreads - 1) / kThreads));
  const size_t sm = smem_bytes(decode_slots<D, T>(), false, 0, table_words<D>());
  auto k = decode_mode_kernel<D, T>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<grid, kThreads, sm, s>>>(in, nwords, offsets, g, mode, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_encode_mode(int dims, const T* in, const Geom& g, const General& mode,
                               uint64_t* scratch, uint32_t slot_words, uint32_t* lengths,
                               cudaStream_t s) {
  switch (dims) {
    case 1: return launch_encode_mode_t<1, T>(in, g, mode, scratch, slot_words, lengths, s);
    case 2: return launch_encode_mode_t<2, T>(in, g, mode, scratch, slot_words, lengths, s);
    case 3: return launch_encode_mode_t<3, T>(in, g, mode, scratch, slot_words, lengths, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t launch_decode_mode(int dims, const uint64_t* in, uint64_t nwords,
                               const unsigned long long* offsets, const Geom& g,
                               const General& mode, T* out, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_decode_mode_t<1, T>(in, nwords, offsets, g, mode, out, s);
    case 2: return launch_decode_mode_t<2, T>(in, nwords, offsets, g, mode, out, s);
    case 3: return launch_decode_mode_t<3, T>(in, nwords, offsets, g, mode, out, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t launch_index_blocks(int dims, const uint64_t* in, uint64_t nwords, uint64_t nblocks,
                                const General& mode, uint64_t first, unsigned long long* offsets,
                                unsigned long long* end, cudaStream_t s) {
  switch (dims) {
    case 1: index_blocks_kernel<1, T><<<1, 1, 0, s>>>(in, nwords, nblocks, mode, first, offsets, end); break;
    case 2: index_blocks_kernel<2, T><<<1, 1, 0, s>>>(in, nwords, nblocks, mode, first, offsets, end); break;
    case 3: index_blocks_kernel<3, T><<<1, 1, 0, s>>>(in, nwords, nblocks, mode, first, offsets, end); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace gzfp
