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
// bit when the offsets are known (the compressor returns them); otherwise
// the starts are found first, by walkers over segments of the stream whose
// chains are joined where they merge (below), or, failing that, by a single
// thread walking every block in order.
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

// ---------------------------------------------------------- parallel index
// A block's length is known only by parsing it, so the block starts of a
// stream without offsets form a chain p -> p + block_bits(p) from block 0.
// A chain started at any other bit soon lands on a start of the true chain
// (on fixed-accuracy streams of smooth fields, after a few hundred to a few
// thousand blocks), and from there on the two are the same chain.  So:
//  1. one walker per segment of the stream records the chain from the
//     segment's first bit to its end (index_walk_kernel, extend = false);
//  2. each walker goes on past its end until its chain reaches a start that
//     a later segment's walker recorded (extend = true): the merge;
//  3. the host follows the merges from segment 0, whose walker starts at
//     block 0, and index_assemble_kernel copies the true chain's pieces --
//     list entries, and re-walked extensions -- into the offsets.
// A walker whose list overflows or whose extension does not merge within
// ext_cap steps makes the host fall back to the serial walk.

GZ_HD uint64_t index_step_bits(uint32_t bits) { return bits ? bits : 1; }

// One walker per warp: lane 0 walks, the other lanes leave at once.  Walkers
// sharing a warp diverge on every block (each parses a different one), so a
// lone lane walks about 5x faster than 32 lanes in lockstep.
template <int D, typename T>
__global__ void index_walk_kernel(IndexJob j, bool extend) {
  const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
  if (gt & 31) return;
  const uint32_t s = gt >> 5;
  if (s >= j.nseg) return;
  const uint64_t total = j.nwords * 64;
  const DevWords words{nullptr, j.in, j.nwords};
  if (!extend) {
    const uint64_t lo = j.first + (uint64_t)s * j.seg_bits, hi = lo + j.seg_bits;
    uint64_t p = lo, n = 0;
    unsigned long long* list = j.lists + (uint64_t)s * j.cap;
    while (p < hi && p < total) {
      if (n == j.cap) {  // more starts than the list holds
        n = j.cap + 1ull;
        break;
      }
      list[n++] = p;
      BitReader<DevWords> r(words, p);
      p += index_step_bits(block_bits<D, T>(r, j.mode));
    }
    j.counts[s] = n;
    j.exits[s] = p;
    return;
  }
  // extension: from the walker's exit to the first start recorded by a
  // later segment
  uint64_t p = j.exits[s], steps = 0, k = s + 1, idx = 0;
  unsigned long long status = 2;
  if (j.counts[s] <= j.cap) {
    for (;;) {
      if (p >= total || k >= j.nseg) {
        status = 1;
        break;
      }
      while (k + 1 < j.nseg && p >= j.first + (k + 1) * j.seg_bits) k++;
      const unsigned long long n = j.counts[k];
      if (n > j.cap) break;  // that list overflowed: no merge can be trusted
      const unsigned long long* list = j.lists + k * j.cap;
      uint64_t lo = 0, hi = n;  // first entry >= p
      while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (list[mid] < p) lo = mid + 1; else hi = mid;
      }
      if (lo < n && list[lo] == p) {
        idx = lo;
        status = 0;
        break;
      }
      if (steps == j.ext_cap) break;
      steps++;
      BitReader<DevWords> r(words, p);
      p += index_step_bits(block_bits<D, T>(r, j.mode));
    }
  }
  unsigned long long* inf = j.info + 4ull * s;
  inf[0] = steps;
  inf[1] = k;
  inf[2] = idx;
  inf[3] = status;
}

// one CTA per piece: list pieces are copied by all threads, walk pieces
// re-walk an extension on one thread; offsets past nblocks are dropped
template <int D, typename T>
__global__ void index_assemble_kernel(IndexJob j, const IndexPiece* pieces,
                                      unsigned long long* offsets, uint64_t nblocks) {
  const IndexPiece pc = pieces[blockIdx.x];
  if (!pc.walk) {
    for (uint64_t i = threadIdx.x; i < pc.count && pc.dst + i < nblocks; i += blockDim.x)
      offsets[pc.dst + i] = j.lists[pc.src + i];
    return;
  }
  if (threadIdx.x != 0) return;
  const DevWords words{nullptr, j.in, j.nwords};
  uint64_t p = j.exits[pc.seg];
  for (uint64_t i = 0; i < pc.count && pc.dst + i < nblocks; i++) {
    offsets[pc.dst + i] = p;
    BitReader<DevWords> r(words, p);
    p += index_step_bits(block_bits<D, T>(r, j.mode));
  }
}

// the bit after the last block
template <int D, typename T>
__global__ void index_end_kernel(IndexJob j, const unsigned long long* offsets, uint64_t nblocks,
                                 unsigned long long* end) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const uint64_t p = offsets[nblocks - 1];
  BitReader<DevWords> r(DevWords{nullptr, j.in, j.nwords}, p);
  *end = p + block_bits<D, T>(r, j.mode);
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

template <int D, typename T>
cudaError_t launch_index_walk_t(const IndexJob& j, bool extend, cudaStream_t s) {
  const unsigned threads = 64;  // two walkers per CTA, one per warp
  index_walk_kernel<D, T><<<(j.nseg * 32 + threads - 1) / threads, threads, 0, s>>>(j, extend);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_index_walk(int dims, const IndexJob& j, bool extend, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_index_walk_t<1, T>(j, extend, s);
    case 2: return launch_index_walk_t<2, T>(j, extend, s);
    case 3: return launch_index_walk_t<3, T>(j, extend, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int D, typename T>
cudaError_t launch_index_assemble_t(const IndexJob& j, const IndexPiece* pieces, uint32_t npieces,
                                    unsigned long long* offsets, uint64_t nblocks,
                                    unsigned long long* end, cudaStream_t s) {
  index_assemble_kernel<D, T><<<npieces, 128, 0, s>>>(j, pieces, offsets, nblocks);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  index_end_kernel<D, T><<<1, 1, 0, s>>>(j, offsets, nblocks, end);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_index_assemble(int dims, const IndexJob& j, const IndexPiece* pieces,
                                  uint32_t npieces, unsigned long long* offsets, uint64_t nblocks,
                                  unsigned long long* end, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_index_assemble_t<1, T>(j, pieces, npieces, offsets, nblocks, end, s);
    case 2: return launch_index_assemble_t<2, T>(j, pieces, npieces, offsets, nblocks, end, s);
    case 3: return launch_index_assemble_t<3, T>(j, pieces, npieces, offsets, nblocks, end, s);
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
