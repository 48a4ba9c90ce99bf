// gzfp_blocks.cuh -- random access to single blocks of a fixed-rate stream.
//
// A list of block indices, each coded from or into its own tile of 4^D
// values (x fastest) in a block buffer: zfp's per-block API
// (zfp_encode_block_* / zfp_decode_block_* and the partial-block forms,
// Z/inc/zfp.h:452-521) as its compressed arrays use it to write back and
// fetch cached blocks (Z/array/zfparray3.h:225-255): block `index` occupies
// bits [index * maxbits, (index + 1) * maxbits) of the stream.  One thread
// per listed block, with the plain path's per-block codec.
#pragma once

#include "gzfp_kernels.cuh"

namespace gzfp {

// zfp's partial-block shape code (Z/array/zfpcodecd.h:5-75): two bits per
// axis, x lowest, each 4 minus the block's extent along that axis.
// Entry i of a list is coded as a one-block field of those extents whose
// values sit in the 4^D tile (strides 1, 4, 16) and whose block starts at
// the slot's first bit.
template <int D>
__device__ __forceinline__ Geom tile_geom(uint32_t shape, uint64_t slot_bit, uint32_t vec) {
  Geom g;
  g.nx = 4 - (shape & 3u);
  g.ny = D >= 2 ? 4 - ((shape >> 2) & 3u) : 1;
  g.nz = D >= 3 ? 4 - ((shape >> 4) & 3u) : 1;
  g.bx = g.by = g.bz = 1;
  g.nblocks = 1;
  g.sx = 1;
  g.sy = 4;
  g.sz = 16;
  g.base = slot_bit;
  g.vec = vec;
  g.dbx = g.dby = FastDiv{1, 1, 0};
  return g;
}

// Clear the stream bits [pos, pos + n) in the words the slot shares with its
// neighbours, so that a rewritten block can be merged in.  The slot's inner
// words are overwritten whole by the bit writer.  Neighbouring slots clear
// and merge disjoint bits of a shared word, so every order gives one result.
__device__ __forceinline__ void clear_slot_edges(uint64_t* words, uint64_t pos, uint32_t n) {
  const uint64_t end = pos + n;
  const uint64_t w0 = pos >> 6, w1 = end >> 6;  // first word, word holding bit `end`
  const uint32_t lo = (uint32_t)(pos & 63), hi = (uint32_t)(end & 63);
  if (lo || w1 == w0) {  // the first word is shared (or holds the whole slot)
    const uint64_t keep = lowmask64(lo) | (w1 == w0 ? ~lowmask64(hi) : 0ull);
    atomicAnd((unsigned long long*)(words + w0), (unsigned long long)keep);
  }
  if (hi && w1 != w0)  // the last word is shared
    atomicAnd((unsigned long long*)(words + w1), (unsigned long long)~lowmask64(hi));
}

template <int D, typename T>
__global__ void __launch_bounds__(kThreads, (MinBlocks<D, T>::value))
    encode_blocks_kernel(const T* __restrict__ tiles, const unsigned long long* __restrict__ index,
                         const uint8_t* __restrict__ shape, uint64_t count, uint32_t maxbits,
                         uint64_t* __restrict__ out, uint64_t nwords, uint32_t vec) {
  extern __shared__ uint64_t smem[];
  const Plane4Tables* t4 = stage_tables<D, kThreads>(smem);
  SmemPlanes ps{smem + table_words<D>() + threadIdx.x, t4};
  const uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= count) return;
  const uint64_t slot = index[i];
  if (slot >= nwords * 64 / maxbits) return;  // slots past the stream are skipped
  const uint64_t pos = slot * maxbits;
  clear_slot_edges(out, pos, maxbits);
  const Geom g = tile_geom<D>(shape ? shape[i] : 0u, pos, vec);
  encode_one<D, T>(tiles + i * (1u << (2 * D)), g, 0, maxbits, DevWords{out, nullptr, nwords}, ps);
}

template <int D, typename T>
__global__ void __launch_bounds__(kThreads, (MinBlocks<D, T>::value))
    decode_blocks_kernel(const uint64_t* __restrict__ in, uint64_t nwords,
                         const unsigned long long* __restrict__ index,
                         const uint8_t* __restrict__ shape, uint64_t count, uint32_t maxbits,
                         T* __restrict__ tiles, uint32_t vec) {
  extern __shared__ uint64_t smem[];
  const Plane4Tables* t4 = stage_tables<D, kThreads>(smem);
  SmemPlanes ps{smem + table_words<D>() + threadIdx.x, t4};
  const uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= count) return;
  const uint64_t slot = index[i];
  if (slot >= nwords * 64 / maxbits) return;  // slots past the stream are skipped
  const Geom g = tile_geom<D>(shape ? shape[i] : 0u, slot * maxbits, vec);
  decode_one<D, T>(tiles + i * (1u << (2 * D)), g, 0, maxbits, DevWords{nullptr, in, nwords}, ps);
}

template <int D, typename T>
cudaError_t launch_encode_blocks_t(const T* tiles, const unsigned long long* index,
                                   const uint8_t* shape, uint64_t count, uint32_t maxbits,
                                   uint64_t* out, uint64_t nwords, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  const dim3 grid((unsigned)((count + kThreads - 1) / kThreads));
  const size_t sm = smem_bytes(store_slots<D, T>(), false, 0, table_words<D>());
  auto k = encode_blocks_kernel<D, T>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const uint32_t vec = (uintptr_t)tiles % (4 * sizeof(T)) == 0 ? 1u : 0u;
  k<<<grid, kThreads, sm, s>>>(tiles, index, shape, count, maxbits, out, nwords, vec);
  return cudaGetLastError();
}

template <int D, typename T>
cudaError_t launch_decode_blocks_t(const uint64_t* in, uint64_t nwords,
                                   const unsigned long long* index, const uint8_t* shape,
                                   uint64_t count, uint32_t maxbits, T* tiles, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  const dim3 grid((unsigned)((count + kThreads - 1) / kThreads));
  const size_t sm = smem_bytes(decode_slots<D, T>(), false, 0, table_words<D>());
  auto k = decode_blocks_kernel<D, T>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const uint32_t vec = (uintptr_t)tiles % (4 * sizeof(T)) == 0 ? 1u : 0u;
  k<<<grid, kThreads, sm, s>>>(in, nwords, index, shape, count, maxbits, tiles, vec);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_encode_blocks(int dims, const T* tiles, const unsigned long long* index,
                                 const uint8_t* shape, uint64_t count, uint32_t maxbits,
                                 uint64_t* out, uint64_t nwords, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_encode_blocks_t<1, T>(tiles, index, shape, count, maxbits, out, nwords, s);
    case 2: return launch_encode_blocks_t<2, T>(tiles, index, shape, count, maxbits, out, nwords, s);
    case 3: return launch_encode_blocks_t<3, T>(tiles, index, shape, count, maxbits, out, nwords, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t launch_decode_blocks(int dims, const uint64_t* in, uint64_t nwords,
                                 const unsigned long long* index, const uint8_t* shape,
                                 uint64_t count, uint32_t maxbits, T* tiles, cudaStream_t s) {
  switch (dims) {
    case 1: return launch_decode_blocks_t<1, T>(in, nwords, index, shape, count, maxbits, tiles, s);
    case 2: return launch_decode_blocks_t<2, T>(in, nwords, index, shape, count, maxbits, tiles, s);
    case 3: return launch_decode_blocks_t<3, T>(in, nwords, index, shape, count, maxbits, tiles, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gzfp
