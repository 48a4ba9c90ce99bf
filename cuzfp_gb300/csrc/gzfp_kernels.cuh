// gzfp_kernels.cuh -- the plain-path CUDA kernels: one thread per zfp block.
//
// Encode: gather 4^D values (consecutive threads own consecutive blocks, so
// a warp's row loads are contiguous), run the block codec in registers,
// write the block's bits into its fixed-rate slot [b*maxbits, (b+1)*maxbits).
// Decode: the inverse, reading the slot and storing the valid values.
//
// Shared memory per CTA: each thread's plane store (the coder walks planes in
// a rolled loop), and, when every block fills whole 64-bit words ("staged"
// mode, maxbits % 64 == 0), a word buffer: the decoder's warp loads its 32
// consecutive stream slots into it with coalesced loads, and the encoder's
// warp assembles its slots there and stores them with coalesced stores.
//
// Replaces cuZFP's cudaEncode / cudaEncode1 / cudaEncode2 and cudaDecode /
// cudaDecode1 / cudaDecode2 (src/cuZFP/encode{1,2,3}.cuh, decode{1,2,3}.cuh).
#pragma once

#include <cuda_runtime.h>

#include "gzfp_array.cuh"

namespace gzfp {

constexpr int kThreads = 128;            // threads (= blocks) per CTA
constexpr int kStride = kThreads + 1;    // staged word buffer row pitch (words)
constexpr uint32_t kMaxStagedWords = 64; // staged decode up to 4096-bit blocks
constexpr uint32_t kMaxStagedOut = 16;   // staged encoder output up to 1024-bit blocks
constexpr uint32_t kPadRows = 2;         // zero rows after each staged slot
// dynamic shared memory of a CTA: the plane store (up to 32 slots of 8
// bytes per thread) and, when staged, the word buffer
inline size_t smem_bytes(int slots, bool staged, uint32_t words_per_block, int tables = 0) {
  size_t b = ((size_t)slots * kThreads + (size_t)tables) * 8;
  if (staged) b += (size_t)(words_per_block + kPadRows) * kStride * 8;
  return b;
}

// per-thread plane store in shared memory, slot i at planes[i * kThreads];
// t4: the CTA's copy of the 4-value plane tables (1D kernels only)
struct SmemPlanes {
  uint64_t* p;
  const Plane4Tables* t4;
  __device__ __forceinline__ uint64_t get(int i) const { return p[i * kThreads]; }
  __device__ __forceinline__ void put(int i, uint64_t v) { p[i * kThreads] = v; }
};

// 4-value blocks code through the plane tables, which each CTA copies into
// the start of its shared memory (7.5 KB); other blocks use none.
template <int D>
__host__ __device__ constexpr int table_words() {
  return D == 1 ? (int)(sizeof(Plane4Tables) / 8) : 0;
}

// Copy the plane tables into shared memory and return them (null for
// D > 1).  Every thread of the CTA must call it before any thread returns.
template <int D, int NT>
__device__ __forceinline__ const Plane4Tables* stage_tables(uint64_t* smem) {
  if constexpr (D != 1) {
    return nullptr;
  } else {
    const uint64_t* src = reinterpret_cast<const uint64_t*>(&kPlane4Tables);
    for (int i = threadIdx.x; i < table_words<1>(); i += NT) smem[i] = src[i];
    __syncthreads();
    return reinterpret_cast<const Plane4Tables*>(smem);
  }
}

// Global stream words.  `merge` ORs a word that neighbouring zfp blocks share
// (only when maxbits is not a multiple of 64; the stream is zeroed first).
struct DevWords {
  uint64_t* out;
  const uint64_t* in;
  uint64_t n;  // words in the stream
  __device__ __forceinline__ void store(uint64_t i, uint64_t v) { out[i] = v; }
  __device__ __forceinline__ void merge(uint64_t i, uint64_t v) {
    atomicOr((unsigned long long*)(out + i), (unsigned long long)v);
  }
  __device__ __forceinline__ uint64_t load(uint64_t i) const { return i < n ? __ldg(in + i) : 0; }
};

// One block's slot in the staged word buffer: word j of the block at
// buf[j * PITCH] (PITCH = threads per CTA + 1, so the 32 lanes of a warp
// hit 32 different banks); words past the slot read as zero.  The buffer has
// two zero rows after the last word of every slot (kPadRows), so a reader
// may load the two words at any bit position up to the slot's end.
template <int PITCH>
struct StagedWords {
  uint64_t* buf;
  uint64_t w0;  // global index of the slot's first word
  uint32_t W;   // words per block
  __device__ __forceinline__ void store(uint64_t i, uint64_t v) { buf[(i - w0) * PITCH] = v; }
  __device__ __forceinline__ void merge(uint64_t i, uint64_t v) { buf[(i - w0) * PITCH] |= v; }
  __device__ __forceinline__ uint64_t load(uint64_t i) const {
    uint64_t j = i - w0;
    return j < W ? buf[j * PITCH] : 0;
  }
};

// Bit reader over a staged slot: only the bit position is kept, and a peek
// loads the two words it spans (the zero rows after the slot cover the end).
template <int PITCH>
struct BitReader<StagedWords<PITCH>> {
  const uint64_t* buf;
  uint32_t pos;  // bit position within the slot
  __device__ __forceinline__ BitReader(StagedWords<PITCH> w, uint64_t p)
      : buf(w.buf), pos((uint32_t)(p - (w.w0 << 6))) {}
  __device__ __forceinline__ uint64_t peek64() const {
    const uint32_t j = pos >> 6, s = pos & 63;
    const uint64_t a = buf[j * PITCH], b = buf[(j + 1) * PITCH];
    const uint32_t a0 = lo32(a), a1 = hi32(a), b0 = lo32(b), b1 = hi32(b);
    const bool ge = s >= 32;
    const uint32_t c0 = ge ? a1 : a0, c1 = ge ? b0 : a1, c2 = ge ? b1 : b0;
    const uint32_t t = s & 31;
    return ((uint64_t)__funnelshift_r(c1, c2, t) << 32) | __funnelshift_r(c0, c1, t);
  }
  __device__ __forceinline__ void skip(uint32_t n) { pos += n; }
  __device__ __forceinline__ uint64_t read(uint32_t n) {
    if (n == 0) return 0;
    const uint64_t v = peek64() & lowmask64(n);
    pos += n;
    return v;
  }
};

// Copy a warp's 32 consecutive slots between the staged buffer (word j of
// lane t at buf[j * PITCH + t]) and the stream, 32 words per step.
template <bool TO_GLOBAL, int PITCH = kStride>
__device__ __forceinline__ void warp_copy(uint64_t* buf, uint64_t* gwords, uint32_t W,
                                          uint32_t nblocks_valid) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t total = nblocks_valid * W;
  uint32_t t = lane / W, j = lane % W;      // slot and word of element `lane`
  const uint32_t dt = 32 / W, dj = 32 % W;  // advance per step of 32 elements
  for (uint32_t gi = lane; gi < total; gi += 32) {
    if (TO_GLOBAL)
      gwords[gi] = buf[j * PITCH + t];
    else
      buf[j * PITCH + t] = __ldg(gwords + gi);
    t += dt;
    j += dj;
    if (j >= W) {
      j -= W;
      t++;
    }
  }
}

// Register budget: the 4^3 double kernels keep a whole block (64 x 64 bits)
// in registers; 168 registers per thread allow 3 CTAs of 128 threads per SM.
template <int D, typename T>
struct MinBlocks {
  static constexpr int value = (D == 3 && sizeof(T) == 8) ? 3 : 4;
};

// Plane-store slots per thread, as many as the block codec touches, so that
// shared memory does not cap the CTAs per SM below what registers allow:
// 4^3 blocks code and decode 32 planes at a time (32 slots; 64-bit values
// go through two 32-plane halves); 2D blocks hold their transposed words
// (16 per 32 bits of value); 1D blocks keep their planes in registers (none).
template <int D, typename T>
__host__ __device__ constexpr int store_slots() {
  return D == 1 ? 0 : D == 2 ? 16 * (int)(sizeof(T) / 4) : 32;
}
template <int D, typename T>
__host__ __device__ constexpr int decode_slots() {
  return D == 3 ? 32 : store_slots<D, T>();
}

// ALIGNED: every block fills whole words (maxbits % 64 == 0, no header
// offset); its words are then assembled in the staged buffer and the warp
// stores its 32 consecutive slots with coalesced stores.
template <int D, typename T, bool ALIGNED = false>
__global__ void __launch_bounds__(kThreads, (MinBlocks<D, T>::value))
    encode_kernel(const T* __restrict__ in, Geom g, uint32_t maxbits, uint64_t* __restrict__ out,
                  uint64_t nwords) {
  extern __shared__ uint64_t smem[];
  const Plane4Tables* t4 = stage_tables<D, kThreads>(smem);
  SmemPlanes ps{smem + table_words<D>() + threadIdx.x, t4};
  const uint64_t b = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if constexpr (ALIGNED) {
    const uint32_t W = maxbits >> 6;
    uint64_t* buf = smem + table_words<D>() + store_slots<D, T>() * kThreads;
    if (b < g.nblocks)
      encode_one<D, T, true>(in, g, b, maxbits, StagedWords<kStride>{buf + threadIdx.x, b * W, W}, ps);
    __syncwarp();
    const uint64_t b0 = b - (threadIdx.x & 31);
    if (b0 < g.nblocks) {
      const uint64_t left = g.nblocks - b0;
      warp_copy<true>(buf + (threadIdx.x & ~31u), out + b0 * W, W, left < 32 ? (uint32_t)left : 32);
    }
  } else {
    if (b < g.nblocks)
      encode_one<D, T>(in, g, b, maxbits, DevWords{out, nullptr, nwords}, ps);
  }
}

// MINB: resident CTAs per SM the register budget is sized for.  The decoder
// is latency-bound on its plane chain, so a fourth CTA is worth a tighter
// register budget whenever shared memory allows one (dec_min_blocks).
template <int D, typename T, bool STAGED, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
    decode_kernel(const uint64_t* __restrict__ in, uint64_t nwords, Geom g, uint32_t maxbits,
                  T* __restrict__ out) {
  extern __shared__ uint64_t smem[];
  const Plane4Tables* t4 = stage_tables<D, kThreads>(smem);
  SmemPlanes ps{smem + table_words<D>() + threadIdx.x, t4};
  const uint64_t b = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (STAGED) {
    const uint32_t W = maxbits >> 6;
    uint64_t* buf = smem + table_words<D>() + decode_slots<D, T>() * kThreads;
    const uint64_t b0 = b - (threadIdx.x & 31);
    if (b0 < g.nblocks) {
      const uint64_t left = g.nblocks - b0;
      warp_copy<false>(buf + (threadIdx.x & ~31u), (uint64_t*)in + b0 * W, W,
                       left < 32 ? (uint32_t)left : 32);
    }
#pragma unroll
    for (uint32_t j = 0; j < kPadRows; j++) buf[(W + j) * kStride + threadIdx.x] = 0;
    __syncwarp();
    if (b < g.nblocks)
      decode_one<D, T>(out, g, b, maxbits, StagedWords<kStride>{buf + threadIdx.x, b * W, W}, ps);
  } else {
    if (b < g.nblocks) decode_one<D, T>(out, g, b, maxbits, DevWords{nullptr, in, nwords}, ps);
  }
}

// kernel launchers shared by the per-type translation units
template <int D, typename T>
cudaError_t launch_encode_t(const T* in, const Geom& g, uint32_t maxbits, uint64_t* out,
                            uint64_t nwords, cudaStream_t s) {
  if (g.nblocks == 0) return cudaSuccess;
  const dim3 grid((unsigned)((g.nblocks + kThreads - 1) / kThreads));
  // staged output for blocks of up to kMaxStagedOut words, when they fit
  // beside the plane store without costing a resident CTA (larger blocks
  // measured faster with direct stores)
  constexpr int MB = MinBlocks<D, T>::value;
  const bool aligned =
      maxbits % 64 == 0 && g.base == 0 && (maxbits >> 6) <= kMaxStagedOut &&
      (smem_bytes(store_slots<D, T>(), true, maxbits >> 6, table_words<D>()) + 1024) * MB <=
          227 * 1024;
  const size_t sm = smem_bytes(store_slots<D, T>(), aligned, maxbits >> 6, table_words<D>());
  auto k = aligned ? encode_kernel<D, T, true> : encode_kernel<D, T>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<grid, kThreads, sm, s>>>(in, g, maxbits, out, nwords);
  return cudaGetLastError();
}

// Shared memory of a staged decode CTA that still lets 4 CTAs share an SM
// (228 KB per SM, 1 KB reserved per CTA).
constexpr size_t kSmemFor4 = 56 * 1024;

template <int D, typename T>
cudaError_t launch_decode_t(const uint64_t* in, uint64_t nwords, const Geom& g, uint32_t maxbits,
                            T* out, cudaStream_t s) {
  if (g.nblocks == 0) return cudaSuccess;
  const dim3 grid((unsigned)((g.nblocks + kThreads - 1) / kThreads));
  const bool staged = maxbits % 64 == 0 && (maxbits >> 6) <= kMaxStagedWords && g.base == 0;
  const size_t sm = smem_bytes(decode_slots<D, T>(), staged, maxbits >> 6, table_words<D>());
  constexpr int MB = MinBlocks<D, T>::value;
  auto k = !staged ? decode_kernel<D, T, false, MB>
           : (MB < 4 && sm <= kSmemFor4) ? decode_kernel<D, T, true, 4>
                                         : decode_kernel<D, T, true, MB>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<grid, kThreads, sm, s>>>(in, nwords, g, maxbits, out);
  return cudaGetLastError();
}

}  // namespace gzfp
