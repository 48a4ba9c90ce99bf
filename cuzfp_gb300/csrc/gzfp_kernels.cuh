// gzfp_kernels.cuh -- the plain-path CUDA kernels: one thread per zfp block.
//
// Encode: gather 4^D values (coalesced across the warp: consecutive threads
// own consecutive blocks along x), run the block codec in registers and
// write the block's bits into its fixed-rate slot [b*maxbits, (b+1)*maxbits).
// Decode: the inverse, reading the slot and storing the valid values.
//
// Replaces cuZFP's cudaEncode / cudaEncode1 / cudaEncode2 and cudaDecode /
// cudaDecode1 / cudaDecode2 (src/cuZFP/encode{1,2,3}.cuh, decode{1,2,3}.cuh).
#pragma once

#include <cuda_runtime.h>

#include "gzfp_array.cuh"

namespace gzfp {

constexpr int kThreads = 128;  // threads (= blocks) per CTA

// Stream word access for the writer / reader.  `merge` ORs a word that two
// neighbouring zfp blocks share (only when maxbits is not a multiple of 64;
// the stream is zeroed first in that case).
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

template <int D, typename T>
__global__ void __launch_bounds__(kThreads) encode_kernel(const T* __restrict__ in, Geom g,
                                                          uint32_t maxbits,
                                                          uint64_t* __restrict__ out,
                                                          uint64_t nwords) {
  const uint64_t b = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (b >= g.nblocks) return;
  encode_one<D, T>(in, g, b, maxbits, DevWords{out, nullptr, nwords});
}

template <int D, typename T>
__global__ void __launch_bounds__(kThreads) decode_kernel(const uint64_t* __restrict__ in,
                                                          uint64_t nwords, Geom g,
                                                          uint32_t maxbits, T* __restrict__ out) {
  const uint64_t b = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (b >= g.nblocks) return;
  decode_one<D, T>(out, g, b, maxbits, DevWords{nullptr, in, nwords});
}

}  // namespace gzfp
