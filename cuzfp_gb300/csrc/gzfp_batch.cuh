// gzfp_batch.cuh -- the batched persistent kernel: many arrays of uneven
// shape, scalar type, dimensionality and rate coded by one launch.
//
// Work list (device memory, built per batch): one descriptor per array and a
// table mapping every chunk -- NT * BPT consecutive zfp blocks of one array
// -- to its array.  A grid of resident CTAs claims chunks from a global
// counter (atomicAdd), optionally one claim ahead so that the claim's
// latency overlaps the current chunk, and codes each block of the chunk
// with the plain path's per-thread code.  Every block's bits are the same
// as a plain launch on that array would produce.
#pragma once

#include "gzfp_kernels.cuh"

namespace gzfp {

// one array of a batch
struct BatchDesc {
  const void* in;        // encode: field; decode: stream words
  void* out;             // encode: stream words; decode: field
  Geom g;
  uint64_t nwords;       // stream words
  uint64_t first_chunk;  // index of the array's first chunk in the batch
  uint32_t maxbits;
  uint32_t kind;         // dims | (8 for double)
};

constexpr uint32_t kKindDouble = 8;

template <int NT>
struct BatchPlanes {
  uint64_t* p;
  __device__ __forceinline__ uint64_t get(int i) const { return p[i * NT]; }
  __device__ __forceinline__ void put(int i, uint64_t v) { p[i * NT] = v; }
};

template <int NT, bool DECODE>
__device__ __forceinline__ void batch_block(const BatchDesc& d, uint64_t b, BatchPlanes<NT>& ps,
                                            const Ctx& c) {
  if (b >= d.g.nblocks) return;
  if (DECODE) {
    const DevWords words{nullptr, (const uint64_t*)d.in, d.nwords};
    switch (d.kind) {
      case 1: decode_one<1, float>((float*)d.out, d.g, b, d.maxbits, words, ps, c); break;
      case 2: decode_one<2, float>((float*)d.out, d.g, b, d.maxbits, words, ps, c); break;
      case 3: decode_one<3, float>((float*)d.out, d.g, b, d.maxbits, words, ps, c); break;
      case 9: decode_one<1, double>((double*)d.out, d.g, b, d.maxbits, words, ps, c); break;
      case 10: decode_one<2, double>((double*)d.out, d.g, b, d.maxbits, words, ps, c); break;
      case 11: decode_one<3, double>((double*)d.out, d.g, b, d.maxbits, words, ps, c); break;
      default: break;
    }
  } else {
    const DevWords words{(uint64_t*)d.out, nullptr, d.nwords};
    switch (d.kind) {
      case 1: encode_one<1, float>((const float*)d.in, d.g, b, d.maxbits, words, ps, c); break;
      case 2: encode_one<2, float>((const float*)d.in, d.g, b, d.maxbits, words, ps, c); break;
      case 3: encode_one<3, float>((const float*)d.in, d.g, b, d.maxbits, words, ps, c); break;
      case 9: encode_one<1, double>((const double*)d.in, d.g, b, d.maxbits, words, ps, c); break;
      case 10: encode_one<2, double>((const double*)d.in, d.g, b, d.maxbits, words, ps, c); break;
      case 11: encode_one<3, double>((const double*)d.in, d.g, b, d.maxbits, words, ps, c); break;
      default: break;
    }
  }
}

// Persistent batch kernel.  NT threads per CTA, bpt blocks per thread per
// chunk.  With `ahead` the next chunk is claimed as soon as the current one
// is known, so the claim's latency overlaps the coding; otherwise after it.
// `counter` must be zero at launch.
template <int NT, bool DECODE>
__global__ void __launch_bounds__(NT, (NT == 64 ? 6 : NT == 128 ? 3 : 1))
    batch_kernel(const BatchDesc* __restrict__ descs, const uint32_t* __restrict__ chunk_item,
                 uint64_t nchunks, unsigned long long* counter, int bpt, int ahead, Ctx c) {
  extern __shared__ uint64_t smem[];
  __shared__ unsigned long long s_claim;
  BatchPlanes<NT> ps{smem + threadIdx.x};
  if (threadIdx.x == 0) s_claim = atomicAdd(counter, 1ull);
  __syncthreads();
  for (;;) {
    const unsigned long long chunk = s_claim;
    if (chunk >= nchunks) break;
    const BatchDesc d = descs[chunk_item[chunk]];
    __syncthreads();  // every thread has read the claim
    if (ahead && threadIdx.x == 0) s_claim = atomicAdd(counter, 1ull);
    const uint64_t first = (chunk - d.first_chunk) * (uint64_t)(NT * bpt);
#pragma unroll 1
    for (int j = 0; j < bpt; j++) batch_block<NT, DECODE>(d, first + (uint64_t)j * NT + threadIdx.x, ps, c);
    if (!ahead && threadIdx.x == 0) s_claim = atomicAdd(counter, 1ull);
    __syncthreads();  // the next claim is visible
  }
}

// shared memory of a batch CTA: 64 plane-store slots per thread
constexpr size_t batch_smem_bytes(int nt) { return (size_t)nt * 64 * 8; }

template <int NT>
cudaError_t launch_batch_t(bool decode, int grid, int bpt, bool ahead, const BatchDesc* descs,
                           const uint32_t* chunk_item, uint64_t nchunks,
                           unsigned long long* counter, cudaStream_t s) {
  const Ctx c{1u, 0xffffffffu};
  const size_t sm = batch_smem_bytes(NT);
  auto k = decode ? batch_kernel<NT, true> : batch_kernel<NT, false>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<grid, NT, sm, s>>>(descs, chunk_item, nchunks, counter, bpt, ahead ? 1 : 0, c);
  return cudaGetLastError();
}

template <int NT>
int batch_occupancy(bool decode) {
  int n = 0;
  auto k = decode ? batch_kernel<NT, true> : batch_kernel<NT, false>;
  const size_t sm = batch_smem_bytes(NT);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NT, sm) != cudaSuccess) return 0;
  return n;
}

}  // namespace gzfp
