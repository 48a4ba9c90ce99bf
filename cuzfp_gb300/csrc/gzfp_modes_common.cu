// Type-independent kernels of the general coding modes: the scan of block
// lengths into start bits and the placement of every block at its start.
#include "gzfp_launch.h"
#include "gzfp_modes.cuh"

namespace gzfp {

// Step 2: exclusive scan of the lengths into 64-bit start bits, in three
// kernels with no waiting between CTAs: per-chunk sums, a scan of the sums
// by one CTA, then a scan inside every chunk.
constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;                             // lengths per thread
constexpr int kScanChunk = kScanThreads * kScanPer;      // lengths per CTA

// inclusive scan of one value per thread across the CTA; returns the CTA total
__device__ __forceinline__ uint64_t cta_inclusive_scan(uint64_t& v, uint64_t* warp_sums) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) warp_sums[warp] = v;
  __syncthreads();
  if (warp == 0) {
    uint64_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const uint64_t total = warp_sums[kScanThreads / 32 - 1];
  if (warp > 0) v += warp_sums[warp - 1];
  __syncthreads();  // warp_sums may be reused
  return total;
}

__global__ void __launch_bounds__(kScanThreads)
    scan_chunk_sums(const uint32_t* __restrict__ lengths, uint64_t n, uint64_t* __restrict__ sums) {
  __shared__ uint64_t ws[kScanThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk;
  uint64_t v = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; j++) {
    const uint64_t i = base + (uint64_t)j * kScanThreads + threadIdx.x;
    if (i < n) v += lengths[i];
  }
  const uint64_t total = cta_inclusive_scan(v, ws);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// sums[0..m) -> their exclusive scan, in place; sums[m] = the grand total
__global__ void __launch_bounds__(kScanThreads) scan_sums(uint64_t* sums, uint64_t m) {
  __shared__ uint64_t ws[kScanThreads / 32];
  uint64_t carry = 0;
  for (uint64_t base = 0; base < m; base += kScanThreads) {
    const uint64_t i = base + threadIdx.x;
    const uint64_t x = i < m ? sums[i] : 0;
    uint64_t v = x;
    const uint64_t total = cta_inclusive_scan(v, ws);
    if (i < m) sums[i] = carry + v - x;
    carry += total;
  }
  if (threadIdx.x == 0) sums[m] = carry;
}

__global__ void __launch_bounds__(kScanThreads)
    scan_chunks(const uint32_t* __restrict__ lengths, uint64_t n, uint64_t first,
                const uint64_t* __restrict__ sums, uint64_t* __restrict__ offsets) {
  __shared__ uint64_t ws[kScanThreads / 32];
  // thread t scans its kScanPer consecutive lengths; the CTA scans the
  // threads' totals
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + (uint64_t)threadIdx.x * kScanPer;
  uint32_t len[kScanPer];
  uint64_t v = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; j++) {
    len[j] = base + j < n ? lengths[base + j] : 0;
    v += len[j];
  }
  const uint64_t mine = v;
  cta_inclusive_scan(v, ws);
  uint64_t pos = first + sums[blockIdx.x] + v - mine;
#pragma unroll
  for (int j = 0; j < kScanPer; j++) {
    if (base + j < n) offsets[base + j] = pos;
    pos += len[j];
  }
}

// Step 3: the len bits of slot b to stream bit offsets[b].  The stream is
// zeroed first; the words a block shares with its neighbours are merged
// with atomicOr, the others stored.
__global__ void __launch_bounds__(kThreads)
    place_blocks(const uint64_t* __restrict__ scratch, uint32_t slot_words,
                 const uint32_t* __restrict__ lengths, const uint64_t* __restrict__ offsets,
                 uint64_t nblocks, uint64_t* __restrict__ out) {
  const uint64_t b = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (b >= nblocks) return;
  const uint32_t len = lengths[b];
  if (len == 0) return;  // every block takes at least one bit; nothing to place
  const uint64_t pos = offsets[b], end = pos + len;
  const uint64_t* src = scratch + b * slot_words;
  const uint32_t sh = (uint32_t)(pos & 63);
  const uint32_t nsrc = (len + 63) >> 6;  // source words holding the block
  const uint64_t w0 = pos >> 6, w1 = (end - 1) >> 6;
  uint64_t prev = 0;
  for (uint64_t wi = w0; wi <= w1; wi++) {
    const uint32_t j = (uint32_t)(wi - w0);
    const uint64_t cur = j < nsrc ? src[j] : 0;
    const uint64_t v = sh ? (cur << sh) | (prev >> (64 - sh)) : cur;
    prev = cur;
    const bool shared = (wi == w0 && sh) || (wi == w1 && (end & 63));
    if (shared)
      atomicOr((unsigned long long*)(out + wi), (unsigned long long)v);
    else
      out[wi] = v;
  }
}

uint32_t block_bound_host(int dims, int P, int ebits, const General& mode) {
  return block_bound(dims, P, ebits, mode);
}

uint64_t scan_sums_count(uint64_t n) { return (n + kScanChunk - 1) / kScanChunk; }

cudaError_t launch_scan_lengths(const uint32_t* lengths, uint64_t n, uint64_t first,
                                uint64_t* sums, unsigned long long* offsets, cudaStream_t s) {
  const uint64_t m = scan_sums_count(n);
  if (m == 0) return cudaMemsetAsync(sums, 0, sizeof(uint64_t), s);
  scan_chunk_sums<<<(unsigned)m, kScanThreads, 0, s>>>(lengths, n, sums);
  scan_sums<<<1, kScanThreads, 0, s>>>(sums, m);
  scan_chunks<<<(unsigned)m, kScanThreads, 0, s>>>(lengths, n, first, sums, (uint64_t*)offsets);
  return cudaGetLastError();
}

cudaError_t launch_place_blocks(const uint64_t* scratch, uint32_t slot_words,
                                const uint32_t* lengths, const unsigned long long* offsets,
                                uint64_t nblocks, uint64_t* out, cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  place_blocks<<<(unsigned)((nblocks + kThreads - 1) / kThreads), kThreads, 0, s>>>(
      scratch, slot_words, lengths, (const uint64_t*)offsets, nblocks, out);
  return cudaGetLastError();
}

__global__ void fill_fixed_offsets(unsigned long long* offsets, uint64_t n, uint64_t first,
                                   uint32_t maxbits) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b < n) offsets[b] = first + b * maxbits;
}

cudaError_t launch_fixed_offsets(unsigned long long* offsets, uint64_t n, uint64_t first,
                                 uint32_t maxbits, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  fill_fixed_offsets<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(offsets, n, first, maxbits);
  return cudaGetLastError();
}

}  // namespace gzfp
