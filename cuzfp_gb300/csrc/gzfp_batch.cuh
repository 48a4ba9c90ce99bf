// gzfp_batch.cuh -- the batched persistent kernels: many arrays of uneven
// shape, scalar type, dimensionality and rate coded by a few launches.
//
// Work list (device memory, built per batch): one descriptor per array,
// grouped by kind (dimensionality x scalar type: float, double, int32,
// int64), and a table mapping every
// chunk -- NT * BPT consecutive zfp blocks of one array -- to its array.
// The chunks of one kind form one contiguous range.  Each kind present in
// the batch gets one persistent kernel specialised for it (so its register
// budget is the plain kernel's, not the union of all kinds): a grid of
// resident CTAs claims chunks of its range from the kind's counter
// (atomicAdd), optionally one claim ahead so that the claim's latency
// overlaps the current chunk, and codes each block with the plain path's
// per-thread code.  Every block's bits are the same as a plain launch on
// that array would produce.
#pragma once

#include <type_traits>

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
  uint32_t kind;         // batch_kind(type, dims), gzfp_batch_launch.h
};

// An array's kind: dims | 8 * (0 float, 1 double, 2 int32, 3 int64).  The
// first six kinds (floating point) and the last six (integer) are compiled
// in separate translation units.
constexpr int kBatchKinds = 12;
constexpr int kBatchFloatKinds = 6;
constexpr uint32_t kBatchKind[kBatchKinds] = {1, 2, 3, 9, 10, 11, 17, 18, 19, 25, 26, 27};

inline int batch_kind_index(uint32_t kind) {
  for (int i = 0; i < kBatchKinds; i++)
    if (kBatchKind[i] == kind) return i;
  return -1;
}

template <int NT>
struct BatchPlanes {
  uint64_t* p;
  const Plane4Tables* t4;  // the CTA's plane tables (1D kinds)
  __device__ __forceinline__ uint64_t get(int i) const { return p[i * NT]; }
  __device__ __forceinline__ void put(int i, uint64_t v) { p[i * NT] = v; }
};

// Blocks of whole 64-bit words, up to this many per block, are decoded from
// a shared-memory copy of the warp's 32 slots made with coalesced loads (as
// the plain decoder does); others read the stream directly.  Encoding
// assembles blocks of whole words, up to kMaxStagedOut per block, in the
// same buffer and the warp stores its 32 slots with coalesced stores (as
// the plain encoder does).
constexpr uint32_t kBatchMaxStagedWords = 32;

// Staging rows an item asks for (0: none).
GZ_HD uint32_t batch_item_staged_w(bool decode, uint32_t maxbits) {
  const uint32_t w = maxbits / 64;
  return maxbits % 64 == 0 && w <= (decode ? kBatchMaxStagedWords : kMaxStagedOut) ? w : 0;
}

// Which path a kernel compiles: kPathDirect (stream words read or written
// in place), kPathStaged (every item it codes is staged: the caller
// guarantees batch_item_staged_w(DECODE, maxbits) != 0 and <= staged_w), or
// kPathEither (decided per item).  A kernel with one path spills less.
constexpr int kPathDirect = 0, kPathStaged = 1, kPathEither = 2;

template <int NT, bool DECODE, int D, typename T, int PATH = kPathEither>
__device__ __forceinline__ void batch_block(const BatchDesc& d, uint64_t b, BatchPlanes<NT>& ps,
                                            uint64_t* sbuf, uint32_t staged_w) {
  if (DECODE) {
    const uint32_t W = d.maxbits >> 6;
    if (PATH == kPathStaged ||
        (PATH == kPathEither && d.maxbits % 64 == 0 && W <= staged_w)) {  // the whole warp (one item)
      const uint32_t lane = threadIdx.x & 31;
      const uint64_t b0 = b - lane;
      if (b0 < d.g.nblocks) {
        const uint64_t left = d.g.nblocks - b0;
        warp_copy<false, NT + 1>(sbuf + (threadIdx.x & ~31u), (uint64_t*)d.in + b0 * W, W,
                                 left < 32 ? (uint32_t)left : 32);
      }
      // zero rows after the slot: the staged bit reader loads two words
#pragma unroll
      for (uint32_t j = 0; j < kPadRows; j++) sbuf[(W + j) * (NT + 1) + threadIdx.x] = 0;
      __syncwarp();
      if (b < d.g.nblocks)
        decode_one<D, T>((T*)d.out, d.g, b, d.maxbits,
                         StagedWords<NT + 1>{sbuf + threadIdx.x, b * W, W}, ps);
      __syncwarp();  // the next chunk's copy reuses the buffer
      return;
    }
    if (b >= d.g.nblocks) return;
    decode_one<D, T>((T*)d.out, d.g, b, d.maxbits,
                     DevWords{nullptr, (const uint64_t*)d.in, d.nwords}, ps);
  } else {
    const uint32_t W = d.maxbits >> 6;
    if (PATH == kPathStaged ||
        (PATH == kPathEither && d.maxbits % 64 == 0 && W <= staged_w && W <= kMaxStagedOut)) {
      if (b < d.g.nblocks)
        encode_one<D, T, true>((const T*)d.in, d.g, b, d.maxbits,
                               StagedWords<NT + 1>{sbuf + threadIdx.x, b * W, W}, ps);
      __syncwarp();
      const uint64_t b0 = b - (threadIdx.x & 31);
      if (b0 < d.g.nblocks) {
        const uint64_t left = d.g.nblocks - b0;
        warp_copy<true, NT + 1>(sbuf + (threadIdx.x & ~31u), (uint64_t*)d.out + b0 * W, W,
                                left < 32 ? (uint32_t)left : 32);
      }
      __syncwarp();  // the next chunk's blocks reuse the buffer
      return;
    }
    if (b >= d.g.nblocks) return;
    encode_one<D, T>((const T*)d.in, d.g, b, d.maxbits,
                     DevWords{(uint64_t*)d.out, nullptr, d.nwords}, ps);
  }
}

// Resident CTAs per SM each kernel's registers are sized for: the plain
// kernels' choice at 128 threads, scaled to the CTA size.
template <int NT, int D, typename T>
struct BatchMinBlocks {
  static constexpr int v = MinBlocks<D, T>::value * 128 / NT;
  static constexpr int value = v < 1 ? 1 : v;
};

// plane-store slots per thread: as the plain kernels
template <bool DECODE, int D, typename T>
struct BatchSlots {
  static constexpr int value = DECODE ? decode_slots<D, T>() : store_slots<D, T>();
};

// The 4^3 64-bit decoder is latency-bound on its plane chain: like the plain
// decoder it gets a tighter register budget for a fourth CTA of 128 threads
// per SM whenever shared memory allows one.
template <int NT, bool DECODE, int D, typename T>
struct BatchMinBlocksWide {
  static constexpr int value =
      DECODE && D == 3 && sizeof(T) == 8 ? 4 * 128 / NT : BatchMinBlocks<NT, D, T>::value;
};

// Grid kernel for one kind: CTA i codes slice i % bpt (NT blocks, one per
// thread) of chunk lo + i / bpt, so the hardware's CTA scheduler spreads the
// kind's chunks over the SMs and no thread loops over blocks.  The block
// code then compiles as in the plain kernels: under a loop, the 4^3 64-bit
// coders spill several hundred bytes per thread at the same register
// budget.  PATH is kPathStaged (every item of [lo, ...) stages, in up to
// staged_w words per block, in shared memory behind the plane store) or
// kPathDirect.
template <int NT, bool DECODE, int D, typename T, int MINB, int PATH>
__global__ void __launch_bounds__(NT, MINB)
    batch_grid_kernel(const BatchDesc* __restrict__ descs,
                      const uint32_t* __restrict__ chunk_item, uint64_t lo, int bpt,
                      uint32_t staged_w) {
  extern __shared__ uint64_t smem[];
  __shared__ BatchDesc s_desc;
  const Plane4Tables* t4 = stage_tables<D, NT>(smem);
  BatchPlanes<NT> ps{smem + table_words<D>() + threadIdx.x, t4};
  uint64_t* sbuf = smem + table_words<D>() + BatchSlots<DECODE, D, T>::value * NT;
  const uint32_t j = blockIdx.x % (uint32_t)bpt;
  const uint64_t chunk = lo + blockIdx.x / (uint32_t)bpt;
  if (threadIdx.x == 0) s_desc = descs[chunk_item[chunk]];
  __syncthreads();
  const BatchDesc& d = s_desc;
  const uint64_t first = (chunk - d.first_chunk) * (uint64_t)(NT * bpt) + (uint64_t)j * NT;
  batch_block<NT, DECODE, D, T, PATH>(d, first + threadIdx.x, ps, sbuf, staged_w);
}

// Persistent kernel for one kind: chunks [lo, hi) of the work list.  NT
// threads per CTA, bpt blocks per thread per chunk, register budget for
// MINB resident CTAs per SM.  `counter` must be zero at launch.  Items of
// up to staged_w words per block are staged in shared memory behind the
// plane store.
template <int NT, bool DECODE, int D, typename T, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    batch_kernel(const BatchDesc* __restrict__ descs, const uint32_t* __restrict__ chunk_item,
                 uint64_t lo, uint64_t hi, unsigned long long* counter, int bpt, int ahead,
                 uint32_t staged_w) {
  extern __shared__ uint64_t smem[];
  __shared__ unsigned long long s_claim;
  __shared__ BatchDesc s_desc;  // the claimed chunk's array, read field by field
  const Plane4Tables* t4 = stage_tables<D, NT>(smem);
  BatchPlanes<NT> ps{smem + table_words<D>() + threadIdx.x, t4};
  uint64_t* sbuf = smem + table_words<D>() + BatchSlots<DECODE, D, T>::value * NT;
  if (threadIdx.x == 0) s_claim = lo + atomicAdd(counter, 1ull);
  __syncthreads();
  for (;;) {
    const unsigned long long chunk = s_claim;
    if (chunk >= hi) break;
    if (threadIdx.x == 0) s_desc = descs[chunk_item[chunk]];
    __syncthreads();  // every thread has read the claim and sees the descriptor
    const BatchDesc& d = s_desc;
    if (ahead && threadIdx.x == 0) s_claim = lo + atomicAdd(counter, 1ull);
    const uint64_t first = (chunk - d.first_chunk) * (uint64_t)(NT * bpt);
#pragma unroll 1
    for (int j = 0; j < bpt; j++)
      batch_block<NT, DECODE, D, T>(d, first + (uint64_t)j * NT + threadIdx.x, ps, sbuf,
                                    staged_w);
    __syncthreads();  // every thread is done with the descriptor
    if (!ahead && threadIdx.x == 0) s_claim = lo + atomicAdd(counter, 1ull);
    __syncthreads();  // the next claim is visible
  }
}

// shared memory of a batch CTA of one kind: the plane store, and the staged
// word buffer (staged_w words per block and the zero rows after them, at
// pitch NT + 1)
template <int NT, bool DECODE, int D, typename T>
GZ_HD size_t batch_smem_bytes(uint32_t staged_w) {
  return ((size_t)NT * BatchSlots<DECODE, D, T>::value + (size_t)table_words<D>()) * 8 +
         (staged_w ? (size_t)(staged_w + kPadRows) * (NT + 1) * 8 : 0);
}

// CTAs of `sm` bytes of shared memory that fit one SM (228 KB, 1 KB
// reserved per CTA)
GZ_HD bool batch_smem_fits(size_t sm, int ctas) { return (sm + 1024) * ctas <= 228 * 1024; }

// The launch of one kind: the kernels (register budget, path) and the
// staging depth they run with.  Encoding stages output only where the
// buffer costs no resident CTA, as the plain encoder; decoding takes the
// wide budget where shared memory allows its CTAs.  The grid kernel stages
// every item when staged_w > 0 (a range of staged items), none otherwise.
template <int NT, bool DECODE, int D, typename T>
struct BatchLaunch {
  void (*persistent)(const BatchDesc*, const uint32_t*, uint64_t, uint64_t, unsigned long long*,
                     int, int, uint32_t);
  void (*grid)(const BatchDesc*, const uint32_t*, uint64_t, int, uint32_t);
  uint32_t staged_w;
  size_t smem;
  explicit BatchLaunch(uint32_t sw) {
    constexpr int MB = BatchMinBlocks<NT, D, T>::value;
    constexpr int WIDE = BatchMinBlocksWide<NT, DECODE, D, T>::value;
    staged_w = sw;
    if (!DECODE && sw && !batch_smem_fits(batch_smem_bytes<NT, DECODE, D, T>(sw), MB)) staged_w = 0;
    smem = batch_smem_bytes<NT, DECODE, D, T>(staged_w);
    const bool wide = WIDE != MB && batch_smem_fits(smem, WIDE);
    persistent = wide ? batch_kernel<NT, DECODE, D, T, WIDE> : batch_kernel<NT, DECODE, D, T, MB>;
    if (staged_w)
      grid = wide ? batch_grid_kernel<NT, DECODE, D, T, WIDE, kPathStaged>
                  : batch_grid_kernel<NT, DECODE, D, T, MB, kPathStaged>;
    else
      grid = wide ? batch_grid_kernel<NT, DECODE, D, T, WIDE, kPathDirect>
                  : batch_grid_kernel<NT, DECODE, D, T, MB, kPathDirect>;
  }
};

// CTAs of one grid launch at most (the rest go to further launches)
constexpr uint64_t kBatchGridPiece = 1ull << 30;

// grid > 0: the persistent kernel on `grid` CTAs, items staged per item up
// to staged_w words; grid == 0: the grid kernel over every (chunk, slice)
// of [lo, hi), every item staged (staged_w > 0: the caller's range holds
// only items with batch_item_staged_w != 0, each at most staged_w) or none
// (staged_w == 0)
template <int NT, bool DECODE, int D, typename T>
cudaError_t launch_batch_kind(int grid, int bpt, bool ahead, uint32_t staged_w,
                              const BatchDesc* descs, const uint32_t* chunk_item, uint64_t lo,
                              uint64_t hi, unsigned long long* counter, cudaStream_t s) {
  const BatchLaunch<NT, DECODE, D, T> L(staged_w);
  cudaError_t e;
  if (grid > 0) {
    e = cudaFuncSetAttribute(L.persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)L.smem);
    if (e != cudaSuccess) return e;
    L.persistent<<<grid, NT, L.smem, s>>>(descs, chunk_item, lo, hi, counter, bpt,
                                          ahead ? 1 : 0, L.staged_w);
    return cudaGetLastError();
  }
  e = cudaFuncSetAttribute(L.grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
  if (e != cudaSuccess) return e;
  const uint64_t per = kBatchGridPiece / (uint64_t)bpt;  // chunks per launch
  for (uint64_t c = lo; c < hi; c += per) {
    const uint64_t n = hi - c < per ? hi - c : per;
    L.grid<<<(unsigned)(n * (uint64_t)bpt), NT, L.smem, s>>>(descs, chunk_item, c, bpt,
                                                              L.staged_w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// resident CTAs per SM of the persistent kernel
template <int NT, bool DECODE, int D, typename T>
int batch_occupancy_kind(uint32_t staged_w) {
  int n = 0;
  const BatchLaunch<NT, DECODE, D, T> L(staged_w);
  if (cudaFuncSetAttribute(L.persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)L.smem) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, L.persistent, NT, L.smem) != cudaSuccess)
    return 0;
  return n;
}

// Dispatch over the six kinds of one group (INTS: kind indices 6..11, the
// integer kinds; else 0..5).
template <int NT, bool DECODE, bool INTS>
cudaError_t launch_batch_t(int kind_index, int grid, int bpt, bool ahead, uint32_t staged_w,
                           const BatchDesc* descs, const uint32_t* chunk_item, uint64_t lo,
                           uint64_t hi, unsigned long long* counter, cudaStream_t s) {
  typedef typename std::conditional<INTS, int32_t, float>::type T4;
  typedef typename std::conditional<INTS, int64_t, double>::type T8;
#define GZFP_KIND(D, T) \
  launch_batch_kind<NT, DECODE, D, T>(grid, bpt, ahead, staged_w, descs, chunk_item, lo, hi, counter, s)
  switch (kind_index - (INTS ? kBatchFloatKinds : 0)) {
    case 0: return GZFP_KIND(1, T4);
    case 1: return GZFP_KIND(2, T4);
    case 2: return GZFP_KIND(3, T4);
    case 3: return GZFP_KIND(1, T8);
    case 4: return GZFP_KIND(2, T8);
    case 5: return GZFP_KIND(3, T8);
    default: return cudaErrorInvalidValue;
  }
#undef GZFP_KIND
}

template <int NT, bool DECODE, bool INTS>
int batch_occupancy_t(int kind_index, uint32_t staged_w) {
  typedef typename std::conditional<INTS, int32_t, float>::type T4;
  typedef typename std::conditional<INTS, int64_t, double>::type T8;
  switch (kind_index - (INTS ? kBatchFloatKinds : 0)) {
    case 0: return batch_occupancy_kind<NT, DECODE, 1, T4>(staged_w);
    case 1: return batch_occupancy_kind<NT, DECODE, 2, T4>(staged_w);
    case 2: return batch_occupancy_kind<NT, DECODE, 3, T4>(staged_w);
    case 3: return batch_occupancy_kind<NT, DECODE, 1, T8>(staged_w);
    case 4: return batch_occupancy_kind<NT, DECODE, 2, T8>(staged_w);
    case 5: return batch_occupancy_kind<NT, DECODE, 3, T8>(staged_w);
    default: return 0;
  }
}

}  // namespace gzfp
