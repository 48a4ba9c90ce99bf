// gzfp_serve_queue.cuh -- the request grids of the device-queue server
// (gzfp_serve_queue.cu): the descriptor a published request carries, the
// per-request kernel, and the launch of a request from the device.  The
// kernels of each scalar type are compiled in their own translation unit
// (gzfp_serve_req_<type>.cu, relocatable device code, as is the scheduler
// that calls their launchers).
#pragma once

#include "gzfp_batch.cuh"

namespace gzfp {

constexpr int kQThreads = 128;  // threads (= blocks) per CTA of a request's grid

// A published request: its descriptor in the batched path's form, the CTAs
// of its grid and which coder runs it: code = kind index (into kBatchKind)
// | kQDecode for decompression.
struct QueueReq {
  BatchDesc d;
  uint32_t ctas;
  uint32_t code;
};
constexpr uint32_t kQDecode = 16;

// per-request device state
struct QueueDev {
  unsigned* finished;             // CTAs of each request done
  unsigned long long* t_first;    // device clock at its first CTA's start
  unsigned long long* t_last;     // ... and at its last CTA's end
  unsigned long long* completed;  // requests done (one counter)
  unsigned* done;                 // host-mapped done flags
};

__device__ __forceinline__ unsigned long long queue_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void queue_st_release_sys(unsigned* p, unsigned v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// registers per thread that let MINB CTAs of kQThreads share an SM
constexpr int queue_maxnreg(int minb) { return 65536 / (kQThreads * minb) / 8 * 8; }

// One request's grid: CTA i codes blocks [128 i, 128 i + 128).  The last CTA
// to finish raises the request's done flag.  The register budget is set with
// __maxnreg__, not __launch_bounds__: measured on GB300, a device-launched
// grid of a kernel with launch bounds and dynamic shared memory gets one
// resident CTA per SM, with __maxnreg__ as many as fit.  PATH: kPathStaged
// (the request stages its words in shared memory) or kPathDirect.
template <bool DECODE, int D, typename T, int MINB, int PATH>
__global__ void __maxnreg__(queue_maxnreg(MINB))
    serve_request_kernel(const __grid_constant__ BatchDesc d, uint32_t p, uint32_t staged_w,
                         QueueDev q) {
  extern __shared__ uint64_t smem[];
  const Plane4Tables* t4 = stage_tables<D, kQThreads>(smem);
  BatchPlanes<kQThreads> ps{smem + table_words<D>() + threadIdx.x, t4};
  uint64_t* sbuf = smem + table_words<D>() + BatchSlots<DECODE, D, T>::value * kQThreads;
  if (threadIdx.x == 0) atomicMin(&q.t_first[p], queue_clock());
  batch_block<kQThreads, DECODE, D, T, PATH>(d, (uint64_t)blockIdx.x * kQThreads + threadIdx.x,
                                             ps, sbuf, staged_w);
  __syncthreads();  // the CTA's blocks are written
  if (threadIdx.x == 0) {
    __threadfence();
    atomicMax(&q.t_last[p], queue_clock());
    if (atomicAdd(&q.finished[p], 1u) + 1 == gridDim.x) {  // every CTA of the request is done
      __threadfence_system();
      queue_st_release_sys(&q.done[p], 1u);
      atomicAdd(q.completed, 1ull);
    }
  }
}

// A coder's launches: register budget as the plain kernels' (the 4^3
// 64-bit decoder's wide budget where shared memory allows its fourth CTA),
// staging depth as the batched path chooses it.
template <bool DECODE, int D, typename T>
struct QueueCoder {
  static constexpr int MB = BatchMinBlocks<kQThreads, D, T>::value;
  static constexpr int WIDE = BatchMinBlocksWide<kQThreads, DECODE, D, T>::value;
  __host__ __device__ static uint32_t staged_w(uint32_t maxbits) {
    const uint32_t sw = batch_item_staged_w(DECODE, maxbits);
    return !DECODE && sw && !batch_smem_fits(batch_smem_bytes<kQThreads, DECODE, D, T>(sw), MB)
               ? 0
               : sw;
  }
  // largest dynamic shared memory a launch asks for
  static size_t max_smem() {
    return batch_smem_bytes<kQThreads, DECODE, D, T>(DECODE ? kBatchMaxStagedWords
                                                            : kMaxStagedOut);
  }
  template <int M, int PATH>
  __device__ static void go(const QueueReq& r, uint32_t p, uint32_t sw, size_t smem,
                            const QueueDev& q) {
    serve_request_kernel<DECODE, D, T, M, PATH>
        <<<r.ctas, kQThreads, smem, cudaStreamFireAndForget>>>(r.d, p, sw, q);
  }
  __device__ static cudaError_t launch(const QueueReq& r, uint32_t p, const QueueDev& q) {
    const uint32_t sw = staged_w(r.d.maxbits);
    const size_t smem = batch_smem_bytes<kQThreads, DECODE, D, T>(sw);
    const bool wide = WIDE != MB && batch_smem_fits(smem, WIDE);
    if (sw)
      wide ? go<WIDE, kPathStaged>(r, p, sw, smem, q) : go<MB, kPathStaged>(r, p, sw, smem, q);
    else
      wide ? go<WIDE, kPathDirect>(r, p, sw, smem, q) : go<MB, kPathDirect>(r, p, sw, smem, q);
    return cudaGetLastError();
  }
  template <int M, int PATH>
  static cudaError_t attr() {
    return cudaFuncSetAttribute(serve_request_kernel<DECODE, D, T, M, PATH>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem());
  }
  static cudaError_t setup() {
    cudaError_t e;
    if ((e = attr<MB, kPathStaged>()) || (e = attr<MB, kPathDirect>())) return e;
    if (WIDE == MB) return cudaSuccess;
    if ((e = attr<WIDE, kPathStaged>()) || (e = attr<WIDE, kPathDirect>())) return e;
    return cudaSuccess;
  }
};

// Every coder of scalar type T: kind index k % 3 + 1 dimensions, direction
// from the code.
template <typename T>
__device__ cudaError_t queue_launch_t(const QueueReq& r, uint32_t p, const QueueDev& q) {
  const bool decode = (r.code & kQDecode) != 0;
  switch ((r.code & (kQDecode - 1)) % 3) {
    case 0: return decode ? QueueCoder<true, 1, T>::launch(r, p, q) : QueueCoder<false, 1, T>::launch(r, p, q);
    case 1: return decode ? QueueCoder<true, 2, T>::launch(r, p, q) : QueueCoder<false, 2, T>::launch(r, p, q);
    default: return decode ? QueueCoder<true, 3, T>::launch(r, p, q) : QueueCoder<false, 3, T>::launch(r, p, q);
  }
}
template <typename T>
cudaError_t queue_setup_t() {
  cudaError_t e;
  if ((e = QueueCoder<false, 1, T>::setup()) || (e = QueueCoder<true, 1, T>::setup()) ||
      (e = QueueCoder<false, 2, T>::setup()) || (e = QueueCoder<true, 2, T>::setup()) ||
      (e = QueueCoder<false, 3, T>::setup()) || (e = QueueCoder<true, 3, T>::setup()))
    return e;
  return cudaSuccess;
}

// Per scalar type (gzfp_serve_req_<type>.cu): launch request p from the
// device, and set the kernels' shared-memory limits from the host.
#define GZFP_QUEUE_DECL(t)                                                              \
  __device__ cudaError_t queue_launch_##t(const QueueReq& r, uint32_t p, const QueueDev& q); \
  cudaError_t queue_setup_##t();
GZFP_QUEUE_DECL(f32)
GZFP_QUEUE_DECL(f64)
GZFP_QUEUE_DECL(i32)
GZFP_QUEUE_DECL(i64)
#undef GZFP_QUEUE_DECL

}  // namespace gzfp
