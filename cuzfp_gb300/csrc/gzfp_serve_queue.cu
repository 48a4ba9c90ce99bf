// gzfp_serve_queue.cu -- the request server's device-queue mode
// (gzfp_serve_config.device_queue = 1).
//
// One persistent kernel stays on the device for the run and drains a request
// table in pinned, device-mapped host memory:
//
//   host                                   device (every CTA)
//   write request r's descriptor           take ticket c (atomicAdd)
//   published += chunks of r  (release)    wait until c < published
//                                          find its request (forward cursor),
//                                          its descriptor (cached on the device)
//                                          code the chunk's blocks
//   poll done[r]                <--------  last chunk of r: done[r] = 1 (release)
//
// Chunks are numbered across requests in publication order and claimed in
// that order, so the device works first-in first-out at chunk granularity
// while the chunks of consecutive requests run side by side on the SMs: a
// request that arrives while others are coded starts as soon as CTAs free
// up, with no launch.  Each block is coded by the batched path's per-block
// code (batch_block), so its bits are those of a plain call.
//
// Waits are bounded: a CTA that finds no work for `idle_exit_us` leaves the
// kernel, handing its ticket to the same CTA of the next launch, and the
// host relaunches the kernel when new work is published and the previous
// launch has ended.  Only the CTAs holding the next few tickets read the
// host-side counters; the others read their mirror in device memory.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <deque>
#include <numeric>
#include <vector>

#include "gzfp_batch.cuh"
#include "gzfp_serve_host.h"

namespace gzfp {
namespace {

constexpr int kQThreads = 128;     // threads per CTA
constexpr int kQMaxBpt = 4;        // blocks per thread per chunk, at most
constexpr int kQSlots = 32;        // plane-store slots (4^3 blocks)
constexpr uint32_t kQStagedW = 32; // decode stages blocks of up to 32 words
constexpr int kQPollers = 16;      // waiting CTAs that read the host-side counters

// A published request: its descriptor in the batched path's form (first_chunk
// in the run's chunk numbering), its chunk count and which coder runs it.
struct QueueReq {
  BatchDesc d;
  uint32_t nchunks;
  uint32_t code;  // 0 / 1: 3D float / double compress; 2 / 3: decompress
  uint32_t bpt;   // blocks per thread of its chunks (1..kQMaxBpt)
  uint32_t pad;
};
constexpr int kQReqWords = (int)(sizeof(QueueReq) / 8);
static_assert(sizeof(QueueReq) % 8 == 0 && kQReqWords <= 32, "descriptor words");

// host-mapped control words
struct QueueCtl {
  unsigned long long published;  // host: chunks of all published requests
  unsigned int stop;             // host: no more requests will come
  unsigned int idle_exits;       // device: CTAs that left on the idle limit
};

// device-memory state
struct QueueDev {
  unsigned long long ticket;     // next chunk to hand out
  unsigned long long published;  // mirror of QueueCtl::published
  unsigned int stop;             // mirror of QueueCtl::stop
};

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire_sys(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(unsigned* p, unsigned v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
template <typename X>
__device__ __forceinline__ X ld_vol(const X* p) {
  return *(const volatile X*)p;
}

size_t queue_smem_bytes() {
  return (size_t)kQSlots * kQThreads * 8 + (size_t)(kQStagedW + kPadRows) * (kQThreads + 1) * 8;
}

// A request's (first chunk, chunk count), from the device copy of its
// descriptor once one CTA has made it, else from host memory.
__device__ __forceinline__ void req_range(const QueueReq* reqs, const QueueReq* dreqs,
                                          const unsigned* ready, uint32_t r,
                                          unsigned long long& first, unsigned& n) {
  if (ld_acquire_gpu(&ready[r])) {
    first = ld_relaxed_gpu((const unsigned long long*)&dreqs[r].d.first_chunk);
    n = (unsigned)ld_relaxed_gpu((const unsigned long long*)&dreqs[r].nchunks);
  } else {
    first = ld_vol(&reqs[r].d.first_chunk);
    n = ld_vol(&reqs[r].nchunks);
  }
}

// One chunk's blocks of one request, per coder: separate functions, so that
// each gets its own register allocation inside the kernel's budget.
template <bool DECODE, typename T>
__device__ __noinline__ void queue_chunk(const BatchDesc& d, uint64_t first, int bpt,
                                         uint64_t* smem_planes, uint64_t* sbuf) {
  BatchPlanes<kQThreads> ps{smem_planes + threadIdx.x, nullptr};
#pragma unroll 1
  for (int j = 0; j < bpt; j++)
    batch_block<kQThreads, DECODE, 3, T>(d, first + (uint64_t)j * kQThreads + threadIdx.x, ps,
                                         sbuf, kQStagedW);
}

// Tickets: a CTA takes the next chunk number with one atomicAdd and waits
// until the host has published that chunk, so chunks are handed out in
// order with no retries.  A CTA that reaches the idle limit while holding a
// ticket leaves it in abandoned[blockIdx.x]; the same CTA of the next
// launch (the grid does not change within a run) takes it up first, so
// every chunk is coded exactly once.
__global__ void __launch_bounds__(kQThreads, 3)
    serve_queue_kernel(const QueueReq* reqs, QueueReq* dreqs, unsigned* ready, QueueCtl* ctl,
                       unsigned* done, QueueDev* dev, unsigned long long* abandoned,
                       unsigned* finished, unsigned long long* t_first,
                       unsigned long long* t_last, unsigned long long idle_ns, uint32_t r0) {
  extern __shared__ uint64_t smem[];
  __shared__ QueueReq s_req;
  __shared__ unsigned long long s_chunk;
  __shared__ uint32_t s_r;
  __shared__ int s_cmd;
  BatchPlanes<kQThreads> ps{smem + threadIdx.x, nullptr};
  uint64_t* sbuf = smem + kQSlots * kQThreads;
  uint32_t r = r0;              // thread 0: request of the last chunk (none before r0 is left)
  uint32_t loaded = 0xffffffffu;  // every thread: the request s_req holds
  bool held = false;            // thread 0: holds ticket t
  unsigned long long t = 0;
  if (threadIdx.x == 0) {
    t = abandoned[blockIdx.x];
    if (t != ~0ull) {
      abandoned[blockIdx.x] = ~0ull;
      held = true;
    }
  }
  for (;;) {
    if (threadIdx.x == 0) {
      if (!held) {
        t = atomicAdd(&dev->ticket, 1ull);
        held = true;
      }
      // wait until chunk t is published; leave when stopped (it never will
      // be) or after idle_ns (handing the ticket on)
      int cmd = 0;
      const unsigned long long t0 = globaltimer();
      unsigned nap = 64;
      for (;;) {
        // the CTAs holding the next kQPollers tickets -- the ones a new
        // request will start on -- read the host's count; the others its
        // mirror
        unsigned long long p = ld_vol(&dev->published);
        const bool poller = t >= p && t < p + kQPollers;
        if (poller) {
          const unsigned long long hp = ld_acquire_sys(&ctl->published);
          if (hp > p) {
            atomicMax(&dev->published, hp);
            p = hp;
          }
        }
        if (t < p) {
          cmd = 1;
          break;
        }
        unsigned stop = ld_vol(&dev->stop);
        if (!stop && poller && ld_acquire_sys(&ctl->stop)) {
          atomicExch(&dev->stop, 1u);
          stop = 1;
        }
        if (stop) break;
        if (globaltimer() - t0 > idle_ns) {
          abandoned[blockIdx.x] = t;
          cmd = 2;
          break;
        }
        __nanosleep(nap);
        nap = nap < 2048 ? 2 * nap : nap;
      }
      if (cmd == 1) {
        held = false;
        // the chunk's request: requests are numbered in publication order and
        // one CTA's tickets only grow, so the cursor moves forward
        for (;;) {
          unsigned long long f;
          unsigned n;
          req_range(reqs, dreqs, ready, r, f, n);
          if (t < f + n) break;
          r++;
        }
        s_r = r;
        s_chunk = t;
        atomicMin(&t_first[r], globaltimer());
      }
      s_cmd = cmd;
    }
    __syncthreads();
    const int cmd = s_cmd;
    if (cmd != 1) {
      if (cmd == 2 && threadIdx.x == 0) atomicAdd_system(&ctl->idle_exits, 1u);
      return;
    }
    const uint32_t rr = s_r;
    if (rr != loaded) {
      // the descriptor: from its device copy, or from host memory with one
      // word per thread (then copied to the device for the other CTAs)
      if (threadIdx.x < 32) {
        const bool rd = ld_acquire_gpu(&ready[rr]) != 0;
        const unsigned lane = threadIdx.x;
        if (lane < (unsigned)kQReqWords) {
          unsigned long long v;
          if (rd) {
            v = ld_relaxed_gpu((const unsigned long long*)&dreqs[rr] + lane);
          } else {
            v = ld_vol((const unsigned long long*)&reqs[rr] + lane);
            ((unsigned long long*)&dreqs[rr])[lane] = v;
          }
          ((unsigned long long*)&s_req)[lane] = v;
        }
        __syncwarp();
        if (!rd && lane == 0) {
          __threadfence();
          st_release_gpu(&ready[rr], 1u);
        }
      }
      __syncthreads();
      loaded = rr;
    }
    const QueueReq& q = s_req;
    const int bpt = (int)q.bpt;
    const uint64_t first = (s_chunk - q.d.first_chunk) * (uint64_t)(kQThreads * bpt);
    switch (q.code) {
      case 0: queue_chunk<false, float>(q.d, first, bpt, smem, sbuf); break;
      case 1: queue_chunk<false, double>(q.d, first, bpt, smem, sbuf); break;
      case 2: queue_chunk<true, float>(q.d, first, bpt, smem, sbuf); break;
      default: queue_chunk<true, double>(q.d, first, bpt, smem, sbuf); break;
    }
    __syncthreads();  // the chunk's blocks are written
    if (threadIdx.x == 0) {
      __threadfence();  // this CTA's writes before its count
      const unsigned old = atomicAdd(&finished[rr], 1u);
      atomicMax(&t_last[rr], globaltimer());
      if (old + 1 == q.nchunks) {  // every chunk of the request is coded
        __threadfence_system();
        st_release_sys(&done[rr], 1u);
      }
    }
    // s_chunk / s_r are rewritten only after the next __syncthreads
  }
}

using Clock = std::chrono::steady_clock;

// device-mapped pinned host memory
template <typename X>
cudaError_t host_mapped(X** h, X** d, size_t n) {
  cudaError_t e = cudaHostAlloc((void**)h, n * sizeof(X), cudaHostAllocMapped);
  if (e) return e;
  memset((void*)*h, 0, n * sizeof(X));
  return cudaHostGetDevicePointer((void**)d, (void*)*h, 0);
}

// everything one run allocates, released in one place
struct QueueRun {
  char* arena = nullptr;
  QueueReq* h_reqs = nullptr;
  QueueReq* d_reqs = nullptr;
  QueueCtl* h_ctl = nullptr;
  QueueCtl* d_ctl = nullptr;
  unsigned* h_done = nullptr;
  unsigned* d_done = nullptr;
  QueueDev* dev = nullptr;
  QueueReq* dreqs = nullptr;               // device copies of the descriptors
  unsigned* ready = nullptr;               // dreqs[i] is filled in
  unsigned long long* abandoned = nullptr; // per CTA: a ticket handed to the next launch
  unsigned* finished = nullptr;
  unsigned long long* t_first = nullptr;
  unsigned long long* t_last = nullptr;
  cudaStream_t ks = nullptr, cs = nullptr;  // kernel stream, copy stream
  cudaEvent_t kdone = nullptr;
  std::vector<cudaEvent_t> events;
  ~QueueRun() {
    if (ks) cudaStreamSynchronize(ks);
    if (cs) cudaStreamSynchronize(cs);
    for (cudaEvent_t ev : events) cudaEventDestroy(ev);
    if (kdone) cudaEventDestroy(kdone);
    if (ks) cudaStreamDestroy(ks);
    if (cs) cudaStreamDestroy(cs);
    cudaFree(arena);
    cudaFree(dev);
    cudaFree(dreqs);
    cudaFree(ready);
    cudaFree(abandoned);
    cudaFree(finished);
    cudaFree(t_first);
    cudaFree(t_last);
    if (h_reqs) cudaFreeHost(h_reqs);
    if (h_ctl) cudaFreeHost(h_ctl);
    if (h_done) cudaFreeHost(h_done);
  }
};

}  // namespace

namespace serve {

int serve_queue_run(const gzfp_serve_request* reqs, int count, const gzfp_serve_config& cfg,
                    gzfp_serve_result* results, gzfp_serve_stats* stats) {
  for (int i = 0; i < count; i++) {
    const gzfp_serve_request& r = reqs[i];
    if (r.nz == 0 || (r.type != GZFP_TYPE_FLOAT && r.type != GZFP_TYPE_DOUBLE))
      return serve_fail(GZFP_ERR_UNSUPPORTED,
                        "the device-queue server codes 3D float and double requests");
    if (r.maxbits < batch_ebits(r.type) + 1 || r.maxbits > (1u << 20))
      return serve_fail(GZFP_ERR_ARG, "bits per block out of range");
    const Geom g = make_geom_blocks(r.nx, r.ny, r.nz);
    if (g.nblocks >= (1ull << 32)) return serve_fail(GZFP_ERR_ARG, "too many blocks");
  }
  int device = 0, sms = 0, occ = 0;
  cudaError_t e;
  QueueRun q;
  const size_t smem = queue_smem_bytes();
  if ((e = cudaGetDevice(&device)) ||
      (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) ||
      (e = cudaFuncSetAttribute(serve_queue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem)) ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_queue_kernel, kQThreads,
                                                         smem)))
    return serve_cuda(e, "device-queue kernel set-up");
  if (occ < 1) return serve_fail(GZFP_ERR_CUDA, "device-queue kernel does not fit on an SM");
  const int grid = sms * occ;  // every CTA resident
  if ((e = cudaMalloc(&q.arena, cfg.budget_bytes)) ||
      (e = host_mapped(&q.h_reqs, &q.d_reqs, (size_t)count)) ||
      (e = host_mapped(&q.h_ctl, &q.d_ctl, 1)) ||
      (e = host_mapped(&q.h_done, &q.d_done, (size_t)count)) ||
      (e = cudaMalloc(&q.dev, sizeof(QueueDev))) ||
      (e = cudaMalloc(&q.dreqs, count * sizeof(QueueReq))) ||
      (e = cudaMalloc(&q.ready, count * sizeof(unsigned))) ||
      (e = cudaMalloc(&q.abandoned, grid * sizeof(unsigned long long))) ||
      (e = cudaMalloc(&q.finished, count * sizeof(unsigned))) ||
      (e = cudaMalloc(&q.t_first, count * sizeof(unsigned long long))) ||
      (e = cudaMalloc(&q.t_last, count * sizeof(unsigned long long))) ||
      (e = cudaStreamCreateWithFlags(&q.ks, cudaStreamNonBlocking)) ||
      (e = cudaStreamCreateWithFlags(&q.cs, cudaStreamNonBlocking)) ||
      (e = cudaEventCreateWithFlags(&q.kdone, cudaEventDisableTiming)) ||
      (e = cudaMemsetAsync(q.dev, 0, sizeof(QueueDev), q.ks)) ||
      (e = cudaMemsetAsync(q.ready, 0, count * sizeof(unsigned), q.ks)) ||
      (e = cudaMemsetAsync(q.abandoned, 0xff, grid * sizeof(unsigned long long), q.ks)) ||
      (e = cudaMemsetAsync(q.finished, 0, count * sizeof(unsigned), q.ks)) ||
      (e = cudaMemsetAsync(q.t_first, 0xff, count * sizeof(unsigned long long), q.ks)) ||
      (e = cudaMemsetAsync(q.t_last, 0, count * sizeof(unsigned long long), q.ks)) ||
      (e = cudaStreamSynchronize(q.ks)))
    return serve_cuda(e, "device-queue set-up");
  Arena arena(cfg.budget_bytes);
  const unsigned long long idle_ns = 1000ull * cfg.idle_exit_us;
  std::vector<int> req_of(count), pub_of(count, -1);  // publication <-> request
  auto launch = [&](uint32_t r0) -> cudaError_t {
    serve_queue_kernel<<<grid, kQThreads, smem, q.ks>>>(
        q.d_reqs, q.dreqs, q.ready, q.d_ctl, q.d_done, q.dev, q.abandoned, q.finished, q.t_first,
        q.t_last, idle_ns, r0);
    cudaError_t le = cudaGetLastError();
    return le ? le : cudaEventRecord(q.kdone, q.ks);
  };

  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return reqs[a].arrival < reqs[b].arrival; });
  std::vector<size_t> offs(count, 0);
  std::vector<int> inflight;                       // published, not yet done
  struct Copy { cudaEvent_t ev; size_t off, bytes; };
  std::deque<Copy> copies;                         // copy_to copies still reading the arena
  std::vector<cudaEvent_t> spare;
  std::deque<int> queue;
  size_t next = 0;
  int completed = 0, publications = 0, kernels = 0, npub = 0;
  unsigned long long published = 0;
  double inflight_sum = 0, busy_time = 0, busy_since = -1, last_progress = 0;
  bool running = false;
  int st = GZFP_OK;
  const Clock::time_point t0 = Clock::now();
  auto now = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };

  while (!st && completed < count) {
    double t = now();
    // the kernel's CTAs leave when idle; note when the launch has ended
    if (running) {
      e = cudaEventQuery(q.kdone);
      if (e == cudaSuccess) running = false;
      else if (e != cudaErrorNotReady) { st = serve_cuda(e, "device-queue kernel"); break; }
    }
    // completions
    for (size_t j = 0; j < inflight.size();) {
      const int r = inflight[j];
      if (!__atomic_load_n(&q.h_done[pub_of[r]], __ATOMIC_ACQUIRE)) { j++; continue; }
      t = now();
      results[r].completed = t;
      last_progress = t;
      completed++;
      const gzfp_serve_request& rq = reqs[r];
      if (rq.copy_to) {  // the arena range is released once the copy has read it
        cudaEvent_t ev = nullptr;
        if (!spare.empty()) { ev = spare.back(); spare.pop_back(); }
        else if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming))) {
          st = serve_cuda(e, "cudaEventCreate"); break;
        } else q.events.push_back(ev);
        if ((e = cudaMemcpyAsync(rq.copy_to, q.arena + offs[r], results[r].output_bytes,
                                 cudaMemcpyDeviceToDevice, q.cs)) ||
            (e = cudaEventRecord(ev, q.cs))) {
          st = serve_cuda(e, "output copy"); break;
        }
        copies.push_back(Copy{ev, offs[r], results[r].output_bytes});
      } else {
        arena.release(offs[r], results[r].output_bytes);
      }
      inflight[j] = inflight.back();
      inflight.pop_back();
      if (inflight.empty()) busy_time += t - busy_since;
    }
    if (st) break;
    while (!copies.empty()) {
      e = cudaEventQuery(copies.front().ev);
      if (e == cudaErrorNotReady) break;
      if (e != cudaSuccess) { st = serve_cuda(e, "output copy"); break; }
      arena.release(copies.front().off, copies.front().bytes);
      spare.push_back(copies.front().ev);
      copies.pop_front();
    }
    if (st) break;
    // arrivals
    while (next < order.size() && reqs[order[next]].arrival <= t) queue.push_back(order[next++]);
    // admission: publish the head of the queue while its output fits
    int added = 0;
    while (!queue.empty() && added < cfg.max_batch) {
      const int r = queue.front();
      const gzfp_serve_request& rq = reqs[r];
      if (results[r].output_bytes > cfg.budget_bytes) {  // can never fit
        results[r].status = GZFP_ERR_CAPACITY;
        results[r].admitted = results[r].completed = t;
        completed++;
        queue.pop_front();
        continue;
      }
      const size_t off = arena.alloc(results[r].output_bytes);
      if (off == SIZE_MAX) break;  // wait for completions to free memory
      queue.pop_front();
      offs[r] = off;
      const bool decode = rq.op == GZFP_SERVE_DECOMPRESS;
      QueueReq& e_r = q.h_reqs[npub];
      req_of[npub] = r;
      pub_of[r] = npub;
      const void* field = decode ? (const void*)(q.arena + off) : rq.input;
      e_r.d.g = make_geom_blocks(rq.nx, rq.ny, rq.nz);
      e_r.d.g.vec =
          (rq.nx % 4 == 0 && (uintptr_t)field % batch_row_align(rq.type) == 0) ? 1u : 0u;
      e_r.d.nwords = (e_r.d.g.nblocks * rq.maxbits + 63) / 64;
      e_r.d.maxbits = rq.maxbits;
      e_r.d.kind = batch_kind(rq.type, 3);
      e_r.d.in = rq.input;           // the field (compress) or stream words (decompress)
      e_r.d.out = q.arena + off;     // the stream words or the field
      e_r.d.first_chunk = published;
      // chunks small enough that a request of under a few waves of blocks
      // still spreads over every CTA, larger for large requests
      const uint64_t wave = (uint64_t)grid * kQThreads;
      e_r.bpt = (uint32_t)std::min<uint64_t>(kQMaxBpt, std::max<uint64_t>(1, e_r.d.g.nblocks / wave));
      const uint64_t chunk = (uint64_t)kQThreads * e_r.bpt;
      e_r.nchunks = (uint32_t)((e_r.d.g.nblocks + chunk - 1) / chunk);
      e_r.code = (decode ? 2u : 0u) + (rq.type == GZFP_TYPE_DOUBLE ? 1u : 0u);
      if (!decode && rq.maxbits % 64) {
        // blocks that share words are merged with atomic ORs: zero the
        // output before the request is published
        if ((e = cudaMemsetAsync(q.arena + off, 0, results[r].output_bytes, q.cs)) ||
            (e = cudaStreamSynchronize(q.cs))) {
          st = serve_cuda(e, "cudaMemsetAsync(stream)"); break;
        }
      }
      // a request is published by the count that covers its chunks: its
      // descriptor (and every earlier one) is written first
      published += e_r.nchunks;
      if (e_r.nchunks == 0) {  // nothing to code (cannot happen: every request has a block)
        st = serve_fail(GZFP_ERR_ARG, "empty request"); break;
      }
      __atomic_store_n(&q.h_ctl->published, published, __ATOMIC_RELEASE);
      t = now();
      results[r].admitted = t;
      results[r].batch = publications;
      if (inflight.empty()) busy_since = t;
      inflight.push_back(r);
      inflight_sum += (double)inflight.size();
      npub++;
      added++;
    }
    if (st) break;
    if (added) publications++;
    // work published and no launch running: (re)launch the kernel
    if (!running && !inflight.empty()) {
      // every publication before the oldest one in flight is done
      int r0 = npub;
      for (int r : inflight) r0 = std::min(r0, pub_of[r]);
      if ((e = launch((uint32_t)r0))) { st = serve_cuda(e, "device-queue kernel launch"); break; }
      running = true;
      kernels++;
    }
    if (inflight.empty() && queue.empty()) last_progress = now();
    if (!inflight.empty() && now() - last_progress > 60.0) {
      st = serve_fail(GZFP_ERR_CUDA, "device-queue server made no progress for 60 s");
      break;
    }
  }

  const double wall = now();
  // no more requests: the kernel leaves once nothing is left to claim
  __atomic_store_n(&q.h_ctl->stop, 1u, __ATOMIC_RELEASE);
  if (running && (e = cudaEventSynchronize(q.kdone)) && !st) st = serve_cuda(e, "device-queue kernel");
  if ((e = cudaStreamSynchronize(q.cs)) && !st) st = serve_cuda(e, "output copy");
  // device clock stamps of every request, relative to the run's first chunk
  std::vector<unsigned long long> tf(count), tl(count);
  if (!st && npub &&
      ((e = cudaMemcpy(tf.data(), q.t_first, npub * 8, cudaMemcpyDeviceToHost)) ||
       (e = cudaMemcpy(tl.data(), q.t_last, npub * 8, cudaMemcpyDeviceToHost))))
    st = serve_cuda(e, "device stamps");
  if (!st) {
    unsigned long long base = ~0ull;
    for (int p = 0; p < npub; p++) base = std::min(base, tf[p]);
    for (int p = 0; p < npub; p++) {
      gzfp_serve_result& res = results[req_of[p]];
      res.device_start = 1e-9 * (double)(tf[p] - base);
      res.device_end = 1e-9 * (double)(tl[p] - base);
    }
  }
  if (stats) {
    double last = 0;
    for (int i = 0; i < count; i++) last = std::max(last, results[i].completed);
    stats->wall = st ? wall : last;
    stats->batches = publications;
    stats->mean_batch = publications ? (double)npub / publications : 0.0;
    stats->peak_bytes = arena.peak();
    stats->busy = stats->wall > 0 ? busy_time / stats->wall : 0.0;
    stats->kernels = kernels;
    stats->mean_inflight = npub ? inflight_sum / npub : 0.0;
  }
  return st;
}

}  // namespace serve
}  // namespace gzfp
