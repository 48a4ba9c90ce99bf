// gzfp_serve_queue.cu -- the request server's device-queue mode
// (gzfp_serve_config.device_queue = 1), for every scalar type and
// dimensionality.
//
// A request table in pinned, device-mapped host memory is drained on the
// device by a persistent scheduler kernel (one thread), which launches each
// published request as its own grid with a device-side launch:
//
//   host                                   scheduler (device)
//   write request p's descriptor           wait until p < published
//   published = p + 1  (release)           read p's descriptor
//                                          launch p's grid (fire and forget)
//   poll done[p]                <--------  p's last CTA: done[p] = 1 (release)
//
// A request's grid is the per-kind kernel of gzfp_serve_queue.cuh (its
// instances in gzfp_serve_req_<type>.cu): one CTA per 128 blocks,
// one block per thread, the descriptor a kernel parameter, and the batched
// path's per-block code (batch_block), so its bits are those of a plain call
// and its register budget is that coder's own.  Grids of consecutive
// requests run side by side as the SMs free up, with no host launch and no
// batching delay.  (Claiming chunks from inside one persistent coding kernel
// was measured slower: that kernel has one register budget for every coder,
// and its loop around the block code makes the 4^3 double coders spill.)
//
// Waits are bounded: a scheduler that sees nothing published for
// `idle_exit_us` leaves, recording how far it launched, and the host starts
// a new one when work is published again.  Requests launched and not yet
// done are capped below the device runtime's pending-launch limit; a
// scheduler held at the cap with no request finishing for 10 s reports an
// error and leaves.  A failed device-side launch is reported, not retried.
//
// These translation units are compiled as relocatable device code and
// linked with the CUDA device runtime (cudadevrt).
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <numeric>
#include <vector>

#include "gzfp_serve_host.h"
#include "gzfp_serve_queue.cuh"

namespace gzfp {
namespace {

constexpr unsigned long long kQMaxLaunched = 1024;  // requests launched and not done, at most
constexpr unsigned long long kQStallNs = 10000000000ull;  // 10 s at the cap with no completion

// host-mapped control words
struct QueueCtl {
  unsigned long long published;  // host: requests published
  unsigned long long launched;   // device: requests launched, written when a scheduler leaves
  unsigned int stop;             // host: no more requests will come
  unsigned int idle_exits;       // device: schedulers that left on the idle limit
  unsigned int ended;            // device: generation of the last scheduler that left
  int error;                     // device: cudaError_t of a failed launch (or a stall)
  unsigned long long error_req;  // device: the request it concerned
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
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(unsigned* p, unsigned v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The scheduler: one thread launches published requests in order, from
// request `next` on.  It leaves when stopped, when nothing is published for
// idle_ns, on a failed launch, or when held at the cap for kQStallNs with no
// request finishing; it then records how far it launched and its
// generation.
__global__ void serve_sched_kernel(const QueueReq* reqs, QueueCtl* ctl, QueueDev q,
                                   unsigned long long next, unsigned long long idle_ns,
                                   unsigned gen) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long launched = next;
  unsigned long long t_idle = globaltimer(), t_prog = t_idle;
  unsigned long long seen = ld_relaxed_gpu(q.completed);
  unsigned nap = 32;
  for (;;) {
    const unsigned long long now = globaltimer();
    if (launched < ld_acquire_sys(&ctl->published)) {
      const unsigned long long c = ld_relaxed_gpu(q.completed);
      if (c != seen) {
        seen = c;
        t_prog = now;
      }
      if (launched - c < kQMaxLaunched) {
        const QueueReq r = reqs[launched];  // written before its publication
        cudaError_t e;
        switch ((r.code & (kQDecode - 1)) / 3) {  // scalar type of the kind
          case 0: e = queue_launch_f32(r, (uint32_t)launched, q); break;
          case 1: e = queue_launch_f64(r, (uint32_t)launched, q); break;
          case 2: e = queue_launch_i32(r, (uint32_t)launched, q); break;
          case 3: e = queue_launch_i64(r, (uint32_t)launched, q); break;
          default: e = cudaErrorInvalidValue; break;
        }
        if (e != cudaSuccess) {
          ctl->error = (int)e;
          ctl->error_req = launched;
          break;
        }
        launched++;
        t_idle = t_prog = now;
        nap = 32;
        continue;
      }
      if (now - t_prog > kQStallNs) {  // at the cap and nothing finishes
        ctl->error = (int)cudaErrorLaunchTimeout;
        ctl->error_req = launched;
        break;
      }
      t_idle = now;  // work is waiting: not idle
    } else {
      if (ld_acquire_sys(&ctl->stop)) break;
      if (now - t_idle > idle_ns) {
        atomicAdd_system(&ctl->idle_exits, 1u);
        break;
      }
    }
    __nanosleep(nap);
    nap = nap < 1024 ? 2 * nap : nap;
  }
  ctl->launched = launched;
  __threadfence_system();
  st_release_sys(&ctl->ended, gen);
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
  QueueDev dev{};  // device pointers (done: host-mapped)
  // schedulers run on a pool of streams: a scheduler's grid completes only
  // once the requests it launched are done, so the next one takes a stream
  // whose last scheduler grid has completed (or a new stream)
  std::vector<cudaStream_t> ks;
  std::vector<cudaEvent_t> kdone;
  cudaStream_t cs = nullptr;  // copy stream
  std::vector<cudaEvent_t> events;
  ~QueueRun() {
    for (cudaStream_t s : ks) cudaStreamSynchronize(s);
    if (cs) cudaStreamSynchronize(cs);
    for (cudaEvent_t ev : events) cudaEventDestroy(ev);
    for (cudaEvent_t ev : kdone) cudaEventDestroy(ev);
    for (cudaStream_t s : ks) cudaStreamDestroy(s);
    if (cs) cudaStreamDestroy(cs);
    cudaFree(arena);
    cudaFree(dev.finished);
    cudaFree(dev.t_first);
    cudaFree(dev.t_last);
    cudaFree(dev.completed);
    if (h_reqs) cudaFreeHost(h_reqs);
    if (h_ctl) cudaFreeHost(h_ctl);
    if (h_done) cudaFreeHost(h_done);
  }
  // a stream whose last scheduler grid has completed
  cudaError_t free_stream(size_t* i) {
    for (size_t j = 0; j < ks.size(); j++) {
      const cudaError_t e = cudaEventQuery(kdone[j]);
      if (e == cudaSuccess) {
        *i = j;
        return cudaSuccess;
      }
      if (e != cudaErrorNotReady) return e;
    }
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking))) return e;
    ks.push_back(s);
    if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming))) return e;
    kdone.push_back(ev);
    *i = ks.size() - 1;
    return cudaSuccess;
  }
};

}  // namespace

namespace serve {

int serve_queue_run(const gzfp_serve_request* reqs, int count, const gzfp_serve_config& cfg,
                    gzfp_serve_result* results, gzfp_serve_stats* stats) {
  for (int i = 0; i < count; i++) {
    const gzfp_serve_request& r = reqs[i];
    if (r.nx == 0 || (r.nz != 0 && r.ny == 0)) return serve_fail(GZFP_ERR_ARG, "bad dimensions");
    if (r.maxbits < batch_ebits(r.type) + 1 || r.maxbits > (1u << 20))
      return serve_fail(GZFP_ERR_ARG, "bits per block out of range");
    const Geom g = make_geom_blocks(r.nx, r.ny ? r.ny : 1, r.nz ? r.nz : 1);
    if ((g.nblocks + kQThreads - 1) / kQThreads >= (1ull << 31))
      return serve_fail(GZFP_ERR_ARG, "too many blocks");
  }
  cudaError_t e;
  QueueRun q;
  if ((e = queue_setup_f32()) || (e = queue_setup_f64()) || (e = queue_setup_i32()) ||
      (e = queue_setup_i64()))
    return serve_cuda(e, "device-queue kernel set-up");
  if ((e = cudaMalloc(&q.arena, cfg.budget_bytes)) ||
      (e = host_mapped(&q.h_reqs, &q.d_reqs, (size_t)count)) ||
      (e = host_mapped(&q.h_ctl, &q.d_ctl, 1)) ||
      (e = host_mapped(&q.h_done, &q.dev.done, (size_t)count)) ||
      (e = cudaMalloc(&q.dev.finished, count * sizeof(unsigned))) ||
      (e = cudaMalloc(&q.dev.t_first, count * sizeof(unsigned long long))) ||
      (e = cudaMalloc(&q.dev.t_last, count * sizeof(unsigned long long))) ||
      (e = cudaMalloc(&q.dev.completed, sizeof(unsigned long long))) ||
      (e = cudaStreamCreateWithFlags(&q.cs, cudaStreamNonBlocking)) ||
      (e = cudaMemsetAsync(q.dev.finished, 0, count * sizeof(unsigned), q.cs)) ||
      (e = cudaMemsetAsync(q.dev.t_first, 0xff, count * sizeof(unsigned long long), q.cs)) ||
      (e = cudaMemsetAsync(q.dev.t_last, 0, count * sizeof(unsigned long long), q.cs)) ||
      (e = cudaMemsetAsync(q.dev.completed, 0, sizeof(unsigned long long), q.cs)) ||
      (e = cudaStreamSynchronize(q.cs)))
    return serve_cuda(e, "device-queue set-up");
  Arena arena(cfg.budget_bytes);
  const unsigned long long idle_ns = 1000ull * cfg.idle_exit_us;
  unsigned gen = 0;  // schedulers started
  auto launch = [&](unsigned long long next) -> cudaError_t {
    size_t i = 0;
    cudaError_t le = q.free_stream(&i);
    if (le) return le;
    gen++;
    serve_sched_kernel<<<1, 32, 0, q.ks[i]>>>(q.d_reqs, q.d_ctl, q.dev, next, idle_ns, gen);
    le = cudaGetLastError();
    return le ? le : cudaEventRecord(q.kdone[i], q.ks[i]);
  };

  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return reqs[a].arrival < reqs[b].arrival; });
  std::vector<int> req_of(count), pub_of(count, -1);  // publication <-> request
  std::vector<size_t> offs(count, 0);
  std::vector<int> inflight;                       // published, not yet done
  struct Copy { cudaEvent_t ev; size_t off, bytes; };
  std::deque<Copy> copies;                         // copy_to copies still reading the arena
  std::vector<cudaEvent_t> spare;
  std::deque<int> queue;
  size_t next = 0;
  int completed = 0, publications = 0, npub = 0;
  double inflight_sum = 0, busy_time = 0, busy_since = -1, last_progress = 0;
  bool running = false;  // a scheduler is in its loop
  int st = GZFP_OK;
  const Clock::time_point t0 = Clock::now();
  auto now = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };
  // a scheduler left: note it, and fail the run if it reported an error
  auto poll_scheduler = [&]() {
    if (!running || __atomic_load_n(&q.h_ctl->ended, __ATOMIC_ACQUIRE) != gen) return;
    running = false;
    const int err = __atomic_load_n(&q.h_ctl->error, __ATOMIC_ACQUIRE);
    if (err) {
      char msg[128];
      snprintf(msg, sizeof msg, "device-side launch of request %llu",
               (unsigned long long)q.h_ctl->error_req);
      st = serve_cuda((cudaError_t)err, msg);
    }
  };

  while (!st && completed < count) {
    double t = now();
    poll_scheduler();
    if (st) break;
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
      const int dims = rq.nz ? 3 : rq.ny ? 2 : 1;
      e_r.d.g = make_geom_blocks(rq.nx, rq.ny ? rq.ny : 1, rq.nz ? rq.nz : 1);
      e_r.d.g.vec =
          (rq.nx % 4 == 0 && (uintptr_t)field % batch_row_align(rq.type) == 0) ? 1u : 0u;
      e_r.d.nwords = (e_r.d.g.nblocks * rq.maxbits + 63) / 64;
      e_r.d.maxbits = rq.maxbits;
      e_r.d.kind = batch_kind(rq.type, dims);
      e_r.d.in = rq.input;           // the field (compress) or stream words (decompress)
      e_r.d.out = q.arena + off;     // the stream words or the field
      e_r.d.first_chunk = 0;
      e_r.ctas = (uint32_t)((e_r.d.g.nblocks + kQThreads - 1) / kQThreads);
      e_r.code = (uint32_t)batch_kind_index(e_r.d.kind) | (decode ? kQDecode : 0u);
      if (!decode && rq.maxbits % 64) {
        // blocks that share words are merged with atomic ORs: zero the
        // output before the request is published
        if ((e = cudaMemsetAsync(q.arena + off, 0, results[r].output_bytes, q.cs)) ||
            (e = cudaStreamSynchronize(q.cs))) {
          st = serve_cuda(e, "cudaMemsetAsync(stream)"); break;
        }
      }
      // a request is published by the count that covers it: its descriptor
      // (and every earlier one) is written first
      npub++;
      __atomic_store_n(&q.h_ctl->published, (unsigned long long)npub, __ATOMIC_RELEASE);
      t = now();
      results[r].admitted = t;
      results[r].batch = publications;
      if (inflight.empty()) busy_since = t;
      inflight.push_back(r);
      inflight_sum += (double)inflight.size();
      added++;
    }
    if (st) break;
    if (added) publications++;
    // work published and no scheduler in its loop: start one where the last
    // one stopped
    if (!running && __atomic_load_n(&q.h_ctl->launched, __ATOMIC_ACQUIRE) < (unsigned long long)npub) {
      if ((e = launch(__atomic_load_n(&q.h_ctl->launched, __ATOMIC_ACQUIRE)))) {
        st = serve_cuda(e, "device-queue scheduler launch"); break;
      }
      running = true;
    }
    if (inflight.empty() && queue.empty()) last_progress = now();
    if (!inflight.empty() && now() - last_progress > 60.0) {
      st = serve_fail(GZFP_ERR_CUDA, "device-queue server made no progress for 60 s");
      break;
    }
  }

  const double wall = now();
  // no more requests: the scheduler leaves once it has launched everything
  // published; every grid (schedulers, and with them their requests) ends
  __atomic_store_n(&q.h_ctl->stop, 1u, __ATOMIC_RELEASE);
  for (cudaStream_t s : q.ks)
    if ((e = cudaStreamSynchronize(s)) && !st) st = serve_cuda(e, "device-queue kernels");
  if ((e = cudaStreamSynchronize(q.cs)) && !st) st = serve_cuda(e, "output copy");
  // device clock stamps of every request, relative to the run's first CTA
  std::vector<unsigned long long> tf(count), tl(count);
  if (!st && npub &&
      ((e = cudaMemcpy(tf.data(), q.dev.t_first, npub * 8, cudaMemcpyDeviceToHost)) ||
       (e = cudaMemcpy(tl.data(), q.dev.t_last, npub * 8, cudaMemcpyDeviceToHost))))
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
    stats->kernels = (int)gen + npub;  // schedulers, and one grid per request
    stats->schedulers = (int)gen;
    stats->mean_inflight = npub ? inflight_sum / npub : 0.0;
  }
  return st;
}

}  // namespace serve
}  // namespace gzfp
