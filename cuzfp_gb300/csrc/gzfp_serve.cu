// gzfp_serve.cu -- the request server of include/gzfp.h ("serving"): its
// entry point, and the slot mode (device_queue = 0; the device-queue mode,
// the default, is in gzfp_serve_queue.cu).
//
// In slot mode one host thread runs an event loop over three things: arrivals (requests
// whose arrival time has passed join a FIFO queue), completions (a slot
// whose batch event has fired releases its requests' output memory) and
// launches (while a slot is free and requests wait, the head of the queue
// is admitted request by request as long as its output fits in the arena,
// and the admitted set is launched on that slot's stream as one compress
// batch and one decompress batch of the batched path).  Slots give the
// overlap: a batch launched while others still run starts on the SMs as
// their CTAs drain, so a new request waits for a free slot, not for the
// whole device.  Admission is strictly FIFO so that a large request is
// never starved by small ones behind it.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <numeric>
#include <vector>

#include "gzfp_batch_host.h"
#include "gzfp_serve_host.h"

namespace {

thread_local char g_serve_error[256];

int sfail(int status, const char* msg) {
  snprintf(g_serve_error, sizeof g_serve_error, "%s", msg);
  gzfp::batch_set_error(g_serve_error);
  return status;
}
int scuda(cudaError_t e, const char* what) {
  snprintf(g_serve_error, sizeof g_serve_error, "%s: %s", what, cudaGetErrorString(e));
  gzfp::batch_set_error(g_serve_error);
  return GZFP_ERR_CUDA;
}

using gzfp::serve::Arena;
using gzfp::serve::kAlign;
using gzfp::serve::output_bytes;
constexpr int kMaxInflight = 8;

struct Slot {
  cudaStream_t s = nullptr;
  cudaEvent_t done = nullptr;
  gzfp::bhost::WorkList wl[2];  // compress, decompress
  gzfp::bhost::Prepared prep[2];
  std::vector<int> reqs;
  std::vector<size_t> offs;
  bool busy = false;
  int batch = -1;
};

using Clock = std::chrono::steady_clock;

}  // namespace

namespace gzfp {
namespace serve {
int serve_fail(int status, const char* msg) { return sfail(status, msg); }
int serve_cuda(cudaError_t e, const char* what) { return scuda(e, what); }
}  // namespace serve
}  // namespace gzfp

extern "C" {

void gzfp_serve_default_config(gzfp_serve_config* cfg) {
  if (!cfg) return;
  cfg->budget_bytes = 40ull << 30;
  cfg->max_batch = 256;
  cfg->max_inflight = 3;
  gzfp_batch_default_config(&cfg->compress_cfg);
  gzfp_batch_default_config(&cfg->decompress_cfg);
  cfg->device_queue = 1;
  cfg->idle_exit_us = 2000;
}

int gzfp_serve_run(const gzfp_serve_request* reqs, int count, const gzfp_serve_config* cfg_in,
                   gzfp_serve_result* results, gzfp_serve_stats* stats) {
  g_serve_error[0] = 0;
  gzfp::batch_set_error("");
  if (count < 0 || (count && (!reqs || !results))) return sfail(GZFP_ERR_ARG, "bad request list");
  gzfp_serve_config cfg;
  gzfp_serve_default_config(&cfg);
  if (cfg_in) cfg = *cfg_in;
  if (cfg.max_batch < 1 || cfg.max_batch > 65535 || cfg.max_inflight < 1 ||
      cfg.max_inflight > kMaxInflight || cfg.budget_bytes < kAlign ||
      !gzfp::bhost::valid_config(cfg.compress_cfg) ||
      !gzfp::bhost::valid_config(cfg.decompress_cfg) ||
      (cfg.device_queue != 0 && cfg.device_queue != 1) || cfg.idle_exit_us < 1 ||
      cfg.idle_exit_us > 10000000u)
    return sfail(GZFP_ERR_ARG, "bad server configuration");
  for (int i = 0; i < count; i++) {
    const gzfp_serve_request& r = reqs[i];
    if ((r.op != GZFP_SERVE_COMPRESS && r.op != GZFP_SERVE_DECOMPRESS) || !r.input ||
        !gzfp::batch_type_ok(r.type) || output_bytes(r) == 0)
      return sfail(GZFP_ERR_ARG, "bad request");
    results[i] = gzfp_serve_result{0.0, 0.0, output_bytes(r), -1, GZFP_OK, 0.0, 0.0};
  }
  if (stats) memset(stats, 0, sizeof *stats);
  if (count == 0) return GZFP_OK;
  if (cfg.device_queue) return gzfp::serve::serve_queue_run(reqs, count, cfg, results, stats);

  // requests in arrival order
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return reqs[a].arrival < reqs[b].arrival; });

  cudaError_t e;
  char* arena_base = nullptr;
  if ((e = cudaMalloc(&arena_base, cfg.budget_bytes))) return scuda(e, "cudaMalloc(arena)");
  Arena arena(cfg.budget_bytes);
  std::vector<Slot> slots(cfg.max_inflight);
  int st = GZFP_OK;
  for (Slot& sl : slots) {
    if ((e = cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking)) ||
        (e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming))) {
      st = scuda(e, "slot set-up");
      break;
    }
  }

  std::deque<int> queue;
  size_t next = 0;
  int completed = 0, batches = 0, kernels = 0;
  long long batched_reqs = 0, inflight_reqs = 0;
  double inflight_sum = 0;
  double busy_time = 0, busy_since = -1;
  int inflight = 0;
  const Clock::time_point t0 = Clock::now();
  auto now = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };

  while (!st && completed < count) {
    double t = now();
    // completions
    for (Slot& sl : slots) {
      if (!sl.busy) continue;
      e = cudaEventQuery(sl.done);
      if (e == cudaErrorNotReady) continue;
      if (e != cudaSuccess) {
        st = scuda(e, "batch");
        break;
      }
      t = now();
      for (size_t j = 0; j < sl.reqs.size(); j++) {
        results[sl.reqs[j]].completed = t;
        arena.release(sl.offs[j], results[sl.reqs[j]].output_bytes);
      }
      completed += (int)sl.reqs.size();
      inflight_reqs -= (long long)sl.reqs.size();
      sl.busy = false;
      if (--inflight == 0) busy_time += t - busy_since;
    }
    if (st) break;
    // arrivals
    while (next < order.size() && reqs[order[next]].arrival <= t) queue.push_back(order[next++]);
    // launch on one free slot
    Slot* free_slot = nullptr;
    for (Slot& sl : slots)
      if (!sl.busy) {
        free_slot = &sl;
        break;
      }
    if (free_slot && !queue.empty()) {
      Slot& sl = *free_slot;
      sl.reqs.clear();
      sl.offs.clear();
      while (!queue.empty() && (int)sl.reqs.size() < cfg.max_batch) {
        const int r = queue.front();
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
        sl.reqs.push_back(r);
        sl.offs.push_back(off);
      }
      if (!sl.reqs.empty()) {
        std::vector<gzfp_batch_item> items[2];
        for (size_t j = 0; j < sl.reqs.size(); j++) {
          const gzfp_serve_request& r = reqs[sl.reqs[j]];
          void* out = arena_base + sl.offs[j];
          gzfp_batch_item it;
          it.type = r.type;
          it.nx = r.nx;
          it.ny = r.ny;
          it.nz = r.nz;
          it.maxbits = r.maxbits;
          if (r.op == GZFP_SERVE_COMPRESS) {
            it.field = const_cast<void*>(r.input);
            it.stream = out;
            it.stream_capacity = results[sl.reqs[j]].output_bytes;
          } else {
            it.field = out;
            it.stream = const_cast<void*>(r.input);
            it.stream_capacity = gzfp_stream_size(r.type, r.nx, r.ny, r.nz, r.maxbits);
          }
          items[r.op].push_back(it);
        }
        for (int d = 0; d < 2 && !st; d++) {
          if (items[d].empty()) continue;
          const gzfp_batch_config& bc = d ? cfg.decompress_cfg : cfg.compress_cfg;
          gzfp::bhost::Prepared& p = sl.prep[d];
          gzfp::bhost::WorkList& wl = sl.wl[d];
          if ((st = gzfp::bhost::prepare(items[d].data(), (int)items[d].size(), d == 1, bc, p)))
            break;
          // the slot is free, so nothing in flight still reads its work list
          if ((e = wl.reserve(p.descs.size(), p.lay.nchunks))) {
            st = scuda(e, "slot work list");
            break;
          }
          memcpy(wl.host, p.descs.data(), p.descs.size() * sizeof(gzfp::BatchDesc));
          if ((e = gzfp::bhost::enqueue(p, wl, d == 1, bc, sl.s))) st = scuda(e, "batch launch");
          kernels += p.kernels(bc.ctas_per_sm == 0);
        }
        for (size_t j = 0; j < sl.reqs.size() && !st; j++) {
          const gzfp_serve_request& r = reqs[sl.reqs[j]];
          if (r.copy_to &&
              (e = cudaMemcpyAsync(r.copy_to, arena_base + sl.offs[j],
                                   results[sl.reqs[j]].output_bytes, cudaMemcpyDeviceToDevice, sl.s)))
            st = scuda(e, "output copy");
        }
        if (!st && (e = cudaEventRecord(sl.done, sl.s))) st = scuda(e, "cudaEventRecord");
        if (st) break;
        sl.busy = true;
        sl.batch = batches++;
        batched_reqs += (long long)sl.reqs.size();
        inflight_reqs += (long long)sl.reqs.size();  // each of them sees the whole batch
        inflight_sum += (double)sl.reqs.size() * (double)inflight_reqs;
        const double ta = now();
        for (int r : sl.reqs) {
          results[r].admitted = ta;
          results[r].batch = sl.batch;
        }
        if (inflight++ == 0) busy_since = ta;
      }
    }
  }

  const double wall = now();
  for (Slot& sl : slots) {
    if (sl.s) cudaStreamSynchronize(sl.s);  // nothing stays in flight, on success or not
    for (auto& wl : sl.wl) wl.release();
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.s) cudaStreamDestroy(sl.s);
  }
  cudaFree(arena_base);
  if (stats) {
    double last = 0;
    for (int i = 0; i < count; i++) last = std::max(last, results[i].completed);
    stats->wall = st ? wall : last;
    stats->batches = batches;
    stats->mean_batch = batches ? (double)batched_reqs / batches : 0.0;
    stats->peak_bytes = arena.peak();
    stats->busy = stats->wall > 0 ? busy_time / stats->wall : 0.0;
    stats->kernels = kernels;
    stats->mean_inflight = batched_reqs ? inflight_sum / (double)batched_reqs : 0.0;
  }
  return st;
}

}  // extern "C"
