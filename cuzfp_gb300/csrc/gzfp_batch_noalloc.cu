// gzfp_batch_noalloc.cu -- gzfp_batch_run_noalloc (include/gzfp.h): the
// batched codec with its work list in a fixed, file-scope device
// array instead of memory allocated per call.
//
// The kernels are the batch path's own (gzfp_batch.cuh); only where their
// scratch lives differs.  Scratch layout, one copy per device (a __device__
// array is instantiated in every context that loads the module):
//   [0, 256)                      claim counters, one per kind (zeroed every call)
//   [256, 256 + descs)            array descriptors, uploaded every call
//   [.., + 4 * kNoAllocMaxChunks) chunk -> array table, built on the device
// Nothing here calls cudaMalloc, cudaMallocHost, cudaFree or an allocating
// library, and no host heap is touched: descriptors are built in a static
// host buffer and uploaded with a pageable cudaMemcpyAsync, which the CUDA
// runtime stages through its own buffers and which returns only once the
// host buffer may be reused.
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "gzfp.h"
#include "gzfp_batch_host.h"
#include "gzfp_batch_launch.h"

namespace {

constexpr int kMaxItems = GZFP_NOALLOC_MAX_ITEMS;
constexpr uint64_t kMaxChunks = GZFP_NOALLOC_MAX_CHUNKS;
constexpr size_t kDescOffset = 256;
constexpr size_t kDescBytes = (size_t)kMaxItems * sizeof(gzfp::BatchDesc);
constexpr size_t kTableOffset = (kDescOffset + kDescBytes + 255) / 256 * 256;
constexpr size_t kScratchBytes = kTableOffset + kMaxChunks * sizeof(uint32_t);
static_assert(sizeof(gzfp::BatchDesc) % 8 == 0, "descriptor alignment");

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;                    // guards g_host
gzfp::BatchDesc g_host[kMaxItems];  // descriptors of the call in flight on the host

// failures are reported through gzfp_batch_last_error
int nfail(int status, const char* msg) {
  gzfp::batch_set_error(msg);
  return status;
}

int ncuda(cudaError_t e, const char* what) {
  char msg[256];
  snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
  return nfail(GZFP_ERR_CUDA, msg);
}

}  // namespace

namespace gzfp {
__global__ void batch_chunk_table(const BatchDesc* __restrict__ descs, int count,
                                  uint32_t* chunk_item, uint64_t nchunks);
}

extern "C" int gzfp_batch_run_noalloc(const gzfp_batch_item* items, int count, int decompress,
                                      const gzfp_batch_config* cfg_in, void* cuda_stream) {
  gzfp::batch_set_error("");
  gzfp_batch_config cfg;
  gzfp_batch_default_config(&cfg);
  if (cfg_in) cfg = *cfg_in;
  if (!gzfp::bhost::valid_config(cfg)) return nfail(GZFP_ERR_ARG, "bad batch configuration");
  if (!items || count < 0) return nfail(GZFP_ERR_ARG, "bad item list");
  if (count > kMaxItems) {
    char msg[160];
    snprintf(msg, sizeof msg, "batch of %d arrays exceeds the no-alloc scratch limit of %d arrays",
             count, kMaxItems);
    return nfail(GZFP_ERR_CAPACITY, msg);
  }
  if (count == 0) return GZFP_OK;
  const bool decode = decompress != 0;
  const cudaStream_t s = (cudaStream_t)cuda_stream;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e) return ncuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return nfail(GZFP_ERR_CUDA, "device index out of range");

  // a capture would record the pageable descriptor upload from g_host, and
  // a replay would upload whatever a later call left there
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if ((e = cudaStreamIsCapturing(s, &cap))) return ncuda(e, "cudaStreamIsCapturing");
  if (cap != cudaStreamCaptureStatusNone)
    return nfail(GZFP_ERR_ARG, "the no-alloc batch call cannot be captured in a CUDA graph");

  std::lock_guard<std::mutex> lock(g_mu);
  // the scratch's address in the current context (looked up on every call:
  // the runtime caches it, and a reset context reloads the module)
  void* scratch = nullptr;
  if ((e = cudaGetSymbolAddress(&scratch, g_scratch)))
    return ncuda(e, "cudaGetSymbolAddress(no-alloc scratch)");
  unsigned char* base = (unsigned char*)scratch;
  unsigned long long* counter = (unsigned long long*)base;
  gzfp::BatchDesc* descs = (gzfp::BatchDesc*)(base + kDescOffset);
  uint32_t* chunk_item = (uint32_t*)(base + kTableOffset);

  // descriptors: the allocating batch path's validation and layout, into
  // the host array
  gzfp::bhost::Layout L;
  const int st = gzfp::bhost::layout(items, count, decode,
                                     (uint64_t)cfg.threads * cfg.blocks_per_thread, g_host, L);
  if (st) return st;
  const uint64_t nchunks = L.nchunks, chunk_blocks = (uint64_t)cfg.threads * cfg.blocks_per_thread;
  const uint64_t *lo = L.lo, *mid = L.mid, *hi = L.hi;
  const uint32_t sw = L.staged_w;
  if (nchunks > kMaxChunks) {
    char msg[160];
    snprintf(msg, sizeof msg, "batch needs %llu chunks of %llu blocks; the no-alloc scratch holds %llu",
             (unsigned long long)nchunks, (unsigned long long)chunk_blocks,
             (unsigned long long)kMaxChunks);
    return nfail(GZFP_ERR_CAPACITY, msg);
  }

  // streams whose blocks share edge words are assembled with atomic ORs and
  // must start at zero, as must the claim counters
  if (!decode)
    for (int i = 0; i < count; i++)
      if (g_host[i].maxbits % 64 &&
          (e = cudaMemsetAsync(g_host[i].out, 0, (size_t)(g_host[i].nwords * 8), s)))
        return ncuda(e, "cudaMemsetAsync(stream)");
  if ((e = cudaMemcpyAsync(descs, g_host, count * sizeof(gzfp::BatchDesc), cudaMemcpyHostToDevice,
                           s)))
    return ncuda(e, "cudaMemcpyAsync(descriptors)");
  gzfp::batch_chunk_table<<<dim3(64, (unsigned)count), 256, 0, s>>>(descs, count, chunk_item,
                                                                    nchunks);
  if ((e = cudaGetLastError())) return ncuda(e, "chunk table launch");
  if ((e = cudaMemsetAsync(counter, 0, gzfp::kBatchKinds * sizeof(unsigned long long), s)))
    return ncuda(e, "cudaMemsetAsync(counters)");

  int sms = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)))
    return ncuda(e, "cudaDeviceGetAttribute");
  const bool ahead = cfg.claim_ahead != 0;
  for (int k = 0; k < gzfp::kBatchKinds && !e; k++) {
    if (hi[k] == lo[k]) continue;
    if (cfg.ctas_per_sm == 0) {  // grid kernels: the staged items, then the others
      if (mid[k] > lo[k])
        e = gzfp::launch_batch(cfg.threads, decode, k, 0, cfg.blocks_per_thread, false, sw, descs,
                               chunk_item, lo[k], mid[k], counter + k, s);
      if (!e && hi[k] > mid[k])
        e = gzfp::launch_batch(cfg.threads, decode, k, 0, cfg.blocks_per_thread, false, 0, descs,
                               chunk_item, mid[k], hi[k], counter + k, s);
      continue;
    }
    int occ = gzfp::batch_occupancy(cfg.threads, decode, k, sw);
    occ = occ > 1 ? occ : 1;
    const int grid = sms * (cfg.ctas_per_sm < occ ? cfg.ctas_per_sm : occ);
    e = gzfp::launch_batch(cfg.threads, decode, k, grid, cfg.blocks_per_thread, ahead, sw, descs,
                           chunk_item, lo[k], hi[k], counter + k, s);
  }
  return e ? ncuda(e, "batch kernel launch") : GZFP_OK;
}
