// gzfp_batch_noalloc.cu -- gzfp_batch_run_noalloc (include/gzfp.h): the
// batched persistent codec with its work list in a fixed, file-scope device
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
void* g_scratch_addr[kMaxDevices];  // per device, set once
std::mutex g_mu;                    // guards g_scratch_addr and g_host
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

  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if ((e = cudaGetSymbolAddress(&p, g_scratch)))
      return ncuda(e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_scratch_addr[dev] = p;
  }
  unsigned char* base = (unsigned char*)g_scratch_addr[dev];
  unsigned long long* counter = (unsigned long long*)base;
  gzfp::BatchDesc* descs = (gzfp::BatchDesc*)(base + kDescOffset);
  uint32_t* chunk_item = (uint32_t*)(base + kTableOffset);

  // descriptors: the same validation and layout as the allocating batch
  // path -- grouped by kind, so each kind's chunks form one range
  const uint64_t chunk_blocks = (uint64_t)cfg.threads * cfg.blocks_per_thread;
  for (int i = 0; i < count; i++) {
    const gzfp_batch_item& it = items[i];
    if (!gzfp::batch_type_ok(it.type)) return nfail(GZFP_ERR_UNSUPPORTED, "unknown scalar type");
    if (it.nx == 0 || (it.nz != 0 && it.ny == 0)) return nfail(GZFP_ERR_ARG, "bad dimensions");
    if (!it.field || !it.stream) return nfail(GZFP_ERR_ARG, "null pointer");
    if (it.maxbits < gzfp::batch_ebits(it.type) + 1 || it.maxbits > (1u << 20))
      return nfail(GZFP_ERR_ARG, "bits per block out of range");
    const gzfp::Geom g = gzfp::make_geom_blocks(it.nx, it.ny ? it.ny : 1, it.nz ? it.nz : 1);
    if (g.nblocks >= (1ull << 32)) return nfail(GZFP_ERR_ARG, "too many blocks");
    if (it.stream_capacity < (g.nblocks * it.maxbits + 63) / 64 * 8)
      return nfail(decode ? GZFP_ERR_ARG : GZFP_ERR_CAPACITY, "stream buffer too small");
  }
  uint64_t nchunks = 0;
  // per kind: staged items in [lo, mid), the others in [mid, hi), as the
  // allocating path groups them
  uint64_t lo[gzfp::kBatchKinds], mid[gzfp::kBatchKinds], hi[gzfp::kBatchKinds];
  uint32_t sw = 0;  // staging depth, as the allocating path chooses it
  int slot = 0;
  for (int k = 0; k < gzfp::kBatchKinds; k++) {
    lo[k] = mid[k] = nchunks;
    for (int pass = 0; pass < 2; pass++) {
      if (pass == 1) mid[k] = nchunks;
      for (int i = 0; i < count; i++) {
      const gzfp_batch_item& it = items[i];
      const int dims = it.nz ? 3 : it.ny ? 2 : 1;
      const uint32_t kind = gzfp::batch_kind(it.type, dims);
      if (kind != gzfp::kBatchKind[k]) continue;
      if ((gzfp::batch_item_staged_w(decode, it.maxbits) != 0) != (pass == 0)) continue;
      gzfp::BatchDesc& d = g_host[slot++];
      d.g = gzfp::make_geom_blocks(it.nx, it.ny ? it.ny : 1, it.nz ? it.nz : 1);
      d.g.vec =
          (it.nx % 4 == 0 && (uintptr_t)it.field % gzfp::batch_row_align(it.type) == 0) ? 1u : 0u;
      d.nwords = (d.g.nblocks * it.maxbits + 63) / 64;
      d.maxbits = it.maxbits;
      d.kind = kind;
      d.in = decode ? it.stream : it.field;
      d.out = decode ? it.field : it.stream;
      d.first_chunk = nchunks;
      nchunks += (d.g.nblocks + chunk_blocks - 1) / chunk_blocks;
      const uint32_t w = gzfp::batch_item_staged_w(decode, it.maxbits);
      sw = w > sw ? w : sw;
      }
    }
    hi[k] = nchunks;
  }
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
