// gzfp_batch_host.h -- host-side building blocks of the batched path,
// shared by the batch entry points (gzfp_batch.cu) and the request server
// (gzfp_serve.cu).
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <vector>

#include "gzfp.h"
#include "gzfp_batch_launch.h"

namespace gzfp {
namespace bhost {

// Host-side description of a batch: descriptors, chunk count, and the
// streams whose blocks share words (zeroed before an encode launch).
struct Prepared {
  std::vector<BatchDesc> descs;  // grouped by kind (kBatchKind order)
  uint64_t nchunks = 0;
  // each kind's chunk range [lo, hi): its staged items in [lo, mid), the
  // others in [mid, hi)
  uint64_t kind_lo[kBatchKinds] = {}, kind_mid[kBatchKinds] = {}, kind_hi[kBatchKinds] = {};
  uint32_t staged_w = 0;  // largest words per block staged in shared memory
  // kernels enqueue launches: the chunk table, and per kind present one
  // persistent kernel or (grid) one grid kernel per non-empty range
  int kernels(bool grid) const {
    int n = nchunks ? 1 : 0;
    for (int k = 0; k < kBatchKinds; k++)
      n += grid ? (kind_mid[k] > kind_lo[k]) + (kind_hi[k] > kind_mid[k]) : kind_hi[k] > kind_lo[k];
    return n;
  }
  std::vector<std::pair<void*, size_t>> zero;
};

// Validate `items` and describe them for one direction and launch shape.
// Returns a gzfp status (the detail goes to gzfp_batch_last_error).
int prepare(const gzfp_batch_item* items, int count, bool decode, const gzfp_batch_config& cfg,
            Prepared& p);

bool valid_config(const gzfp_batch_config& c);

// Device work list of one batch in flight: descriptors, chunk table and
// one claim counter per kind, a pinned host copy of the descriptors, and an event
// recorded after the batch's kernel so that the next user of the list can
// wait for it.
struct WorkList {
  BatchDesc* descs = nullptr;
  BatchDesc* host = nullptr;  // pinned
  size_t desc_cap = 0;
  uint32_t* chunk_item = nullptr;
  size_t chunk_cap = 0;
  unsigned long long* counter = nullptr;
  cudaEvent_t done = nullptr;

  cudaError_t reserve(size_t ndesc, size_t nchunks);
  void release();
};

// Queue one prepared batch on stream s: zeroing, descriptor upload from
// wl.host (which must already hold p.descs), chunk table, counter reset and
// the persistent kernel.
cudaError_t enqueue(const Prepared& p, WorkList& wl, bool decode, const gzfp_batch_config& cfg,
                    cudaStream_t s);

}  // namespace bhost
}  // namespace gzfp
