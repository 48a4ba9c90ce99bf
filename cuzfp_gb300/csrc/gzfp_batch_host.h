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

// The layout of a batch's descriptors: per kind its chunk range [lo, hi),
// its staged items in [lo, mid) and the others in [mid, hi); the chunk
// count; the largest words per block staged in shared memory.
struct Layout {
  uint64_t nchunks = 0;
  uint64_t lo[kBatchKinds] = {}, mid[kBatchKinds] = {}, hi[kBatchKinds] = {};
  uint32_t staged_w = 0;
};

// Validate `items` and write one descriptor per item into descs[0..count),
// grouped by kind (kBatchKind order), each kind's staged items first, with
// chunks of chunk_blocks blocks.  No heap use: the no-alloc entry point
// calls it too.  Returns a gzfp status (the detail goes to
// gzfp_batch_last_error).
int layout(const gzfp_batch_item* items, int count, bool decode, uint64_t chunk_blocks,
           BatchDesc* descs, Layout& L);

// Host-side description of a batch: descriptors, their layout, and the
// streams whose blocks share words (zeroed before an encode launch).
struct Prepared {
  std::vector<BatchDesc> descs;
  Layout lay;
  // kernels enqueue launches: the chunk table, and per kind present one
  // persistent kernel or (grid) one grid kernel per non-empty range
  int kernels(bool grid) const {
    int n = lay.nchunks ? 1 : 0;
    for (int k = 0; k < kBatchKinds; k++)
      n += grid ? (lay.mid[k] > lay.lo[k]) + (lay.hi[k] > lay.mid[k]) : lay.hi[k] > lay.lo[k];
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
// the per-kind kernels.
cudaError_t enqueue(const Prepared& p, WorkList& wl, bool decode, const gzfp_batch_config& cfg,
                    cudaStream_t s);

}  // namespace bhost
}  // namespace gzfp
