// gzfp_serve_host.h -- host-side pieces shared by the request server's two
// modes (gzfp_serve.cu: batches on slots; gzfp_serve_queue.cu: a device
// request queue drained by a persistent scheduler kernel).
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <map>

#include "gzfp.h"
#include "gzfp_arena.h"
#include "gzfp_batch_launch.h"

namespace gzfp {
namespace serve {

inline size_t output_bytes(const gzfp_serve_request& r) {
  const unsigned ny = r.ny ? r.ny : 1, nz = r.nz ? r.nz : 1;
  if (r.op == GZFP_SERVE_COMPRESS) return gzfp_stream_size(r.type, r.nx, r.ny, r.nz, r.maxbits);
  return (size_t)r.nx * ny * nz * batch_scalar_size(r.type);
}

// The device-queue mode (gzfp_serve_queue.cu): same contract as
// gzfp_serve_run.
int serve_queue_run(const gzfp_serve_request* reqs, int count, const gzfp_serve_config& cfg,
                    gzfp_serve_result* results, gzfp_serve_stats* stats);

// error reporting of the serving entry points (gzfp_serve.cu)
int serve_fail(int status, const char* msg);
int serve_cuda(cudaError_t e, const char* what);

}  // namespace serve
}  // namespace gzfp
