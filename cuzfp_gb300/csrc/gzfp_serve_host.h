// gzfp_serve_host.h -- host-side pieces shared by the request server's two
// modes (gzfp_serve.cu: batches on slots; gzfp_serve_queue.cu: a device
// request queue drained by a persistent scheduler kernel).
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <map>

#include "gzfp.h"
#include "gzfp_batch_launch.h"

namespace gzfp {
namespace serve {

constexpr size_t kAlign = 256;

// First-fit allocator over one device arena; free ranges keyed by offset
// and merged with their neighbours on release.
class Arena {
 public:
  explicit Arena(size_t size) : size_(size) { free_[0] = size; }
  // offset of `bytes` (rounded up to kAlign), or SIZE_MAX if nothing fits
  size_t alloc(size_t bytes) {
    bytes = (bytes + kAlign - 1) / kAlign * kAlign;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      const size_t off = it->first, rest = it->second - bytes;
      free_.erase(it);
      if (rest) free_[off + bytes] = rest;
      used_ += bytes;
      peak_ = std::max(peak_, used_);
      return off;
    }
    return SIZE_MAX;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + kAlign - 1) / kAlign * kAlign;
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t peak() const { return peak_; }

 private:
  size_t size_, used_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
};

inline size_t output_bytes(const gzfp_serve_request& r) {
  const unsigned ny = r.ny ? r.ny : 1, nz = r.nz ? r.nz : 1;
  if (r.op == GZFP_SERVE_COMPRESS) return gzfp_stream_size(r.type, r.nx, r.ny, r.nz, r.maxbits);
  return (size_t)r.nx * ny * nz * batch_scalar_size(r.type);
}

// The device-queue mode (gzfp_serve_queue.cu): same contract as
// gzfp_serve_run, for 3D float and double requests.
int serve_queue_run(const gzfp_serve_request* reqs, int count, const gzfp_serve_config& cfg,
                    gzfp_serve_result* results, gzfp_serve_stats* stats);

// error reporting of the serving entry points (gzfp_serve.cu)
int serve_fail(int status, const char* msg);
int serve_cuda(cudaError_t e, const char* what);

}  // namespace serve
}  // namespace gzfp
