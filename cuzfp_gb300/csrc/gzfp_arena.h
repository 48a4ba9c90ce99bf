// gzfp_arena.h -- the request server's output arena: a first-fit allocator
// of offsets into one device buffer (gzfp_serve.cu, gzfp_serve_queue.cu).
// Plain C++, no CUDA: the CPU tests build it on its own.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <iterator>
#include <map>

namespace gzfp {
namespace serve {

constexpr size_t kAlign = 256;

// First-fit allocator over one arena of `size` bytes; free ranges keyed by
// offset and merged with their neighbours on release.  Sizes are rounded
// up to kAlign, so every offset is a multiple of kAlign.
class Arena {
 public:
  explicit Arena(size_t size) : size_(size) {
    if (size) free_[0] = size;
  }
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
  // give back a range that alloc(bytes) returned at `off`
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
  size_t used() const { return used_; }
  size_t size() const { return size_; }
  // free ranges, for checks: how many, and the largest
  size_t free_ranges() const { return free_.size(); }
  size_t largest_free() const {
    size_t m = 0;
    for (const auto& f : free_) m = std::max(m, f.second);
    return m;
  }

 private:
  size_t size_, used_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
};

}  // namespace serve
}  // namespace gzfp
