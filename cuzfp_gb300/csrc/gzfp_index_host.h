// gzfp_index_host.h -- the host step of the parallel index of a
// general-mode stream (gzfp_modes.cuh, gzfp_modes_api.cu): follow the true
// chain of block starts from segment 0 through the walkers' merges and cut
// it into pieces for the assembly kernel.  Plain C++, no CUDA: the CPU tests
// build it on its own.
#pragma once

#include <stdint.h>

#include <vector>

namespace gzfp {

// One piece of the true chain: `count` block starts that go to offsets
// [dst, dst + count), either copied from a walker's list (src: entry index
// in the lists) or re-walked from a walker's exit (walk = 1, seg: the
// segment whose extension it is).
struct IndexPiece {
  unsigned long long src;
  unsigned long long count;
  unsigned long long dst;
  unsigned long long seg;
  unsigned long long walk;
};

// The walkers' results, per segment s of nseg (lists of at most cap
// entries): counts[s] entries in its list (cap + 1: the list overflowed),
// and info[4 s ..]: extension steps, the segment it merged into, the index
// of the merge start in that segment's list, and a status (0 merged, 1 ran
// to the end of the stream, 2 no merge within the step limit).  Fills
// `pieces` with the chain's first nblocks starts and returns true, or
// returns false when the chain cannot be joined (an overflowed list, a
// failed extension, a merge that does not move forward, fewer starts than
// blocks); the caller then walks the stream serially.
inline bool index_pieces(uint64_t nseg, uint64_t cap, const unsigned long long* counts,
                         const unsigned long long* info, uint64_t nblocks,
                         std::vector<IndexPiece>& pieces) {
  pieces.clear();
  uint64_t dst = 0, seg = 0, start = 0;
  for (uint64_t it = 0; it <= nseg && dst < nblocks; it++) {
    const unsigned long long n = counts[seg];
    if (n > cap) return false;
    if (n > start) {
      pieces.push_back(IndexPiece{seg * cap + start, n - start, dst, 0, 0});
      dst += n - start;
    }
    const unsigned long long* inf = info + 4 * seg;
    if (inf[3] == 2) return false;  // no merge within the extension's cap
    if (inf[0]) {
      pieces.push_back(IndexPiece{0, inf[0], dst, seg, 1});
      dst += inf[0];
    }
    if (inf[3] == 1) break;  // the chain ran to the end of the stream
    if (inf[1] <= seg || inf[1] >= nseg) return false;
    seg = inf[1];
    start = inf[2];
  }
  return dst >= nblocks;  // fewer starts than blocks: the serial walk reports it
}

}  // namespace gzfp
