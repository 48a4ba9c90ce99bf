// CPU model of the parallel index of a general-mode stream: synthetic
// streams where the block at bit p is step(p) bits long, walkers and their
// extensions as the kernels run them (gzfp_modes.cuh, index_walk_kernel),
// the host's chain resolution itself (gzfp_index_host.h), and the
// assembly.  Checks that the resolved offsets are the true chain from bit
// 0, and that the resolver refuses what it must (overflowed lists, failed
// extensions).  Prints "ok" and exits 0, else names the first failure.
#include <stdio.h>

#include <algorithm>
#include <random>
#include <vector>

#include "gzfp_index_host.h"

using gzfp::IndexPiece;
typedef unsigned long long u64;

struct Stream {
  u64 total;                    // bits
  std::vector<uint32_t> len;    // block length at every bit (>= 1)
  u64 step(u64 p) const { return p < total ? len[p] : 1; }
};

struct Walk {
  u64 nseg, cap, seg_bits, ext_cap;
  std::vector<u64> lists, counts, exits, info;
};

static Walk run_walkers(const Stream& st, u64 nseg, u64 cap, u64 ext_cap) {
  Walk w{nseg, cap, (st.total + nseg - 1) / nseg, ext_cap, {}, {}, {}, {}};
  w.lists.assign(nseg * cap, 0);
  w.counts.assign(nseg, 0);
  w.exits.assign(nseg, 0);
  w.info.assign(4 * nseg, 0);
  for (u64 s = 0; s < nseg; s++) {  // segment walks
    const u64 lo = s * w.seg_bits, hi = lo + w.seg_bits;
    u64 p = lo, n = 0;
    while (p < hi && p < st.total) {
      if (n == cap) {
        n = cap + 1;
        break;
      }
      w.lists[s * cap + n++] = p;
      p += st.step(p);
    }
    w.counts[s] = n;
    w.exits[s] = p;
  }
  for (u64 s = 0; s < nseg; s++) {  // extensions
    u64 p = w.exits[s], steps = 0, k = s + 1, idx = 0, status = 2;
    if (w.counts[s] <= cap) {
      for (;;) {
        if (p >= st.total || k >= nseg) {
          status = 1;
          break;
        }
        while (k + 1 < nseg && p >= (k + 1) * w.seg_bits) k++;
        const u64 n = w.counts[k];
        if (n > cap) break;
        const u64* list = &w.lists[k * cap];
        const u64* f = std::lower_bound(list, list + n, p);
        if (f != list + n && *f == p) {
          idx = (u64)(f - list);
          status = 0;
          break;
        }
        if (steps == ext_cap) break;
        steps++;
        p += st.step(p);
      }
    }
    w.info[4 * s] = steps;
    w.info[4 * s + 1] = k;
    w.info[4 * s + 2] = idx;
    w.info[4 * s + 3] = status;
  }
  return w;
}

static std::vector<u64> assemble(const Stream& st, const Walk& w,
                                 const std::vector<IndexPiece>& pieces, u64 nblocks) {
  std::vector<u64> off(nblocks, ~0ull);
  for (const IndexPiece& pc : pieces) {
    if (!pc.walk) {
      for (u64 i = 0; i < pc.count && pc.dst + i < nblocks; i++) off[pc.dst + i] = w.lists[pc.src + i];
    } else {
      u64 p = w.exits[pc.seg];
      for (u64 i = 0; i < pc.count && pc.dst + i < nblocks; i++) {
        off[pc.dst + i] = p;
        p += st.step(p);
      }
    }
  }
  return off;
}

static int fail(const char* what, u64 a, u64 b) {
  printf("FAIL %s (%llu, %llu)\n", what, a, b);
  return 1;
}

int main() {
  int cases = 0, joined = 0;
  for (unsigned seed = 1; seed <= 300; seed++) {
    std::mt19937_64 rng(seed);
    // block lengths: mostly near a mean, so chains started anywhere merge
    // after a while; the first block's start is bit 0
    const u64 mean = 8 + rng() % 120, total = 20000 + rng() % 200000;
    Stream st{total, std::vector<uint32_t>(total)};
    for (u64 p = 0; p < total; p++) st.len[p] = (uint32_t)(1 + mean / 2 + rng() % mean);
    std::vector<u64> truth;
    for (u64 p = 0; p < total; p += st.step(p)) truth.push_back(p);
    const u64 nblocks = truth.size();
    const u64 nseg = 1 + rng() % 64;
    const u64 per = (nblocks + nseg - 1) / nseg;
    const u64 cap = (seed % 7 == 0) ? std::max<u64>(1, per / 3) : 4 * per + 256;  // some overflow
    const u64 ext_cap = (seed % 11 == 0) ? 2 : 16384;                          // some fail
    const Walk w = run_walkers(st, nseg, cap, ext_cap);
    std::vector<IndexPiece> pieces;
    const bool ok = gzfp::index_pieces(nseg, cap, w.counts.data(), w.info.data(), nblocks, pieces);
    cases++;
    // refusals: the first segment on the true chain (0) overflowed, or its
    // chain hit a failed merge; otherwise joined
    if (!ok) {
      bool must = false;
      for (u64 s = 0; s < nseg; s++) must |= w.counts[s] > cap || w.info[4 * s + 3] == 2;
      if (!must) return fail("refused a joinable chain", seed, nseg);
      continue;
    }
    joined++;
    const std::vector<u64> off = assemble(st, w, pieces, nblocks);
    for (u64 b = 0; b < nblocks; b++)
      if (off[b] != truth[b]) return fail("offset differs from the true chain", seed, b);
  }
  if (joined < cases / 2) return fail("too few joined cases", joined, cases);
  printf("ok\n");
  return 0;
}
