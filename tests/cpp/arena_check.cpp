// Randomised check of the request server's output arena (gzfp_arena.h)
// against a model: the live allocations as intervals.  Prints "ok" and
// exits 0 when every property holds, else names the first failure.
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <random>
#include <vector>

#include "gzfp_arena.h"

using gzfp::serve::Arena;
using gzfp::serve::kAlign;

struct Live {
  size_t off, bytes, rounded;
};

static int fail(const char* what, size_t a, size_t b) {
  printf("FAIL %s (%zu, %zu)\n", what, a, b);
  return 1;
}

// the lowest offset where `need` bytes fit between the live ranges, or SIZE_MAX
static size_t first_fit(const std::vector<Live>& live, size_t size, size_t need) {
  std::vector<Live> s = live;
  std::sort(s.begin(), s.end(), [](const Live& a, const Live& b) { return a.off < b.off; });
  size_t at = 0;
  for (const Live& l : s) {
    if (l.off >= at && l.off - at >= need) return at;
    at = std::max(at, l.off + l.rounded);
  }
  return size >= at && size - at >= need ? at : SIZE_MAX;
}

static int run(unsigned seed, size_t size, size_t max_request, int steps) {
  std::mt19937_64 rng(seed);
  Arena arena(size);
  std::vector<Live> live;
  size_t used = 0, peak = 0;
  for (int step = 0; step < steps; step++) {
    const bool grow = live.empty() || rng() % 100 < 55;
    if (grow) {
      const size_t bytes = 1 + rng() % max_request;
      const size_t rounded = (bytes + kAlign - 1) / kAlign * kAlign;
      const size_t expect = first_fit(live, size, rounded);
      const size_t off = arena.alloc(bytes);
      if (off != expect) return fail("not the first fit", off, expect);
      if (off == SIZE_MAX) continue;
      if (off % kAlign) return fail("unaligned offset", off, kAlign);
      if (off + rounded > size) return fail("past the end", off, rounded);
      for (const Live& l : live)
        if (off < l.off + l.rounded && l.off < off + rounded) return fail("overlap", off, l.off);
      live.push_back({off, bytes, rounded});
      used += rounded;
      peak = std::max(peak, used);
    } else {
      const size_t i = rng() % live.size();
      arena.release(live[i].off, live[i].bytes);
      used -= live[i].rounded;
      live[i] = live.back();
      live.pop_back();
    }
    if (arena.used() != used) return fail("used", arena.used(), used);
    if (arena.peak() != peak) return fail("peak", arena.peak(), peak);
  }
  // everything back: one free range, the whole arena
  for (const Live& l : live) arena.release(l.off, l.bytes);
  if (arena.used() != 0) return fail("used after release", arena.used(), 0);
  if (arena.free_ranges() != 1 || arena.largest_free() != size)
    return fail("ranges not merged", arena.free_ranges(), arena.largest_free());
  // and a request of the whole arena fits again, one more byte does not
  if (arena.alloc(size) != 0) return fail("whole arena", 0, size);
  if (arena.alloc(1) != SIZE_MAX) return fail("full arena", 1, 0);
  return 0;
}

int main() {
  int bad = 0;
  // small arenas with requests near their size (frequent refusals and
  // fragmentation), larger ones with small requests (many ranges)
  for (unsigned seed = 1; seed <= 40 && !bad; seed++) {
    bad |= run(seed, 64 * kAlign, 20 * kAlign, 4000);
    bad |= run(1000 + seed, 4096 * kAlign, 40 * kAlign + 17, 4000);
    bad |= run(2000 + seed, 7 * kAlign, kAlign + 1, 2000);
  }
  if (!bad) printf("ok\n");
  return bad;
}
