// Properties of the host-staged calls' slab decomposition (gzfp_slabs.h)
// over many shapes, bit budgets and scalar sizes: the slabs tile the block
// layers and the planes exactly once, every slab's blocks start on a 64-bit
// stream word, each slab's own geometry holds exactly its blocks, its
// stream is the matching word range of the whole stream, and a slab stays
// within the size target unless one alignment quantum of layers exceeds
// it.  Prints "ok" and exits 0, else names the first failure.
#include <stdio.h>

#include <random>

#include "gzfp_slabs.h"

typedef unsigned long long u64;

static int fail(const char* what, u64 a, u64 b, u64 c) {
  printf("FAIL %s (%llu, %llu, %llu)\n", what, a, b, c);
  return 1;
}

static int check(unsigned nx, unsigned ny, unsigned nz, int dims, unsigned maxbits, size_t scalar) {
  const gzfp::Geom g = gzfp::make_geom_blocks(nx, ny ? ny : 1, nz ? nz : 1);
  const gzfp_host::Slabs p = gzfp_host::plan_slabs(g, dims, maxbits, scalar);
  const u64 words = (g.nblocks * maxbits + 63) / 64;
  u64 layers = 0, planes = 0, blocks = 0, w_end = 0;
  for (u64 j = 0; j < p.count; j++) {
    const gzfp_host::Slab s = gzfp_host::slab_at(p, j);
    if (s.plane0 != planes) return fail("planes not contiguous", j, s.plane0, planes);
    if (s.block0 != blocks) return fail("blocks not contiguous", j, s.block0, blocks);
    if (s.block0 * maxbits % 64) return fail("slab not word-aligned", j, s.block0, maxbits);
    if (s.g.nblocks != s.blocks) return fail("slab geometry", j, s.g.nblocks, s.blocks);
    const u64 w0 = s.block0 * maxbits / 64, nw = (s.blocks * maxbits + 63) / 64;
    if (w0 != w_end) return fail("stream words not contiguous", j, w0, w_end);
    w_end = w0 + nw;
    planes += s.planes;
    blocks += s.blocks;
    layers += s.blocks / p.layer_blocks;
    const u64 bytes = s.planes * p.plane_values * scalar;
    const u64 quantum_layers = 64;  // at most 64 layers make any slab word-aligned
    if (bytes > gzfp_host::kSlabTarget && p.per_slab > quantum_layers)
      return fail("slab above target", j, bytes, p.per_slab);
  }
  if (planes != p.extent) return fail("planes not covered", planes, p.extent, 0);
  if (blocks != g.nblocks) return fail("blocks not covered", blocks, g.nblocks, 0);
  if (layers != p.layers) return fail("layers not covered", layers, p.layers, 0);
  if (w_end != words) return fail("stream size", w_end, words, 0);
  return 0;
}

int main() {
  std::mt19937_64 rng(7);
  const size_t scalars[] = {4, 8};
  int n = 0;
  for (int it = 0; it < 20000; it++) {
    const int dims = 1 + (int)(rng() % 3);
    const size_t scalar = scalars[rng() % 2];
    unsigned nx, ny = 0, nz = 0;
    if (dims == 1) {
      nx = 1 + (unsigned)(rng() % ((it % 50 == 0) ? (1u << 28) : 200000u));
    } else if (dims == 2) {
      nx = 1 + (unsigned)(rng() % 5000);
      ny = 1 + (unsigned)(rng() % 5000);
    } else {
      nx = 1 + (unsigned)(rng() % 400);
      ny = 1 + (unsigned)(rng() % 400);
      nz = 1 + (unsigned)(rng() % 400);
    }
    const unsigned values = 1u << (2 * dims);
    // any budget from the smallest header to 64 bits a value
    const unsigned maxbits = 1 + (unsigned)(rng() % (values * 64));
    if (check(nx, ny, nz, dims, maxbits, scalar)) return 1;
    n++;
  }
  // the configurations the bench and the tests use
  if (check(512, 512, 512, 3, 1024, 8) || check((1u << 28) - 3, 0, 0, 1, 48, 4) ||
      check(16381, 16383, 0, 2, 192, 4) || check(301, 257, 203, 3, 467, 4))
    return 1;
  printf("ok\n");
  return n > 0 ? 0 : 1;
}
