// gzfp_slabs.h -- the slab decomposition of host-staged calls
// (gzfp_api.cu): whole block layers along the slowest axis (z in 3D, y in
// 2D, x in 1D), so many that every slab starts on a 64-bit stream word and
// is coded as an independent array whose stream is exactly the matching
// word range of the whole stream.  Host code only; the CPU tests build it
// on its own.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include "gzfp_array.cuh"

namespace gzfp_host {

constexpr uint64_t kSlabTarget = 32ull << 20;  // field bytes per slab

// Slab decomposition of an array: `layers` block layers of `layer_blocks`
// blocks and 4 planes of `plane_values` values each (the last layer may
// hold fewer than 4 of the axis' `extent` planes), `per_slab` layers a slab.
struct Slabs {
  int dims;
  unsigned nx, ny;
  uint64_t extent, layers, layer_blocks, plane_values, per_slab, count;
};

inline Slabs plan_slabs(const gzfp::Geom& g, int dims, unsigned maxbits, size_t scalar) {
  Slabs p;
  p.dims = dims;
  p.nx = g.nx;
  p.ny = g.ny;
  if (dims == 3) {
    p.extent = g.nz, p.layers = g.bz, p.layer_blocks = (uint64_t)g.bx * g.by;
    p.plane_values = (uint64_t)g.nx * g.ny;
  } else if (dims == 2) {
    p.extent = g.ny, p.layers = g.by, p.layer_blocks = g.bx, p.plane_values = g.nx;
  } else {
    p.extent = g.nx, p.layers = g.bx, p.layer_blocks = 1, p.plane_values = 1;
  }
  // slab boundaries on whole words: per_slab * layer_blocks * maxbits % 64 == 0
  const uint64_t bits = p.layer_blocks * maxbits;
  int tz = 0;
  while (tz < 6 && !((bits >> tz) & 1)) tz++;
  const uint64_t quantum = 64ull >> tz;
  const uint64_t layer_bytes = 4 * p.plane_values * scalar;
  uint64_t per = kSlabTarget / layer_bytes / quantum * quantum;
  if (per < quantum) per = quantum;
  if (per >= p.layers) per = p.layers;
  p.per_slab = per;
  p.count = (p.layers + per - 1) / per;
  return p;
}

// Slab j: first plane, plane count, first block, block count, and the
// array geometry it is coded as.
struct Slab {
  uint64_t plane0, planes, block0, blocks;
  gzfp::Geom g;
};

inline Slab slab_at(const Slabs& p, uint64_t j) {
  Slab s;
  const uint64_t l0 = j * p.per_slab;
  const uint64_t l1 = l0 + p.per_slab < p.layers ? l0 + p.per_slab : p.layers;
  s.plane0 = 4 * l0;
  s.planes = (4 * l1 < p.extent ? 4 * l1 : p.extent) - s.plane0;
  s.block0 = l0 * p.layer_blocks;
  s.blocks = (l1 - l0) * p.layer_blocks;
  const unsigned n = (unsigned)s.planes;
  s.g = p.dims == 3   ? gzfp::make_geom_blocks(p.nx, p.ny, n)
        : p.dims == 2 ? gzfp::make_geom_blocks(p.nx, n, 1)
                      : gzfp::make_geom_blocks(n, 1, 1);
  return s;
}

}  // namespace gzfp_host
