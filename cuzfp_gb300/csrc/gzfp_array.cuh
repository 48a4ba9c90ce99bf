// gzfp_array.cuh -- array-level pieces of the codec: block geometry, the
// gather / scatter of one block with zfp's edge padding, and the bit writer /
// reader over the fixed-rate stream.  Like gzfp_block.cuh these are
// host+device so the CPU tests run the exact per-thread code of the kernels.
#pragma once

#include "gzfp_block.cuh"

namespace gzfp {

// Geometry of a contiguous a[nz][ny][nx] field cut into 4^D blocks; unused
// axes have size 1.  Blocks are numbered x fastest, then y, then z, the order
// of zfp's block loops (Z/src/template/compress.c:60-104).
// Division of a 32-bit value by a fixed divisor d >= 1 as a multiply-high
// and a shift (round-up method): n / d = (umulhi(n, m) + n) >> s.
struct FastDiv {
  uint32_t d, m, s;
};

GZ_HD FastDiv make_fastdiv(uint32_t d) {
  uint32_t s = 0;
  while ((1ull << s) < d) s++;
  const uint32_t m = (uint32_t)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
  return FastDiv{d, m, s};
}

GZ_HD uint32_t fast_div(uint32_t n, const FastDiv& f) {
#if defined(__CUDA_ARCH__)
  const uint32_t hi = __umulhi(n, f.m);
#else
  const uint32_t hi = (uint32_t)(((uint64_t)n * f.m) >> 32);
#endif
  return (uint32_t)(((uint64_t)hi + n) >> f.s);
}

// Geometry of an nx x ny x nz field cut into 4^D blocks (fewer than 2^32 of
// them); unused axes have size 1.  Value (x, y, z) sits at element
// x*sx + y*sy + z*sz of the field pointer: a contiguous a[nz][ny][nx] has
// (sx, sy, sz) = (1, nx, nx*ny), and zfp's strided fields any signed strides
// (Z/src/template/compress.c, compress_strided).
struct Geom {
  uint32_t nx, ny, nz;
  uint32_t bx, by, bz;  // blocks per axis
  uint64_t nblocks;
  int64_t sx, sy, sz;   // element strides
  uint64_t base;        // stream bit of block 0 (after a header; 0 without)
  uint32_t vec;  // rows of full blocks may be moved as one 16/32-byte vector
  FastDiv dbx, dby;
};

GZ_HD Geom make_geom_blocks(uint32_t nx, uint32_t ny, uint32_t nz) {
  Geom g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.bx = (nx + 3) / 4;
  g.by = (ny + 3) / 4;
  g.bz = (nz + 3) / 4;
  g.nblocks = (uint64_t)g.bx * g.by * g.bz;
  g.sx = 1;
  g.sy = nx;
  g.sz = (int64_t)nx * ny;
  g.base = 0;
  g.vec = 0;
  g.dbx = make_fastdiv(g.bx);
  g.dby = make_fastdiv(g.by);
  return g;
}

GZ_HD void block_coords(const Geom& g, uint64_t b, uint32_t& ix, uint32_t& iy, uint32_t& iz) {
  const uint32_t b32 = (uint32_t)b;
  const uint32_t r = fast_div(b32, g.dbx);
  ix = b32 - r * g.bx;
  iz = fast_div(r, g.dby);
  iy = r - iz * g.by;
}

// zfp's pad_block (Z/src/template/encode.c:55-74) as an index map: with c
// valid values along an axis, padded position p reads position map(c, p):
// c = 3 -> {0,1,2,0}, c = 2 -> {0,1,1,0}, c = 1 -> {0,0,0,0}.  Padding is
// applied x, then y, then z, each copying already padded values, so the
// 3D result is separable.
GZ_HD uint32_t pad_index(uint32_t c, uint32_t p) {
  const uint32_t lut = c >= 4 ? 0xE4u : c == 3 ? 0x24u : c == 2 ? 0x14u : 0x00u;
  return (lut >> (2 * p)) & 3u;
}

GZ_HD uint32_t valid_count(uint32_t n, uint32_t i) {
  uint32_t c = n - 4 * i;
  return c > 4 ? 4 : c;
}

template <typename T>
GZ_HD typename FT<T>::UInt load_bits(const T* p) {
  typedef typename FT<T>::UInt UInt;
#if defined(__CUDA_ARCH__)
  return (UInt)__ldg((const UInt*)p);
#else
  UInt v;
  __builtin_memcpy(&v, p, sizeof v);
  return v;
#endif
}

// Four consecutive values of a row as one vector access (device only; the
// caller guarantees 16-byte (float) / 32-byte (double) alignment).
GZ_HD void load_row(const float* p, uint32_t* r) {
#if defined(__CUDA_ARCH__)
  asm("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "l"(p));
#else
  __builtin_memcpy(r, p, 16);
#endif
}
GZ_HD void load_row(const double* p, uint64_t* r) {
#if defined(__CUDA_ARCH__)
  asm("ld.global.nc.v4.u64 {%0,%1,%2,%3}, [%4];"
      : "=l"(r[0]), "=l"(r[1]), "=l"(r[2]), "=l"(r[3]) : "l"(p));
#else
  __builtin_memcpy(r, p, 32);
#endif
}
GZ_HD void store_row(float* p, const uint32_t* r) {
#if defined(__CUDA_ARCH__)
  asm volatile("st.global.v4.u32 [%0], {%1,%2,%3,%4};"
               :: "l"(p), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]) : "memory");
#else
  __builtin_memcpy(p, r, 16);
#endif
}
GZ_HD void store_row(double* p, const uint64_t* r) {
#if defined(__CUDA_ARCH__)
  asm volatile("st.global.v4.u64 [%0], {%1,%2,%3,%4};"
               :: "l"(p), "l"(r[0]), "l"(r[1]), "l"(r[2]), "l"(r[3]) : "memory");
#else
  __builtin_memcpy(p, r, 32);
#endif
}

// Integer fields move exactly like the floating-point type of the same size.
GZ_HD void load_row(const int32_t* p, uint32_t* r) { load_row((const float*)p, r); }
GZ_HD void load_row(const int64_t* p, uint64_t* r) { load_row((const double*)p, r); }
GZ_HD void store_row(int32_t* p, const uint32_t* r) { store_row((float*)p, r); }
GZ_HD void store_row(int64_t* p, const uint64_t* r) { store_row((double*)p, r); }

// Gather block (ix, iy, iz) as raw IEEE bits, padded at partial edges.
template <int D, typename T>
GZ_HD void gather(const T* in, const Geom& g, uint32_t ix, uint32_t iy, uint32_t iz,
                  typename FT<T>::UInt* raw) {
  const uint32_t cx = valid_count(g.nx, ix);
  const uint32_t cy = D >= 2 ? valid_count(g.ny, iy) : 1;
  const uint32_t cz = D >= 3 ? valid_count(g.nz, iz) : 1;
  const int64_t sx = g.sx, sy = g.sy, sz = g.sz;
  const T* base = in + 4 * (ix * sx + iy * sy + iz * sz);
  constexpr int DY = D >= 2 ? 4 : 1, DZ = D >= 3 ? 4 : 1;
  const bool full = cx == 4 && (D < 2 || cy == 4) && (D < 3 || cz == 4);
  if (full && g.vec) {
#pragma unroll
    for (int z = 0; z < DZ; z++)
#pragma unroll
      for (int y = 0; y < DY; y++) load_row(base + y * sy + z * sz, raw + 16 * z + 4 * y);
  } else if (full) {
#pragma unroll
    for (int z = 0; z < DZ; z++)
#pragma unroll
      for (int y = 0; y < DY; y++)
#pragma unroll
        for (int x = 0; x < 4; x++) raw[16 * z + 4 * y + x] = load_bits(base + x * sx + y * sy + z * sz);
  } else {
#pragma unroll
    for (int z = 0; z < DZ; z++)
#pragma unroll
      for (int y = 0; y < DY; y++)
#pragma unroll
        for (int x = 0; x < 4; x++)
          raw[16 * z + 4 * y + x] =
              load_bits(base + pad_index(cx, x) * sx + pad_index(cy, y) * sy + pad_index(cz, z) * sz);
  }
}

// Store the valid part of block (ix, iy, iz) (Z/src/template/decode3.c:6-25).
template <int D, typename T>
GZ_HD void scatter(T* out, const Geom& g, uint32_t ix, uint32_t iy, uint32_t iz,
                   const typename FT<T>::UInt* raw) {
  typedef typename FT<T>::UInt UInt;
  const uint32_t cx = valid_count(g.nx, ix);
  const uint32_t cy = D >= 2 ? valid_count(g.ny, iy) : 1;
  const uint32_t cz = D >= 3 ? valid_count(g.nz, iz) : 1;
  const int64_t sx = g.sx, sy = g.sy, sz = g.sz;
  UInt* base = (UInt*)out + 4 * (ix * sx + iy * sy + iz * sz);
  constexpr int DY = D >= 2 ? 4 : 1, DZ = D >= 3 ? 4 : 1;
  if (g.vec && cx == 4 && (D < 2 || cy == 4) && (D < 3 || cz == 4)) {
#pragma unroll
    for (int z = 0; z < DZ; z++)
#pragma unroll
      for (int y = 0; y < DY; y++) store_row((T*)base + y * sy + z * sz, raw + 16 * z + 4 * y);
    return;
  }
#pragma unroll
  for (int z = 0; z < DZ; z++)
#pragma unroll
    for (int y = 0; y < DY; y++)
#pragma unroll
      for (int x = 0; x < 4; x++)
        if ((uint32_t)x < cx && (uint32_t)y < cy && (uint32_t)z < cz)
          base[x * sx + y * sy + z * sz] = raw[16 * z + 4 * y + x];
}

// ------------------------------------------------------------- bit writer
// Writes one block's bits, LSB first into 64-bit words, starting at absolute
// bit `pos` of the stream (Z/src/inline/bitstream.c:258-283 word layout).
// Words that another block also touches (the first and last word when the
// block does not start / end on a word boundary) go through `Words::merge`,
// every other word through `Words::store`.
template <class Words, bool ALIGNED = false>
struct BitWriter {
  Words words;
  uint64_t wi;      // index of the word being filled
  uint64_t acc;     // its pending bits
  uint32_t fill;    // number of pending bits
  uint64_t first;   // index of a shared first word, or ~0
  uint64_t last;    // index of a shared last word, or ~0

  GZ_HD BitWriter(Words w, uint64_t pos, uint32_t maxbits) : words(w) {
    wi = pos >> 6;
    fill = (uint32_t)(pos & 63);
    acc = 0;
    uint64_t end = pos + maxbits;
    first = fill ? wi : ~0ull;
    last = (end & 63) ? (end >> 6) : ~0ull;
  }
  GZ_HD void emit() {
    if (!ALIGNED && (wi == first || wi == last))
      words.merge(wi, acc);
    else
      words.store(wi, acc);
    wi++;
  }
  // append the low n (<= 64) bits of v; v has no bits at or above n
  GZ_HD void put(uint64_t v, uint32_t n) {
    acc |= v << fill;  // fill < 64
    const uint32_t f = fill + n;
    if (f >= 64) {
      emit();
      acc = (v >> 1) >> (63 - fill);  // the bits of v that did not fit
      fill = f - 64;
    } else {
      fill = f;
    }
  }
  GZ_HD void zeros(uint32_t n) {
    while (n >= 64) {
      put(0, 64);
      n -= 64;
    }
    if (n) put(0, n);
  }
  // the block ends mid-word: hand over the partial last word
  GZ_HD void finish() {
    if (fill) emit();
  }
};

// ------------------------------------------------------------- bit reader
template <class Words>
struct BitReader {
  Words words;
  uint64_t wi;
  uint64_t w0, w1;
  uint32_t off;

  GZ_HD BitReader(Words w, uint64_t pos) : words(w) {
    wi = pos >> 6;
    off = (uint32_t)(pos & 63);
    w0 = words.load(wi);
    w1 = words.load(wi + 1);
  }
  GZ_HD uint64_t peek64() const {
    // the 64 bits from `off` of (w1:w0): one funnel shift per result word
    const uint32_t a0 = lo32(w0), a1 = hi32(w0), a2 = lo32(w1), a3 = hi32(w1);
    const bool ge = off >= 32;
    const uint32_t s = off & 31;
    const uint32_t b0 = ge ? a1 : a0, b1 = ge ? a2 : a1, b2 = ge ? a3 : a2;
    return ((uint64_t)fshr(b1, b2, s) << 32) | fshr(b0, b1, s);
  }
  GZ_HD void skip(uint32_t n) {  // n <= 64
    off += n;
    if (off >= 64) {
      off -= 64;
      wi++;
      w0 = w1;
      w1 = words.load(wi + 1);
    }
  }
  GZ_HD uint64_t read(uint32_t n) {  // n <= 64
    if (n == 0) return 0;
    uint64_t v = peek64() & lowmask64(n);
    skip(n);
    return v;
  }
};

// ------------------------------------------------------- per-block drivers

template <int D, typename T, bool ALIGNED = false, class Words, class PS>
GZ_HD void encode_one(const T* in, const Geom& g, uint64_t b, uint32_t maxbits, Words words,
                      PS& ps) {
  typedef typename FT<T>::UInt UInt;
  constexpr int BS = 1 << (2 * D);
  uint32_t ix, iy, iz;
  block_coords(g, b, ix, iy, iz);
  UInt raw[BS];
  gather<D, T>(in, g, ix, iy, iz, raw);
  BitWriter<Words, ALIGNED> w(words, g.base + b * (uint64_t)maxbits, maxbits);
  encode_block<D, T>(raw, maxbits, w, ps);
  w.finish();
}

template <int D, typename T, class Words, class PS>
GZ_HD void decode_one(T* out, const Geom& g, uint64_t b, uint32_t maxbits, Words words, PS& ps) {
  typedef typename FT<T>::UInt UInt;
  constexpr int BS = 1 << (2 * D);
  uint32_t ix, iy, iz;
  block_coords(g, b, ix, iy, iz);
  BitReader<Words> r(words, g.base + b * (uint64_t)maxbits);
  if constexpr (D == 3 && !FT<T>::INT && sizeof(T) == 8) {
    // 4^3 double blocks hand over their values one z slice at a time, so
    // that the inverse transform does not keep all 64 values live (the
    // register budget of the 4-CTA decoder spills otherwise)
    const uint32_t cx = valid_count(g.nx, ix), cy = valid_count(g.ny, iy),
                   cz = valid_count(g.nz, iz);
    const int64_t sx = g.sx, sy = g.sy, sz = g.sz;
    UInt* base = (UInt*)out + 4 * (ix * sx + iy * sy + iz * sz);
    const bool vec = g.vec && cx == 4 && cy == 4 && cz == 4;
    decode_block_mode<3, T, true>(r, FixedRate{maxbits}, nullptr, ps, [&](int z, const UInt* rs) {
      if (vec) {
#pragma unroll
        for (int y = 0; y < 4; y++) store_row((T*)base + y * sy + z * sz, rs + 4 * y);
      } else {
#pragma unroll
        for (int y = 0; y < 4; y++)
#pragma unroll
          for (int x = 0; x < 4; x++)
            if ((uint32_t)x < cx && (uint32_t)y < cy && (uint32_t)z < cz)
              base[x * sx + y * sy + z * sz] = rs[4 * y + x];
      }
    });
    return;
  }
  UInt raw[BS];
  decode_block<D, T>(r, maxbits, raw, ps);
  scatter<D, T>(out, g, ix, iy, iz, raw);
}

}  // namespace gzfp
