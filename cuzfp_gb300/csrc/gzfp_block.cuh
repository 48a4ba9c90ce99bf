// gzfp_block.cuh -- per-block ZFP fixed-rate codec, one thread per block.
//
// Every function here works on one 4^d block held in registers.  It is
// written once and compiled for sm_103a by nvcc (the product kernels in
// gzfp_kernels.cu); the same source also builds for the host so the CPU
// test suite can check the block logic against the oracle without a GPU.
//
// Arithmetic follows zfp 0.5.0 as vendored by cuZFP
// (src/thirdparty_builtin/zfp-0.5.0, abbreviated Z/) step for step; the GPU
// formulation differs in how the work is organised, not in what is computed:
//   * the common exponent is read from the IEEE exponent fields instead of
//     frexp (Z/src/template/encode.c:10-33);
//   * f64 quantisation shifts the significand instead of multiplying by
//     ldexp(1, 62 - emax) (encode.c:36-52), because GB300's FP64 pipe runs
//     at a small fraction of its integer rate; the result is identical;
//   * bit planes are obtained by transposing 32x32 (or SIMD 16x16 / 4x4)
//     bit matrices in registers instead of the per-plane gather loop of
//     encode_ints (encode.c:133-137);
//   * the group-test coder of encode_ints / decode_ints (encode.c:122-151,
//     Z/src/template/decode.c:73-105) is evaluated one run of zeros at a
//     time with count-trailing-zeros instead of one bit at a time.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define GZ_HD __host__ __device__ __forceinline__
#define GZ_CX __host__ __device__ constexpr
#else
#define GZ_HD inline
#define GZ_CX constexpr
#endif

namespace gzfp {

// ------------------------------------------------------------ bit helpers

GZ_HD uint64_t shr64(uint64_t v, uint32_t s) { return s < 64 ? v >> s : 0; }
GZ_HD uint64_t shl64(uint64_t v, uint32_t s) { return s < 64 ? v << s : 0; }
GZ_HD uint64_t lowmask64(uint32_t n) { return n >= 64 ? ~0ull : (1ull << n) - 1; }

// number of trailing zeros; 64 for zero
GZ_HD uint32_t ctz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__clzll((long long)__brevll(x));
#else
  return x ? (uint32_t)__builtin_ctzll(x) : 64u;
#endif
}
GZ_HD uint32_t ctz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__clz((int)__brev(x));
#else
  return x ? (uint32_t)__builtin_ctz(x) : 32u;
#endif
}
GZ_HD int popcount64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}
// number of leading zeros; 64 for zero
GZ_HD uint32_t clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__clzll((long long)x);
#else
  return x ? (uint32_t)__builtin_clzll(x) : 64u;
#endif
}

GZ_HD uint32_t clz32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__clz((int)x);
#else
  return x ? (uint32_t)__builtin_clz(x) : 32u;
#endif
}
GZ_HD uint32_t popcount32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__popc(x);
#else
  return (uint32_t)__builtin_popcount(x);
#endif
}

GZ_HD uint32_t umin(uint32_t a, uint32_t b) { return a < b ? a : b; }
GZ_HD uint32_t lo32(uint64_t v) { return (uint32_t)v; }
GZ_HD uint32_t hi32(uint64_t v) { return (uint32_t)(v >> 32); }

// ----------------------------------------------------------- scalar traits

template <typename T>
struct FT;

template <>
struct FT<float> {
  typedef uint32_t UInt;
  typedef int32_t Int;
  static constexpr bool INT = false;  // integer field: no exponent, no cast
  static constexpr int P = 32;       // integer precision
  static constexpr int EBITS = 8;    // exponent bits (Z/src/traitsf.h)
  static constexpr int EBIAS = 127;  // (1 << (EBITS - 1)) - 1
  static constexpr int MANT = 23;    // stored significand bits
  static constexpr int EMAXF = 127;  // largest finite unbiased exponent
  static constexpr uint32_t NB = 0xaaaaaaaau;  // negabinary mask
};

template <>
struct FT<double> {
  typedef uint64_t UInt;
  typedef int64_t Int;
  static constexpr bool INT = false;
  static constexpr int P = 64;
  static constexpr int EBITS = 11;  // Z/src/traitsd.h
  static constexpr int EBIAS = 1023;
  static constexpr int MANT = 52;
  static constexpr int EMAXF = 1023;
  static constexpr uint64_t NB = 0xaaaaaaaaaaaaaaaaull;
};

// Integer fields (zfp_type_int32 / int64): the values are the block's
// integers; zfp codes them with no exponent and no cast, over the whole
// budget, with maxprec 64 so every plane is eligible
// (Z/src/template/encode.c:154-185, decode.c:107-135).
template <>
struct FT<int32_t> {
  typedef uint32_t UInt;
  typedef int32_t Int;
  static constexpr bool INT = true;
  static constexpr int P = 32;
  static constexpr uint32_t NB = 0xaaaaaaaau;
};

template <>
struct FT<int64_t> {
  typedef uint64_t UInt;
  typedef int64_t Int;
  static constexpr bool INT = true;
  static constexpr int P = 64;
  static constexpr uint64_t NB = 0xaaaaaaaaaaaaaaaaull;
};

constexpr int kMinExp = -1074;  // ZFP_MIN_EXP (Z/inc/zfp.h:80)

// ------------------------------------------------------------ permutations
// Coefficient orders of Z/src/template/codec{1,2,3}.c (perm_1/2/3): a fixed
// part of the stream format, so the tables are kept value for value.

template <int D>
struct Perm;
template <>
struct Perm<1> {
  static GZ_HD constexpr int at(int i) { return i; }
};
template <>
struct Perm<2> {
  static GZ_HD constexpr int at(int i) {
    switch (i) {
      case 0: return 0; case 1: return 1; case 2: return 4; case 3: return 5; case 4: return 2; case 5: return 8;
      case 6: return 6; case 7: return 9; case 8: return 3; case 9: return 12; case 10: return 10; case 11: return 7;
      case 12: return 13; case 13: return 11; case 14: return 14; case 15: return 15;
      default: return 0;
    }
  }
};
template <>
struct Perm<3> {
  static GZ_HD constexpr int at(int i) {
    switch (i) {
      case 0: return 0; case 1: return 1; case 2: return 4; case 3: return 16; case 4: return 20; case 5: return 17;
      case 6: return 5; case 7: return 2; case 8: return 8; case 9: return 32; case 10: return 21; case 11: return 6;
      case 12: return 18; case 13: return 24; case 14: return 9; case 15: return 33; case 16: return 36; case 17: return 3;
      case 18: return 12; case 19: return 48; case 20: return 22; case 21: return 25; case 22: return 37; case 23: return 40;
      case 24: return 34; case 25: return 10; case 26: return 7; case 27: return 19; case 28: return 28; case 29: return 13;
      case 30: return 49; case 31: return 52; case 32: return 41; case 33: return 38; case 34: return 26; case 35: return 23;
      case 36: return 29; case 37: return 53; case 38: return 11; case 39: return 35; case 40: return 44; case 41: return 14;
      case 42: return 50; case 43: return 56; case 44: return 42; case 45: return 27; case 46: return 39; case 47: return 45;
      case 48: return 30; case 49: return 54; case 50: return 57; case 51: return 60; case 52: return 51; case 53: return 15;
      case 54: return 43; case 55: return 46; case 56: return 58; case 57: return 61; case 58: return 55; case 59: return 31;
      case 60: return 62; case 61: return 59; case 62: return 47; case 63: return 63;
      default: return 0;
    }
  }
};


// ----------------------------------------------------------------- lifting

// Wrap-around integer arithmetic.  zfp writes these steps on signed ints,
// whose overflow C leaves undefined; two's-complement wrap is what its
// builds compute, and integer fields near the type limits do overflow.
GZ_HD int32_t add_(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
GZ_HD int32_t sub_(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
GZ_HD int32_t shl1_(int32_t a) { return (int32_t)((uint32_t)a << 1); }
GZ_HD int64_t add_(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }
GZ_HD int64_t sub_(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
GZ_HD int64_t shl1_(int64_t a) { return (int64_t)((uint64_t)a << 1); }

// zfp's lifting steps (Z/src/template/encode.c:77-103, decode.c:28-54) in
// two's-complement wrap-around arithmetic with arithmetic right shifts.
template <typename Int>
GZ_HD void fwd_lift(Int& x, Int& y, Int& z, Int& w) {
  x = add_(x, w); x >>= 1; w = sub_(w, x);
  z = add_(z, y); z >>= 1; y = sub_(y, z);
  x = add_(x, z); x >>= 1; z = sub_(z, x);
  w = add_(w, y); w >>= 1; y = sub_(y, w);
  w = add_(w, (Int)(y >> 1)); y = sub_(y, (Int)(w >> 1));
}

template <typename Int>
GZ_HD void inv_lift(Int& x, Int& y, Int& z, Int& w) {
  y = add_(y, (Int)(w >> 1)); w = sub_(w, (Int)(y >> 1));
  y = add_(y, w); w = shl1_(w); w = sub_(w, y);
  z = add_(z, x); x = shl1_(x); x = sub_(x, z);
  y = add_(y, z); z = shl1_(z); z = sub_(z, y);
  w = add_(w, x); x = shl1_(x); x = sub_(x, w);
}

// decorrelating transform: lines along x (stride 1), y (stride 4), z (16)
template <int D, typename Int>
GZ_HD void fwd_xform(Int* q) {
  constexpr int L = 1 << (2 * (D - 1));  // lines per axis
#pragma unroll
  for (int a = 0; a < D; a++) {
    const int s = 1 << (2 * a);
#pragma unroll
    for (int l = 0; l < L; l++) {
      const int base = (l % s) + (l / s) * s * 4;
      fwd_lift(q[base], q[base + s], q[base + 2 * s], q[base + 3 * s]);
    }
  }
}

template <int D, typename Int>
GZ_HD void inv_xform(Int* q) {
  constexpr int L = 1 << (2 * (D - 1));
#pragma unroll
  for (int a = D - 1; a >= 0; a--) {
    const int s = 1 << (2 * a);
#pragma unroll
    for (int l = 0; l < L; l++) {
      const int base = (l % s) + (l / s) * s * 4;
      inv_lift(q[base], q[base + s], q[base + 2 * s], q[base + 3 * s]);
    }
  }
}

// ------------------------------------------------------ bit-matrix transpose
// Transposes every N x N bit tile held in N 32-bit words (N = 4, 16 or 32;
// 32/N tiles side by side in each word): afterwards bit c of word r in tile
// g equals bit r of word c in tile g before.  Recursive block swap; the
// 16- and 8-bit stages are byte permutes.

GZ_HD uint32_t perm_bytes(uint32_t a, uint32_t b, uint32_t sel) {
#if defined(__CUDA_ARCH__)
  return __byte_perm(a, b, sel);
#else
  uint64_t v = ((uint64_t)b << 32) | a;
  uint32_t r = 0;
  for (int i = 0; i < 4; i++) r |= (uint32_t)((v >> (8 * ((sel >> (4 * i)) & 7))) & 0xff) << (8 * i);
  return r;
#endif
}

template <int N>
GZ_HD void transpose_tiles(uint32_t* t) {
  if constexpr (N > 16) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
      uint32_t a = t[k], b = t[k + 16];
      t[k] = perm_bytes(a, b, 0x5410);       // a.lo16 | b.lo16 << 16
      t[k + 16] = perm_bytes(a, b, 0x7632);  // a.hi16 | b.hi16 << 16
    }
  }
  if constexpr (N > 8) {
#pragma unroll
    for (int k = 0; k < N; k++) {
      if (k & 8) continue;
      uint32_t a = t[k], b = t[k + 8];
      t[k] = perm_bytes(a, b, 0x6240);      // bytes a0 b0 a2 b2
      t[k + 8] = perm_bytes(a, b, 0x7351);  // bytes a1 b1 a3 b3
    }
  }
#pragma unroll
  for (int j = (N > 4 ? 4 : N / 2); j > 0; j >>= 1) {
    const uint32_t m = j == 4 ? 0x0f0f0f0fu : j == 2 ? 0x33333333u : 0x55555555u;
#pragma unroll
    for (int k = 0; k < N; k++) {
      if (k & j) continue;
      uint32_t a = t[k], b = t[k + j];
      t[k] = (a & m) | ((b << j) & ~m);
      t[k + j] = ((a >> j) & m) | (b & ~m);
    }
  }
}

// ------------------------------------------------------- transposed planes
// Bit planes of the 4^D negabinary coefficients.  For integer precision P the
// coefficients are cut into P/32 32-bit slices G; slice G of coefficient i
// goes to word tw[G * BS + i] and each run of N = min(BS, 32) words is
// transposed tile by tile.  Plane k (bit k of every coefficient) is then
// found in slice G = k / 32 at row (k % 32) % N, tile (k % 32) / N; for
// BS = 64 the two 32-coefficient halves sit in consecutive runs of 32 words.

template <int D, int P>
struct Planes {
  static constexpr int BS = 1 << (2 * D);
  static constexpr int N = BS < 32 ? BS : 32;
  static constexpr int NW = BS * (P / 32);
  uint32_t tw[NW];

  template <typename UInt>
  GZ_HD void load(const UInt* u, int G) {
#pragma unroll
    for (int i = 0; i < BS; i++) tw[G * BS + i] = (uint32_t)((uint64_t)u[i] >> (32 * G));
  }
  GZ_HD void transpose(int G) {
#pragma unroll
    for (int h = 0; h < BS / N; h++) transpose_tiles<N>(tw + G * BS + h * N);
  }
  GZ_HD uint64_t plane(int k) const {
    const int G = k / 32, kk = k % 32;
    if constexpr (BS == 64) {
      return (uint64_t)tw[G * 64 + kk] | ((uint64_t)tw[G * 64 + 32 + kk] << 32);
    } else {
      const int r = kk % N, g = kk / N;
      return (tw[G * BS + r] >> (g * N)) & ((1u << N) - 1);
    }
  }
  GZ_HD void set_plane(int k, uint64_t x) {
    const int G = k / 32, kk = k % 32;
    if constexpr (BS == 64) {
      tw[G * 64 + kk] = (uint32_t)x;
      tw[G * 64 + 32 + kk] = (uint32_t)(x >> 32);
    } else {
      const int r = kk % N, g = kk / N;
      tw[G * BS + r] |= (uint32_t)x << (g * N);
    }
  }
  template <typename UInt>
  GZ_HD void store(UInt* u) const {
#pragma unroll
    for (int i = 0; i < BS; i++) {
      uint64_t v = tw[i];
      if (P == 64) v |= (uint64_t)tw[BS + i] << 32;
      u[i] = (UInt)v;
    }
  }
};

// ------------------------------------------------------ plane (de)coder
// The embedded coder of encode_ints / decode_ints (Z/src/template/
// encode.c:122-151, decode.c:73-105).  Per bit plane x (bit i = bit k of
// coefficient i) with n coefficients already significant: the first n bits
// verbatim, then group tests -- a 1 if any bit is left, followed by the run
// of zeros up to and including the next one (a one in the last position is
// implied) -- and a final 0 test.  Output stops where the block's bit
// budget is spent, exactly where the bit-serial coder stops.
//
// A plane's group tests have a closed form.  With the m ones above the
// frontier at relative positions q_0 < ... < q_{m-1}, the one of rank j
// lands at bit q_j + 1 + j after the first test bit and is followed by a
// test bit that is 1 except after the last one.  So with the rank spread
// S = sum_j 2^(q_j + j), the group part is 1 | 2S | 4(S - 2^(q_{m-1}+m-1))
// and has q_{m-1} + m + 2 bits.  Planes whose code fits one 64-bit word
// (the common case for smooth data) are coded in one step this way; the
// rest -- a one in the last position, long codes, the budget running out --
// take the bit-exact general routines below.

// General one-plane coder (clips at the budget).
template <int BS, class W>
GZ_HD void encode_plane(uint64_t x, uint32_t& n, uint32_t& bits, W& w) {
  uint32_t m = n < bits ? n : bits;
  w.put(x & lowmask64(m), m);
  bits -= m;
  uint64_t y = shr64(x, n);
  while (n < (uint32_t)BS && bits) {
    if (y == 0) {
      w.put(0, 1);
      bits--;
      break;
    }
    uint32_t t = ctz64(y);
    uint32_t lim = BS - 1 - n;
    uint64_t pat;
    uint32_t len, adv;
    if (t < lim) {  // test 1, t zeros, the one
      pat = 1u | (2ull << t);
      len = t + 2;
      adv = t + 1;
    } else {  // test 1, zeros up to the implied one in the last position
      pat = 1;
      len = lim + 1;
      adv = BS - n;
    }
    uint32_t l = len < bits ? len : bits;
    w.put(pat & lowmask64(l), l);
    bits -= l;
    y = shr64(y, adv);
    n += adv;
  }
}

// Group tests of one plane, from the reader's position (the first test bit)
// on, with x holding the plane's verbatim bits: the bit-serial loop of
// decode_ints (Z/src/template/decode.c:88-99), including its rule that a
// run cut off by the budget still deposits a one at the current position.
template <int BS, class R>
GZ_HD uint64_t decode_group(uint64_t x, uint32_t& n, uint32_t& bits, R& r) {
  while (n < (uint32_t)BS && bits) {
    uint64_t w = r.peek64();
    bits--;
    if (!(w & 1)) {
      r.skip(1);
      break;
    }
    uint32_t t = ctz64(w >> 1);
    uint32_t lim = BS - 1 - n;
    if (lim > bits) lim = bits;
    if (t < lim) {
      r.skip(t + 2);
      bits -= t + 1;
      n += t;
    } else {
      r.skip(lim + 1);
      bits -= lim;
      n += lim;
    }
    x |= 1ull << n;
    n++;
  }
  return x;
}

// General one-plane decoder: the verbatim bits, then the group tests.
template <int BS, class R>
GZ_HD uint64_t decode_plane(uint32_t& n, uint32_t& bits, R& r) {
  uint32_t m = n < bits ? n : bits;
  uint64_t x = r.read(m);
  bits -= m;
  return decode_group<BS>(x, n, bits, r);
}

// Rank spread of the ones of z: the one of rank j moves from bit q to bit
// q + j.  With z_i = z without its i lowest ones, the spread is
// z + z_1 + 2 z_2 + 4 z_3 + ... (the one of rank j is counted once in z and
// 2^(i-1) times for each i = 1..j, 2^j times in all), so up to three ones
// cost two clears and three adds; more ones loop.
GZ_HD uint64_t rank_spread(uint64_t z) {
  const uint64_t z1 = z & (z - 1);
  const uint64_t z2 = z1 & (z1 - 1);
  const uint64_t z3 = z2 & (z2 - 1);
  const uint64_t z4 = z3 & (z3 - 1);
  uint64_t z5 = z4 & (z4 - 1);
  uint64_t S = z + z1 + (z2 << 1) + (z3 << 2) + (z4 << 3) + (z5 << 4);
  for (uint32_t j = 5; z5; j++) {
    z5 &= z5 - 1;
    S += z5 << j;
  }
  return S;
}

// Rank spread of a plane of at most 16 bits: below 2^31.
GZ_HD uint32_t rank_spread32(uint32_t z) {
  const uint32_t z1 = z & (z - 1);
  uint32_t z2 = z1 & (z1 - 1);
  uint32_t S = z + z1 + (z2 << 1);
  for (uint32_t j = 2; z2; j++) {
    z2 &= z2 - 1;
    S += z2 << j;
  }
  return S;
}

// code_planes for blocks of at most 16 values (1D and 2D): a plane has at
// most 16 bits and its whole code -- verbatim bits, then group tests -- at
// most 16 + 33 bits, so it is built in 32-bit arithmetic and written in one
// piece.  Same bits as the general form below.
template <int BS, bool STOP_FULL = false, class W, class PlaneFn>
GZ_HD int code_planes_small(int k, int k_low, uint32_t& n, uint32_t& bits, W& w,
                            PlaneFn&& plane) {
  static_assert(BS <= 16, "at most 16 values per block");
  // STOP_FULL: return as soon as every coefficient is significant
  for (; k >= k_low && bits && !(STOP_FULL && n == (uint32_t)BS); k--) {
    const uint32_t x = (uint32_t)plane(k);
    const uint32_t bl = 32 - clz32(x);      // bit length of the plane
    const bool full = n == (uint32_t)BS;
    const bool any = bl > n;                // a one above the frontier
    if (any && bl >= (uint32_t)BS) {        // a one in the last position is implied
      encode_plane<BS>(x, n, bits, w);
      continue;
    }
    const uint32_t xh = full ? 0u : x >> n;
    const uint32_t hb = bl - 1 - n;
    const uint32_t m = popcount32(xh);
    const uint32_t S = rank_spread32(xh);
    const uint64_t grp =
        any ? (1 | ((uint64_t)S << 1) | ((uint64_t)(S - (1u << ((hb + m - 1) & 31))) << 2)) : 0;
    const uint32_t hlen = full ? (uint32_t)BS : n;
    const uint32_t head = full ? x : x & ((1u << n) - 1);
    const uint32_t glen = full ? 0 : any ? hb + m + 2 : 1;
    n = any ? bl : n;
    const uint32_t len = hlen + glen;
    const uint32_t l = len < bits ? len : bits;
    w.put(((uint64_t)head | (grp << hlen)) & lowmask64(l), l);
    bits -= l;
  }
  return k;
}

// Code planes k, k-1, ... down to k_low while budget remains; plane(k)
// yields plane k.  Returns the index of the next plane.  A plane's code is
// written as two pieces -- its n verbatim bits, then its group tests (at
// most 64 bits) -- so the loop body has no data-dependent branch except the
// rare general path (a one implied by the last position, or group tests
// longer than 64 bits), and the 32 threads of a warp (32 blocks) stay
// converged plane after plane.  A budget that ends inside a plane just
// truncates its code, as the bit-serial coder does.
template <int BS, class W, class PlaneFn>
GZ_HD int code_planes(int k, int k_low, uint32_t& n, uint32_t& bits, W& w, PlaneFn&& plane) {
  if constexpr (BS <= 16) return code_planes_small<BS>(k, k_low, n, bits, w, plane);
  // The frontier after a plane is max(n, bit length of the plane), so the
  // chain from one plane to the next is a single max; the rest of a plane's
  // code depends on n but not on the previous plane's code.
  for (; k >= k_low && bits; k--) {
    const uint64_t x = plane(k);
    const uint32_t bl = 64 - clz64(x);              // bit length of the plane
    const bool full = n == (uint32_t)BS;            // all significant: plane verbatim
    const bool any = bl > n;                        // a one above the frontier
    const uint32_t sh = full ? 0 : n;
    const uint64_t xh = full ? 0 : x >> sh;         // ones above the frontier
    const uint32_t hb = bl - 1 - n;                 // top one, relative to the frontier
    const uint32_t m = (uint32_t)popcount64(xh);
    if (any && (bl >= (uint32_t)BS || hb + m > 62)) {
      encode_plane<BS>(x, n, bits, w);
      continue;
    }
    const uint64_t S = rank_spread(xh);
    const uint64_t grp = any ? (1 | (S << 1) | ((S - (1ull << ((hb + m - 1) & 63))) << 2)) : 0;
    const uint32_t hlen = full ? (uint32_t)BS : n;
    const uint64_t head = full ? x : x & ((1ull << sh) - 1);
    const uint32_t glen = full ? 0 : any ? hb + m + 2 : 1;
    n = any ? bl : n;
    if (hlen + glen <= 64) {  // both pieces in one word (most planes)
      const uint32_t len = hlen + glen;
      const uint64_t code = head | (glen ? grp << (hlen & 63) : 0);
      const uint32_t l = len < bits ? len : bits;
      w.put(code & lowmask64(l), l);
      bits -= l;
    } else {
      uint32_t l = hlen < bits ? hlen : bits;
      w.put(head & lowmask64(l), l);
      bits -= l;
      l = glen < bits ? glen : bits;
      w.put(grp & lowmask64(l), l);
      bits -= l;
    }
  }
  return k;
}

// The group tests of one plane from a 64-bit window w of the stream, of
// which `used` bits (the plane's verbatim bits) are taken, with `bits` the
// budget from the window's start and `pos` the frontier: decode_ints'
// loops (Z/src/template/decode.c:88-99) one new coefficient at a time,
// including the budget ending inside a run (a one is still deposited where
// it ends) and the implied one in the last position.  Ones go into x;
// `used` and `pos` advance.  Returns false, with nothing final, when the
// group runs past the window; the caller then decodes it from the stream.
// Every plane, the last one in the budget included, takes this one path,
// so the lanes of a warp do not split at their blocks' last planes.
template <int BS, typename X>
GZ_HD bool group_in_window(uint64_t w, uint32_t bits, uint32_t& used, uint32_t& pos, X& x) {
  if (pos >= (uint32_t)BS || used >= bits) return true;  // no group tests
  bool more = (w >> used) & 1;  // the first test bit (used < 64 here)
  used++;
  uint64_t g = shr64(w, used);
  while (more) {
    const uint32_t t = ctz64(g);  // zeros before the next one in the window
    const uint32_t rem = bits - used, lim = (uint32_t)BS - 1 - pos;
    uint32_t z = t < rem ? t : rem;
    z = z < lim ? z : lim;  // zeros read before the run ends
    if (used + z + 2 > 64) return false;
    const uint32_t c = z + ((z == t && t < rem && t < lim) ? 1u : 0u);  // with the one, if read
    x |= (X)1 << (pos + z);
    g >>= c;
    used += c;
    pos += z + 1;
    more = false;
    if (pos < (uint32_t)BS && used < bits) {  // the next test bit
      more = g & 1;
      g >>= 1;
      used++;
    }
  }
  return true;
}

// uncode_planes for blocks of at most 16 values: the verbatim bits and the
// group tests of a plane (at most 16 + 33 bits) come from one 64-bit window.
// Same bits as the general form below.  UNIFIED: every plane, the one the
// budget ends in included, goes through group_in_window, so a warp's lanes
// do not split at their blocks' last planes (faster for 2D blocks of 32-bit
// values; for 64-bit values and 4^3 blocks the split form measured faster).
template <int BS, bool STOP_FULL = false, bool UNIFIED = false, class R, class StoreFn>
GZ_HD int uncode_planes_small(int k, int k_low, uint32_t& n, uint32_t& bits, R& r,
                              StoreFn&& store) {
  static_assert(BS <= 16, "at most 16 values per block");
  for (; k >= k_low && bits && !(STOP_FULL && n == (uint32_t)BS); k--) {
    if constexpr (UNIFIED) {
      const uint32_t h = n < bits ? n : bits;  // verbatim bits (n == BS once all are significant)
      const uint64_t w = r.peek64();
      const uint32_t x0 = (uint32_t)w & ((1u << h) - 1);
      uint32_t x = x0, used = h, pos = n;
      if (group_in_window<BS>(w, bits, used, pos, x)) {
        r.skip(used);
        bits -= used;
        n = pos;
        store(k, x);
      } else {
        r.skip(h);
        bits -= h;
        store(k, decode_group<BS>(x0, n, bits, r));
      }
      continue;
    }
    const bool full = n == (uint32_t)BS;
    const uint32_t hlen = full ? (uint32_t)BS : n;
    if (hlen > bits) {  // the budget ends inside the verbatim bits
      store(k, decode_plane<BS>(n, bits, r));
      continue;
    }
    const uint64_t w = r.peek64();
    uint32_t x = (uint32_t)w & ((1u << hlen) - 1);
    if (full || bits == hlen) {
      r.skip(hlen);
      bits -= hlen;
      store(k, x);
      continue;
    }
    const bool test = (w >> hlen) & 1;
    uint64_t g = (w >> hlen) >> 1;
    uint32_t used = hlen + 1, pos = n;  // bits of the window taken so far
    bool ok = true;
    bool more = test;
    while (more && ok) {  // runs once per one of the plane
      const uint32_t t = ctz64(g);
      ok = pos + t < (uint32_t)BS - 1 && used + t + 2 <= 64 && used + t + 2 <= bits;
      if (ok) {
        x |= 1u << (pos + t);
        more = (g >> (t + 1)) & 1;
        g = (g >> (t + 1)) >> 1;
        used += t + 2;
        pos += t + 1;
      }
    }
    if (ok) {
      r.skip(used);
      bits -= used;
      n = test ? pos : n;
      store(k, x);
    } else {
      r.skip(hlen);
      bits -= hlen;
      store(k, decode_group<BS>(x, n, bits, r));  // group tests not consumed yet
    }
  }
  return k;
}

// Decode planes k, ... down to k_low while budget remains, handing each to
// store(k, x).  Returns the index of the next plane.  The verbatim bits are
// read first; the group tests are then decoded from a fresh 64-bit window
// when they lie inside it and the budget, with no one implied by the last
// position.  Otherwise (the plane the budget ends in, and rarely others)
// the general routine decodes the group tests.
template <int BS, bool UNIFIED = false, class R, class StoreFn>
GZ_HD int uncode_planes(int k, int k_low, uint32_t& n, uint32_t& bits, R& r, StoreFn&& store) {
  if constexpr (BS <= 16)
    return uncode_planes_small<BS, false, UNIFIED>(k, k_low, n, bits, r, store);
  for (; k >= k_low && bits; k--) {
    const bool full = n == (uint32_t)BS;
    const uint32_t hlen = full ? (uint32_t)BS : n;
    if (hlen > bits) {  // the budget ends inside the verbatim bits
      store(k, decode_plane<BS>(n, bits, r));
      continue;
    }
    uint64_t x = r.peek64() & lowmask64(hlen);
    r.skip(hlen);
    bits -= hlen;
    if (full || !bits) {
      store(k, x);
      continue;
    }
    const uint64_t w = r.peek64();
    const bool test = w & 1;
    uint64_t g = w >> 1;
    uint32_t used = 1, pos = n;
    bool ok = true;
    bool more = test;
    while (more && ok) {  // runs once per one of the plane
      const uint32_t t = ctz64(g);
      ok = pos + t < (uint32_t)BS - 1 && used + t + 2 <= 64 && used + t + 2 <= bits;
      if (ok) {
        x |= 1ull << (pos + t);
        more = (g >> (t + 1)) & 1;
        g = (g >> (t + 1)) >> 1;
        used += t + 2;
        pos += t + 1;
      }
    }
    if (ok) {
      r.skip(used);
      bits -= used;
      n = test ? pos : n;
      store(k, x);
    } else {
      store(k, decode_group<BS>(x, n, bits, r));  // group tests not consumed yet
    }
  }
  return k;
}

// Planes k, ... down to k_low of a 4^3 block while budget remains, decoded
// as one flat sequence of steps, each of which reads one token: a plane's
// verbatim bits with its first group test, or one run of a group (its
// zeros, the one -- read, implied by the last position, or placed where the
// budget ends, as decode_ints places it (Z/src/template/decode.c:88-99) --
// and the test after it).  A warp's lanes step through tokens, not planes,
// so a plane with many new ones in one lane does not hold the others at
// that plane.  Same bits as uncode_planes<64>.
// 32-bit helpers for the token loop: the low/high words of 64-bit values,
// so that shifts by a variable amount are one funnel shift per word
GZ_HD uint32_t fshr(uint32_t lo, uint32_t hi, uint32_t s) {  // (hi:lo) >> s, s < 32
#if defined(__CUDA_ARCH__)
  return __funnelshift_r(lo, hi, s);
#else
  return s ? (lo >> s) | (hi << (32 - s)) : lo;
#endif
}

template <class R, class StoreFn>
GZ_HD int uncode_flat64(int k, int k_low, uint32_t& n, uint32_t& bits, R& r, StoreFn&& store) {
  uint32_t xl = 0, xh = 0;  // the plane being built
  uint32_t pos = n;
  bool grp = false;
  while (k >= k_low && (bits || grp)) {
    const uint64_t w64 = r.peek64();
    const uint32_t wl = lo32(w64), wh = hi32(w64);
    uint32_t c;
    if (!grp) {  // verbatim bits, cut by the budget
      const uint32_t h = umin(n, bits);  // n <= 64
      // low h bits of w
      xl = h >= 32 ? wl : wl & ((1u << h) - 1u);
      xh = h >= 64 ? wh : h > 32 ? wh & ((1u << (h - 32)) - 1u) : 0u;
      c = h;
      pos = n;
    } else {  // zeros up to the next one, the last position or the budget's end
      const uint32_t t = wl ? ctz32(wl) : 32 + ctz32(wh);
      const uint32_t lim = umin(63 - pos, bits);
      const bool read = t < lim;
      const uint32_t z = read ? t : lim;
      c = read ? t + 1 : lim;
      const uint32_t p = pos + z;
      const uint32_t b = 1u << (p & 31);
      xl |= p < 32 ? b : 0u;
      xh |= p < 32 ? 0u : b;
      pos = p + 1;
    }
    const uint32_t rest = bits - c;
    const bool has_test = pos < 64 && rest > 0;  // c < 64 here
    const uint32_t tw = c < 32 ? wl : wh;
    const bool test = has_test && ((tw >> (c & 31)) & 1u);
    c += has_test ? 1u : 0u;
    bits = rest - (has_test ? 1u : 0u);
    r.skip(c);
    grp = test;
    if (!test) {  // the plane is complete
      store(k, ((uint64_t)xh << 32) | xl);
      k--;
      n = pos;
    }
  }
  return k;
}

// ------------------------------------------------- runs at frontier 0 and 1
// In a block of smooth data the first coefficient is often the only
// significant one for many planes: each such plane is that coefficient's
// bit and a 0 test bit, and a run of them is the coefficient's bit segment
// (plane k first) spread to every other bit.  Runs at frontier 0 (all-zero
// planes, one 0 bit each) and 1 are coded and decoded whole; the other
// planes go one at a time through the small-block coder.  (Used for 2D
// blocks; 4-value blocks use the plane tables below.)

// bit i of x (below 2^32) to bit 2i
GZ_HD uint64_t spread2(uint64_t x) {
  x &= 0xffffffffull;
  x = (x | (x << 16)) & 0x0000ffff0000ffffull;
  x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
  x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  return (x | (x << 1)) & 0x5555555555555555ull;
}
// inverse: bit 2i of x to bit i (odd bits ignored)
GZ_HD uint64_t compact2(uint64_t x) {
  x &= 0x5555555555555555ull;
  x = (x | (x >> 1)) & 0x3333333333333333ull;
  x = (x | (x >> 2)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x >> 4)) & 0x00ff00ff00ff00ffull;
  x = (x | (x >> 8)) & 0x0000ffff0000ffffull;
  return (x | (x >> 16)) & 0x00000000ffffffffull;
}
GZ_HD uint32_t brev_u(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __brev(x);
#else
  x = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
  x = ((x >> 2) & 0x33333333u) | ((x & 0x33333333u) << 2);
  x = ((x >> 4) & 0x0f0f0f0fu) | ((x & 0x0f0f0f0fu) << 4);
  x = ((x >> 8) & 0x00ff00ffu) | ((x & 0x00ff00ffu) << 8);
  return (x >> 16) | (x << 16);
#endif
}
GZ_HD uint64_t brev_u(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __brevll(x);
#else
  return ((uint64_t)brev_u((uint32_t)x) << 32) | brev_u((uint32_t)(x >> 32));
#endif
}


// Code planes k, k-1, ... of a block of at most 16 values while the
// frontier is 0 or 1, in runs: u0 is the first coefficient, above0 / above1
// the OR of the coefficients at positions >= 0 / >= 1 (a plane brings a new
// coefficient at the highest set bit among those at or above the
// frontier), plane(k) a plane for the planes that bring one.  Returns the
// next plane; the same bits as code_planes<BS>.
template <int BS, typename UInt, class W, class PlaneFn>
GZ_HD int code_runs01(UInt u0, UInt above0, UInt above1, int k, int k_low, uint32_t& n,
                      uint32_t& bits, W& w, PlaneFn&& plane) {
  constexpr int P = 8 * sizeof(UInt);
  while (k >= k_low && bits && n <= 1) {
    // the highest plane at or below k with a one at a position >= n (no
    // such one sits above k, or n would be larger)
    const UInt hi = n ? above1 : above0;
    const int kstop = hi ? P - 1 - (int)(sizeof(UInt) == 8 ? clz64((uint64_t)hi)
                                                           : clz32((uint32_t)hi))
                         : -1;
    const int lo = kstop > k_low - 1 ? kstop : k_low - 1;
    if (k > lo) {  // planes k .. lo + 1: a run
      const uint32_t gw = n + 1;
      const uint32_t cmax = 64 / gw;
      uint32_t r = (uint32_t)(k - lo);
      while (r && bits) {
        const uint32_t c = r < cmax ? r : cmax;
        const uint64_t seg = (uint64_t)(brev_u(u0) >> (P - 1 - k)) & lowmask64(c);
        const uint64_t code = n ? spread2(seg) : 0;
        const uint32_t len = c * gw;
        const uint32_t l = len < bits ? len : bits;
        w.put(code & lowmask64(l), l);
        bits -= l;
        k -= (int)c;
        r -= c;
      }
    }
    // then, in the same step (so that a warp's lanes stay together), plane
    // k = kstop, which brings a new coefficient
    if (k < k_low || !bits) break;
    k = code_planes_small<BS>(k, k, n, bits, w, plane);
  }
  return k;
}

// Decode planes k, k-1, ... of a block of at most 16 values while the
// frontier is 0 or 1: runs add their bits of the first coefficient to u0,
// the planes that bring a new coefficient go to store(k, x).  Returns the
// next plane; the same bits as uncode_planes<BS>.
template <int BS, bool UNIFIED = false, typename UInt, class R, class StoreFn>
GZ_HD int uncode_runs01(UInt& u0, int k, int k_low, uint32_t& n, uint32_t& bits, R& r,
                        StoreFn&& store) {
  constexpr int P = 8 * sizeof(UInt);
  // with a budget this small the runs are too short to pay for themselves
  if (bits < 32) return k;
  while (k >= k_low && bits && n <= 1) {
    const uint32_t gw = n + 1;
    // whole planes that fit the window, the budget and the planes left
    uint32_t c = 64 / gw;
    if ((uint32_t)(k - k_low + 1) < c) c = (uint32_t)(k - k_low + 1);
    if (bits / gw < c) c = bits / gw;
    uint32_t rr = 0;
    uint64_t win = 0;
    if (c) {  // the run ends at the first test bit that is 1
      win = r.peek64();
      const uint64_t tests = (n ? 0xaaaaaaaaaaaaaaaaull : ~0ull) & lowmask64(c * gw);
      const uint64_t hit = win & tests;
      rr = hit ? (uint32_t)popcount64(tests & lowmask64(ctz64(hit))) : c;
    }
    if (rr) {  // rr planes of verbatim bits and 0 tests
      if (n) {
        // bit j of seg is bit k - j of the coefficient
        const uint64_t seg = compact2(win) & lowmask64(rr);
        u0 |= brev_u((UInt)seg) >> (P - 1 - k);
      }
      r.skip(rr * gw);
      bits -= rr * gw;
      k -= (int)rr;
    }
    // then, in the same step, one plane one at a time: one that brings a
    // new coefficient, the budget's last, or a plane past the window
    if (k < k_low || !bits) break;
    k = uncode_planes_small<BS, false, UNIFIED>(k, k, n, bits, r, store);
  }
  return k;
}

// ------------------------------------------------------ 4-value blocks
// A plane of a 4-value block has 4 bits, and with the frontier n (0..4)
// they alone determine the plane's code in encode_ints
// (Z/src/template/encode.c:122-151): n verbatim bits, then the group tests,
// at most 7 bits in all.  Decoding a plane (decode_ints, Z/src/template/
// decode.c:73-105) reads at most 7 bits and depends only on n, those bits
// and how many of them the budget still allows.  So both directions are
// table lookups with no data-dependent branch: the encoder codes two planes
// per lookup, the decoder one.  A budget that ends inside a plane cuts the
// encoder's output there, as the bit-serial coder stops there; for the
// decoder the budget is part of the index, and zfp's rule that a run cut
// off by the budget still deposits a one is in the table.

struct Plane4Tables {
  // planes k and k - 1: index n * 256 + x_k + 16 * x_{k-1}; entry = both
  // codes (14 bits, plane k's first) | plane k's code length << 14 | both
  // lengths << 17 | frontier after plane k << 21 | after both << 24
  uint32_t enc2[5 * 256];
  // one plane, with r = min(7, bits left) >= 1: index n * 256 + (r == 7 ?
  // 128 + the next 7 bits : 2^r + the next r bits); entry = the plane's 4
  // bits | bits read << 4 | frontier after << 7
  uint16_t dec[5 * 256];
};

struct Code4 {
  uint32_t code, len, n;
};

// encode_ints for one plane x (4 bits) at frontier n, with no budget limit
GZ_CX Code4 plane4_code(uint32_t x, uint32_t n) {
  uint32_t code = x & ((1u << n) - 1), len = n, m = n, xs = x >> n;
  while (m < 4) {  // group tests
    const uint32_t t = xs != 0;
    code |= t << len++;
    if (!t) break;
    while (m < 3) {  // up to the next one; a one in the last position is implied
      const uint32_t b = xs & 1u;
      code |= b << len++;
      if (b) break;
      xs >>= 1;
      m++;
    }
    xs >>= 1;
    m++;
  }
  return Code4{code, len, m};
}

// decode_ints for one plane at frontier n from the r-bit budget v (bit 0
// first): the plane's bits, the bits read, the new frontier
GZ_CX Code4 plane4_decode(uint32_t v, uint32_t r, uint32_t n) {
  const uint32_t m = n < r ? n : r;
  uint32_t x = v & ((1u << m) - 1), pos = m, b = r - m;
  while (n < 4 && b) {
    b--;
    if (!((v >> pos++) & 1u)) break;  // group test 0: no one left
    while (n < 3 && b) {
      b--;
      if ((v >> pos++) & 1u) break;
      n++;
    }
    x += 1u << n;  // also when the budget ended the run
    n++;
  }
  return Code4{x, pos, n};
}

GZ_CX Plane4Tables make_plane4_tables() {
  Plane4Tables t{};
  for (uint32_t n = 0; n <= 4; n++) {
    for (uint32_t i = 0; i < 256; i++) {
      const Code4 a = plane4_code(i & 15u, n);
      const Code4 c = plane4_code(i >> 4, a.n);
      t.enc2[n * 256 + i] = (a.code | (c.code << a.len)) | (a.len << 14) |
                            ((a.len + c.len) << 17) | (a.n << 21) | (c.n << 24);
    }
    for (uint32_t r = 1; r <= 7; r++)
      for (uint32_t v = 0; v < (1u << r); v++) {
        const Code4 d = plane4_decode(v, r, n);
        t.dec[n * 256 + (r == 7 ? 128 + v : (1u << r) + v)] =
            (uint16_t)(d.code | (d.len << 4) | (d.n << 7));
      }
  }
  return t;
}

#if defined(__CUDACC__)
// device copy, built by the compiler; kernels stage it in shared memory
__device__ const __align__(16) Plane4Tables kPlane4Tables = make_plane4_tables();
#endif

// host copy (host builds and tests)
inline const Plane4Tables* plane4_tables_host() {
  static const Plane4Tables t = make_plane4_tables();
  return &t;
}

// Planes k, k-1, ... down to k_low of a 4-value block while budget
// remains, from the tables.  k starts at P - 1.  The 4x4 bit tiles of each
// 32-bit slice of the coefficients are transposed, so word i holds planes
// 32G + 4c + i at bits 4c..4c+3; the words are shifted up a tile at a time
// and two planes make one table index.
template <typename UInt, class W>
GZ_HD void code_planes_4(const UInt* u, int k, int k_low, uint32_t& n, uint32_t& bits, W& w,
                         const Plane4Tables& t) {
  constexpr int NS = (int)sizeof(UInt) / 4;  // 32-bit slices
  auto pair = [&](uint32_t xb) {  // planes k, k - 1 (xb = x_k | x_{k-1} << 4)
    if (k < k_low || !bits) return;
    const uint32_t e = t.enc2[n * 256 + xb];
    const bool two = k - 1 >= k_low;
    const uint32_t len = two ? (e >> 17) & 15u : (e >> 14) & 7u;
    n = two ? (e >> 24) & 7u : (e >> 21) & 7u;
    const uint32_t l = len < bits ? len : bits;
    w.put(e & ((1u << l) - 1), l);
    bits -= l;
    k -= 2;
  };
#pragma unroll
  for (int G = NS - 1; G >= 0; G--) {
    uint32_t tw[4];
#pragma unroll
    for (int i = 0; i < 4; i++) tw[i] = (uint32_t)((uint64_t)u[i] >> (32 * G));
    transpose_tiles<4>(tw);
#pragma unroll 1
    for (int c = 7; c >= 0 && k >= k_low && bits; c--) {
      pair((tw[3] >> 28) | ((tw[2] >> 24) & 0xf0u));
      pair((tw[1] >> 28) | ((tw[0] >> 24) & 0xf0u));
#pragma unroll
      for (int i = 0; i < 4; i++) tw[i] <<= 4;
    }
  }
}

// Decode planes k = P - 1, ... down to k_low of a 4-value block while
// budget remains, from the tables, into u (zero on entry).  The stream is
// read through a 64-bit window refilled when fewer than 7 bits are left in
// it; the planes are shifted into the transposed words of code_planes_4.
template <typename UInt, class R>
GZ_HD void uncode_planes_4(UInt* u, int k, int k_low, uint32_t& n, uint32_t& bits, R& r,
                           const Plane4Tables& t) {
  constexpr int NS = (int)sizeof(UInt) / 4;
  uint64_t win = r.peek64();
  uint32_t avail = 64, taken = 0;  // bits of win not yet used; used since the last skip
  auto one = [&]() -> uint32_t {   // plane k
    if (k < k_low || !bits) return 0u;
    if (avail < 7) {
      r.skip(taken);
      taken = 0;
      win = r.peek64();
      avail = 64;
    }
    const uint32_t v = (uint32_t)win & 127u;
    const uint32_t idx = bits >= 7 ? 128u + v : (1u << bits) + (v & ((1u << bits) - 1));
    const uint32_t e = t.dec[n * 256 + idx];
    const uint32_t used = (e >> 4) & 7u;
    n = e >> 7;
    win >>= used;
    avail -= used;
    taken += used;
    bits -= used;
    k--;
    return e & 15u;
  };
#pragma unroll
  for (int G = NS - 1; G >= 0; G--) {
    uint32_t tw[4] = {0, 0, 0, 0};
    int c = 7;
#pragma unroll 1
    for (; c >= 0 && k >= k_low && bits; c--) {
      const uint32_t x3 = one(), x2 = one(), x1 = one(), x0 = one();
      tw[3] = (tw[3] << 4) | x3;
      tw[2] = (tw[2] << 4) | x2;
      tw[1] = (tw[1] << 4) | x1;
      tw[0] = (tw[0] << 4) | x0;
    }
    const uint32_t sh = 4u * (uint32_t)(c + 1);  // tiles not reached are zero
#pragma unroll
    for (int i = 0; i < 4; i++) tw[i] = sh < 32 ? tw[i] << sh : 0u;
    transpose_tiles<4>(tw);
#pragma unroll
    for (int i = 0; i < 4; i++) u[i] |= (UInt)((uint64_t)tw[i] << (32 * G));
  }
  r.skip(taken);
}

// --------------------------------------------------------- float <-> bits

GZ_HD float bits_f32(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  __builtin_memcpy(&f, &b, 4);
  return f;
#endif
}
GZ_HD uint32_t f32_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t b;
  __builtin_memcpy(&b, &f, 4);
  return b;
#endif
}
GZ_HD double bits_f64(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double f;
  __builtin_memcpy(&f, &b, 8);
  return f;
#endif
}
GZ_HD uint64_t f64_bits(double f) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(f);
#else
  uint64_t b;
  __builtin_memcpy(&b, &f, 8);
  return b;
#endif
}

// IEEE multiply then truncating float -> int32 conversion that saturates and
// maps NaN to 0 (cvt.rzi.s32.f32 semantics)
GZ_HD int32_t mul_to_i32(float s, float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rz(__fmul_rn(s, x));
#else
  volatile float v = s * x;
  float p = v;
  if (p != p) return 0;
  if (p >= 2147483648.0f) return INT32_MAX;
  if (p < -2147483648.0f) return INT32_MIN;
  return (int32_t)p;
#endif
}

GZ_HD float i32_scaled(int32_t q, float s) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(__int2float_rn(q), s);
#else
  volatile float v = (float)q * s;
  return v;
#endif
}

GZ_HD double i64_scaled(int64_t q, double s) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(__ll2double_rn(q), s);
#else
  volatile double v = (double)q * s;
  return v;
#endif
}

// 2^e as a float / double, exact (denormal or zero below the normal range,
// as ldexp rounds it)
GZ_HD float pow2f(int e) {
  if (e > 127) return bits_f32(0x7f800000u);
  if (e >= -126) return bits_f32((uint32_t)(e + 127) << 23);
  if (e >= -149) return bits_f32(1u << (e + 149));
  return 0.0f;
}
GZ_HD double pow2d(int e) {
  if (e > 1023) return bits_f64(0x7ff0000000000000ull);
  if (e >= -1022) return bits_f64((uint64_t)(e + 1023) << 52);
  if (e >= -1074) return bits_f64(1ull << (e + 1074));
  return 0.0;
}

// ------------------------------------------------------------- quantise
// Block-floating-point conversion of Z/src/template/encode.c:36-52:
// q = (Int)(x * 2^(P-2-emax)).

// f32: the scale multiply is exact, so the hardware float path is used.
GZ_HD void quantize(const uint32_t* raw, int32_t* q, int n, int emax) {
  const float s = pow2f(30 - emax);
  for (int i = 0; i < n; i++) q[i] = mul_to_i32(s, bits_f32(raw[i]));
}

// f64: shift the significand into place (exact), except in the regime where
// 2^(62-emax) overflows to +inf, where zfp's product is +-inf or NaN and the
// conversion saturates (see the oracle's header on defined behaviour).
// With maxE the largest biased exponent, a value of biased exponent E and
// significand M (53 bits with the hidden one) maps to
// |q| = (M << 9) >> (maxE - E): M << 9 < 2^62 never loses bits.
GZ_HD void quantize(const uint64_t* raw, int64_t* q, int n, int emax) {
  if (emax >= 62 - 1023) {
    const uint32_t maxE = (uint32_t)(emax + 1022);  // >= 61
    uint32_t minE = 0x7ff;
#pragma unroll
    for (int i = 0; i < n; i++) {
      uint32_t E = (uint32_t)(raw[i] >> 52) & 0x7ffu;
      minE = E < minE ? E : minE;
    }
    if (minE != 0) {  // no zeros or denormals: every value has the hidden one
#pragma unroll
      for (int i = 0; i < n; i++) {
        const uint32_t hi = (uint32_t)(raw[i] >> 32), lo = (uint32_t)raw[i];
        const uint32_t E = (hi >> 20) & 0x7ffu;
        const uint32_t d = umin(maxE - E, 63u);
        const uint64_t M9 = ((uint64_t)((hi & 0xfffffu) | 0x100000u) << 41) | ((uint64_t)lo << 9);
        const uint64_t mag = M9 >> d;
        const uint64_t s = (uint64_t)((int64_t)(int32_t)hi >> 31);  // 0 or all ones
        q[i] = (int64_t)((mag ^ s) - s);
      }
    } else {
#pragma unroll
      for (int i = 0; i < n; i++) {
        const uint32_t hi = (uint32_t)(raw[i] >> 32), lo = (uint32_t)raw[i];
        const uint32_t E = (hi >> 20) & 0x7ffu;
        const uint32_t d = umin(maxE - (E ? E : 1u), 63u);
        const uint64_t M9 = ((uint64_t)((hi & 0xfffffu) | (E ? 0x100000u : 0u)) << 41) |
                            ((uint64_t)lo << 9);
        const uint64_t mag = M9 >> d;
        const uint64_t s = (uint64_t)((int64_t)(int32_t)hi >> 31);
        q[i] = (int64_t)((mag ^ s) - s);
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < n; i++) {
      uint64_t a = raw[i] & 0x7fffffffffffffffull;
      q[i] = a == 0 ? 0 : (raw[i] >> 63) ? INT64_MIN : INT64_MAX;
    }
  }
}

// ----------------------------------------------------------- dequantise
// Inverse of quantize (Z/src/template/decode.c:9-25): x = (Scalar)q * 2^(emax-(P-2)).

GZ_HD void dequantize(const int32_t* q, uint32_t* raw, int n, int emax) {
  const float s = pow2f(emax - 30);
  for (int i = 0; i < n; i++) raw[i] = f32_bits(i32_scaled(q[i], s));
}

// f64: wherever the result is a normal number for every nonzero q
// (-960 <= emax <= 1022), the round-to-nearest int64 -> double conversion
// runs on the conversion unit (it shares the FP64 pipe, which is otherwise
// idle here) and the power-of-two scale is an integer add to the exponent
// field; outside that range the full IEEE multiply is used.
GZ_HD void dequantize(const int64_t* q, uint64_t* raw, int n, int emax) {
  if (emax >= -960 && emax <= 1022) {
    const uint64_t scale = (uint64_t)(int64_t)(emax - 62) << 52;
#pragma unroll
    for (int i = 0; i < n; i++) {
#if defined(__CUDA_ARCH__)
      const uint64_t d = f64_bits(__ll2double_rn(q[i]));
#else
      const uint64_t d = f64_bits((double)q[i]);
#endif
      raw[i] = q[i] ? d + scale : 0;
    }
  } else {
    const double s = pow2d(emax - 62);
    for (int i = 0; i < n; i++) raw[i] = f64_bits(i64_scaled(q[i], s));
  }
}

// 4^3 blocks: transpose the 32-bit slice G of the 64 coefficients and put
// planes 32G .. 32G+31 into store slots 0..31 (slot = plane - 32G).
template <int G, typename UInt, class PS>
GZ_HD void planes_to_store(const UInt* u, PS& ps) {
  uint32_t t[64];
#pragma unroll
  for (int i = 0; i < 64; i++) t[i] = (uint32_t)((uint64_t)u[i] >> (32 * G));
  transpose_tiles<32>(t);
  transpose_tiles<32>(t + 32);
#pragma unroll
  for (int kk = 0; kk < 32; kk++) ps.put(kk, (uint64_t)t[kk] | ((uint64_t)t[32 + kk] << 32));
}

// Inverse of planes_to_store: slots base + kk for kk in (lo, hi] hold planes
// 32G + kk, the others are zero; OR the slice into the coefficients.
// The low and high 32 bits of the planes (coefficients 0..31 and 32..63)
// are transposed one after the other, which keeps 32 words live, not 64.
template <int G, typename UInt, class PS>
GZ_HD void store_to_coeffs(const PS& ps, int base, int lo, int hi, UInt* u) {
#pragma unroll
  for (int h = 0; h < 2; h++) {
    uint32_t t[32];
#pragma unroll
    for (int kk = 0; kk < 32; kk++)
      t[kk] = (kk > lo && kk <= hi) ? (uint32_t)(ps.get(base + kk) >> (32 * h)) : 0u;
    transpose_tiles<32>(t);
#pragma unroll
    for (int i = 0; i < 32; i++) u[32 * h + i] |= (UInt)((uint64_t)t[i] << (32 * G));
  }
}

// ------------------------------------------------------------- block codec
// The transposed planes are consumed by a rolled loop, so they live in a
// per-thread plane store `PS` (shared memory on the GPU, an array on the
// host): slot i holds a 64-bit value, get(i) / put(i, v).  For 4^3 blocks a
// slot is one plane of the current 32-plane half; for smaller blocks the
// slots are the words of Planes::tw.

// Front end of the encoder: block-floating-point conversion, decorrelating
// transform, sequency reordering and negabinary mapping.
template <int D, typename T>
GZ_HD void front_end(const typename FT<T>::UInt* raw, int emax, typename FT<T>::UInt* u) {
  typedef FT<T> F;
  typedef typename F::UInt UInt;
  typedef typename F::Int Int;
  constexpr int BS = 1 << (2 * D);
  Int q[BS];
  quantize(raw, q, BS, emax);
  fwd_xform<D>(q);
#pragma unroll
  for (int i = 0; i < BS; i++) u[i] = (UInt)(((UInt)q[Perm<D>::at(i)] + (UInt)F::NB) ^ (UInt)F::NB);
}

// Front end of the encoder for an integer block: transform, order, map.
template <int D, typename T>
GZ_HD void front_end_int(const typename FT<T>::UInt* raw, typename FT<T>::UInt* u) {
  typedef FT<T> F;
  typedef typename F::UInt UInt;
  typedef typename F::Int Int;
  constexpr int BS = 1 << (2 * D);
  Int q[BS];
#pragma unroll
  for (int i = 0; i < BS; i++) q[i] = (Int)raw[i];
  fwd_xform<D>(q);
#pragma unroll
  for (int i = 0; i < BS; i++) u[i] = (UInt)(((UInt)q[Perm<D>::at(i)] + (UInt)F::NB) ^ (UInt)F::NB);
}

// ----------------------------------------------------------- coding modes
// zfp's four stream parameters (zfp_stream minbits, maxbits, maxprec,
// minexp; Z/inc/zfp.h:129-135).  FixedRate is the setting of
// zfp_stream_set_rate -- minbits = maxbits, maxprec = the type's precision,
// minexp = ZFP_MIN_EXP -- with only maxbits left open, which is what the
// fixed-rate kernels compile; General holds all four (fixed precision,
// fixed accuracy, or any setting of zfp_stream_set_params).
struct FixedRate {
  static constexpr bool kGeneral = false;
  uint32_t maxbits;
  GZ_HD uint32_t min_bits() const { return maxbits; }
  // planes a floating-point block codes: precision() of
  // Z/src/template/codec{1,2,3}.c with maxprec = P, minexp = ZFP_MIN_EXP
  template <int D, int P>
  GZ_HD int precision(int emax) const {
    const int prec = emax - kMinExp + 2 * D + 2;
    return prec < 0 ? 0 : prec > P ? P : prec;
  }
  template <int P>
  GZ_HD int int_kmin() const { return 0; }
};

struct General {
  static constexpr bool kGeneral = true;
  uint32_t minbits, maxbits, maxprec;
  int minexp;
  GZ_HD uint32_t min_bits() const { return minbits; }
  // MIN(maxprec, MAX(0, emax - minexp + 2 * (D + 1))), at most P
  template <int D, int P>
  GZ_HD int precision(int emax) const {
    int prec = emax - minexp + 2 * D + 2;
    prec = prec < 0 ? 0 : prec;
    prec = prec > (int)maxprec ? (int)maxprec : prec;
    return prec > P ? P : prec;
  }
  // lowest plane of an integer block: P - maxprec (Z/src/template/encode.c:127)
  template <int P>
  GZ_HD int int_kmin() const { return (uint32_t)P > maxprec ? P - (int)maxprec : 0; }
};

// Encode one block of raw IEEE bit patterns (gathered and padded)
// (Z/src/template/encode.c:154-234): exactly maxbits bits in fixed-rate
// mode; in general mode as many as the block takes (at most maxbits, at
// least minbits).  Returns the bits written.
//
// 4^3 double blocks are coded one 32-bit slice (32 planes) at a time; the
// bottom slice waits in plane-store slots 32..63 while the top one is coded,
// so only half of the block's coefficients stay in registers.
template <int D, typename T, class Mode, class W, class PS>
GZ_HD uint32_t encode_block_mode(const typename FT<T>::UInt* raw, const Mode& mode, W& w,
                                 PS& ps) {
  typedef FT<T> F;
  typedef typename F::UInt UInt;
  constexpr int BS = 1 << (2 * D);
  constexpr int P = F::P;
  typedef Planes<D, P> PL;
  const uint32_t maxbits = mode.maxbits;

  UInt u[BS];
  uint32_t bits;
  int kmin;
  if constexpr (F::INT) {
    front_end_int<D, T>(raw, u);
    bits = maxbits;
    kmin = mode.template int_kmin<P>();
  } else {
    // largest exponent field and a nonzero test, from the IEEE bits
    uint32_t maxh = 0, orl = 0;
#pragma unroll
    for (int i = 0; i < BS; i++) {
      uint32_t h = (uint32_t)((uint64_t)raw[i] >> (P - 32)) & 0x7fffffffu;
      maxh = h > maxh ? h : maxh;
      if (P == 64) orl |= (uint32_t)raw[i];
    }
    if constexpr (!Mode::kGeneral) {
      if ((maxh | orl) == 0) {  // all zero: one 0 bit, zero padding
        w.zeros(maxbits);
        return maxbits;
      }
    }
    const int maxE = (int)(maxh >> (F::MANT - (P - 32)));
    const int emax = maxE - (F::EBIAS - 1);  // frexp exponent, >= 1 - EBIAS
    const int prec = mode.template precision<D, P>(emax);
    if constexpr (Mode::kGeneral) {
      // all zero, or nothing above minexp: one 0 bit, zero padding to minbits
      if ((maxh | orl) == 0 || prec == 0) {
        const uint32_t z = mode.min_bits() > 1 ? mode.min_bits() : 1;
        w.zeros(z);
        return z;
      }
    }
    const uint32_t e = (uint32_t)(emax + F::EBIAS);
    w.put(2 * (uint64_t)e + 1, F::EBITS + 1);
    front_end<D, T>(raw, emax, u);
    bits = maxbits - (F::EBITS + 1);
    kmin = P - prec;
  }
  const uint32_t budget = bits;
  uint32_t n = 0;
  int k = P - 1;
  if constexpr (BS == 64 && P == 64) {
    // the low halves wait in registers while the top 32 planes are coded
    uint32_t lo[64];
#pragma unroll
    for (int i = 0; i < 64; i++) lo[i] = (uint32_t)u[i];
    planes_to_store<1>(u, ps);
    k = code_planes<BS>(k, kmin > 32 ? kmin : 32, n, bits, w,
                        [&](int kk) { return ps.get(kk - 32); });
    if (k >= kmin && bits) {
      planes_to_store<0>(lo, ps);
      code_planes<BS>(k, kmin, n, bits, w, [&](int kk) { return ps.get(kk); });
    }
  } else if constexpr (BS == 64) {
    planes_to_store<0>(u, ps);
    code_planes<BS>(k, kmin, n, bits, w, [&](int kk) { return ps.get(kk); });
  } else if constexpr (D == 1) {
    code_planes_4(u, k, kmin, n, bits, w, *ps.t4);
  } else {
    PL pl;
#pragma unroll
    for (int G = 0; G < P / 32; G++) {
      pl.load(u, G);
      pl.transpose(G);
    }
#pragma unroll
    for (int i = 0; i < PL::NW; i++) ps.put(i, pl.tw[i]);
    auto plane = [&](int kp) {
      const int G = kp >> 5, kk = kp & 31, r = kk % PL::N, g = kk / PL::N;
      const uint32_t word = (uint32_t)ps.get(G * BS + r);
      return (uint64_t)((word >> (g * PL::N)) & ((1u << PL::N) - 1));
    };
    // runs while the first coefficient alone is significant
    if constexpr (BS <= 16) {
      UInt above1 = 0;
#pragma unroll
      for (int i = 1; i < BS; i++) above1 |= u[i];
      k = code_runs01<BS>(u[0], (UInt)(u[0] | above1), above1, k, kmin, n, bits, w, plane);
    }
    if (k >= kmin && bits) code_planes<BS>(k, kmin, n, bits, w, plane);
  }
  if constexpr (!Mode::kGeneral) {
    w.zeros(bits);  // pad to exactly maxbits
    return maxbits;
  } else {
    const uint32_t used = (maxbits - budget) + (budget - bits);  // header + coded planes
    const uint32_t pad = used < mode.minbits ? mode.minbits - used : 0;
    w.zeros(pad);
    return used + pad;
  }
}

template <int D, typename T, class W, class PS>
GZ_HD void encode_block(const typename FT<T>::UInt* raw, uint32_t maxbits, W& w, PS& ps) {
  encode_block_mode<D, T>(raw, FixedRate{maxbits}, w, ps);
}

// Decode one block from a reader positioned at its first bit into raw IEEE
// bit patterns (Z/src/template/decode.c:137-165).  Returns the bits the
// block takes in the stream (fixed rate: maxbits; the reader is not moved
// past a block's padding).
struct NoSlice {
  template <typename U>
  GZ_HD void operator()(int, const U*) const {}
};

// SLICED (4^3 floating-point blocks): the values of z slice z go to
// slice(z, 16 values) as soon as they are final, and raw is not written.
template <int D, typename T, bool SLICED = false, class Mode, class R, class PS,
          class SliceFn = NoSlice>
GZ_HD uint32_t decode_block_mode(R& r, const Mode& mode, typename FT<T>::UInt* raw, PS& ps,
                                 SliceFn&& slice = SliceFn{}) {
  typedef FT<T> F;
  typedef typename F::UInt UInt;
  typedef typename F::Int Int;
  constexpr int BS = 1 << (2 * D);
  constexpr int P = F::P;
  typedef Planes<D, P> PL;
  const uint32_t maxbits = mode.maxbits;

  int emax = 0, kmin = 0;
  uint32_t bits = maxbits;
  if constexpr (F::INT) {
    kmin = mode.template int_kmin<P>();
  } else {
    const uint64_t head = r.peek64();
    if (!(head & 1)) {
      if constexpr (D == 3 && SLICED) {
        UInt zs[16];
#pragma unroll
        for (int i = 0; i < 16; i++) zs[i] = 0;
#pragma unroll
        for (int z = 0; z < 4; z++) slice(z, zs);
      } else {
#pragma unroll
        for (int i = 0; i < BS; i++) raw[i] = 0;
      }
      return mode.min_bits() > 1 ? mode.min_bits() : 1;
    }
    r.skip(F::EBITS + 1);
    emax = (int)((head >> 1) & ((1u << F::EBITS) - 1)) - F::EBIAS;
    kmin = P - mode.template precision<D, P>(emax);
    bits = maxbits - (F::EBITS + 1);
  }
  const uint32_t budget = bits;

  uint32_t n = 0;
  int k = P - 1;
  UInt u[BS];
  if constexpr (BS == 64) {
    // planes of the top half into the store, then into the coefficients'
    // top 32-bit slices; the bottom half only if decoding reaches it
#pragma unroll
    for (int i = 0; i < BS; i++) u[i] = 0;
    if constexpr (P == 64) {
      // top-half planes into the store, folded into the coefficients before
      // the bottom half reuses the store
      const int top = k;
      k = uncode_flat64(k, kmin > 32 ? kmin : 32, n, bits, r,
                        [&](int kk, uint64_t x) { ps.put(kk - 32, x); });
      store_to_coeffs<1>(ps, 0, k - 32, top - 32, u);
      if (k >= kmin && bits) {
        const int top0 = k;
        k = uncode_flat64(k, kmin, n, bits, r, [&](int kk, uint64_t x) { ps.put(kk, x); });
        store_to_coeffs<0>(ps, 0, k, top0, u);
      }
    } else {
      const int top = k;
      k = uncode_flat64(k, kmin, n, bits, r, [&](int kk, uint64_t x) { ps.put(kk, x); });
      store_to_coeffs<0>(ps, 0, k, top, u);
    }
  } else if constexpr (D == 1) {
#pragma unroll
    for (int i = 0; i < BS; i++) u[i] = 0;
    uncode_planes_4(u, k, kmin, n, bits, r, *ps.t4);
  } else {
#pragma unroll
    for (int i = 0; i < PL::NW; i++) ps.put(i, 0);
    auto store = [&](int kp, uint64_t x) {
      const int G = kp >> 5, kk = kp & 31, rr = kk % PL::N, g = kk / PL::N;
      ps.put(G * BS + rr, ps.get(G * BS + rr) | (x << (g * PL::N)));
    };
    UInt u0 = 0;  // the runs' bits of the first coefficient
    if constexpr (BS <= 16)
      k = uncode_runs01<BS, P == 32>(u0, k, kmin, n, bits, r, store);
    if (k >= kmin && bits) uncode_planes<BS, P == 32>(k, kmin, n, bits, r, store);
    PL pl;
#pragma unroll
    for (int i = 0; i < PL::NW; i++) pl.tw[i] = (uint32_t)ps.get(i);
#pragma unroll
    for (int G = 0; G < P / 32; G++) pl.transpose(G);
    pl.store(u);
    u[0] |= u0;
  }

  Int q[BS];
#pragma unroll
  for (int i = 0; i < BS; i++) q[Perm<D>::at(i)] = (Int)((u[i] ^ (UInt)F::NB) - (UInt)F::NB);
  if constexpr (D == 3 && !F::INT && SLICED) {
    // inverse lifts along z, then each z slice to the end (y, x, values,
    // sink) before the next, so that a finished slice's values are dead
#pragma unroll
    for (int l = 0; l < 16; l++) inv_lift(q[l], q[l + 16], q[l + 32], q[l + 48]);
#pragma unroll
    for (int z = 0; z < 4; z++) {
      Int* qs = q + 16 * z;
#pragma unroll
      for (int x = 0; x < 4; x++) inv_lift(qs[x], qs[x + 4], qs[x + 8], qs[x + 12]);
#pragma unroll
      for (int y = 0; y < 4; y++) inv_lift(qs[4 * y], qs[4 * y + 1], qs[4 * y + 2], qs[4 * y + 3]);
      UInt rs[16];
      dequantize(qs, rs, 16, emax);
      slice(z, rs);
    }
    const uint32_t used = (maxbits - budget) + (budget - bits);
    return used < mode.min_bits() ? mode.min_bits() : used;
  }
  inv_xform<D>(q);
  if constexpr (F::INT) {
#pragma unroll
    for (int i = 0; i < BS; i++) raw[i] = (UInt)q[i];
  } else {
    dequantize(q, raw, BS, emax);
  }
  const uint32_t used = (maxbits - budget) + (budget - bits);
  return used < mode.min_bits() ? mode.min_bits() : used;
}

template <int D, typename T, class R, class PS>
GZ_HD void decode_block(R& r, uint32_t maxbits, typename FT<T>::UInt* raw, PS& ps) {
  decode_block_mode<D, T>(r, FixedRate{maxbits}, raw, ps);
}

// The bits a block takes in a general-mode stream, from a reader at its
// first bit: the plane decoding of decode_block without the deposit, the
// transform or the values (for locating the blocks of a stream whose block
// offsets are not known).
template <int D, typename T, class R>
GZ_HD uint32_t block_bits(R& r, const General& mode) {
  typedef FT<T> F;
  constexpr int BS = 1 << (2 * D);
  constexpr int P = F::P;
  int kmin;
  uint32_t bits = mode.maxbits, hdr = 0;
  if constexpr (F::INT) {
    kmin = mode.template int_kmin<P>();
  } else {
    const uint64_t head = r.peek64();
    if (!(head & 1)) return mode.minbits > 1 ? mode.minbits : 1;
    r.skip(F::EBITS + 1);
    const int emax = (int)((head >> 1) & ((1u << F::EBITS) - 1)) - F::EBIAS;
    kmin = P - mode.template precision<D, P>(emax);
    hdr = F::EBITS + 1;
    bits -= hdr;
  }
  const uint32_t budget = bits;
  uint32_t n = 0;
  if constexpr (BS == 64)  // the decoder's token loop for 4^3 blocks
    uncode_flat64(P - 1, kmin, n, bits, r, [](int, uint64_t) {});
  else
    uncode_planes<BS>(P - 1, kmin, n, bits, r, [](int, uint64_t) {});
  const uint32_t used = hdr + (budget - bits);
  return used < mode.minbits ? mode.minbits : used;
}

// Plane store backed by a plain array (host builds and tests).
struct LocalPlanes {
  uint64_t v[64];
  const Plane4Tables* t4 = plane4_tables_host();
  GZ_HD uint64_t get(int i) const { return v[i]; }
  GZ_HD void put(int i, uint64_t x) { v[i] = x; }
};

}  // namespace gzfp
