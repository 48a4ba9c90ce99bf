/*
 * zfp_oracle.c -- CPU restatement of the zfp 0.5.0 fixed-rate codec.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * codec in cuzfp_gb300/csrc and the timed CPU baseline ("port") of bench.py.
 * Nothing in the product library links, loads or calls it.
 *
 * It restates, in independent code, the algorithm of the zfp 0.5.0 sources
 * vendored by cuZFP under src/thirdparty_builtin/zfp-0.5.0 (abbreviated Z/):
 *
 *   rate -> bits per block          Z/src/zfp.c:405-430  (wra = 0)
 *   exponent / exponent_block       Z/src/template/encode.c:10-33
 *   fwd_cast (block floating point) Z/src/template/encode.c:36-52
 *   pad_block                       Z/src/template/encode.c:55-74
 *   fwd_lift                        Z/src/template/encode.c:77-103
 *   int2uint / fwd_order            Z/src/template/encode.c:106-119
 *   encode_ints (bit-plane coder)   Z/src/template/encode.c:122-151
 *   encode_block / zfp_encode_block Z/src/template/encode.c:154-234
 *   precision()                     Z/src/template/codec{1,2,3}.c
 *   perm_1 / perm_2 / perm_3        Z/src/template/codec{1,2,3}.c
 *   fwd_xform / gather_partial      Z/src/template/encode{1,2,3}.c
 *   block loops (z, y, x order)     Z/src/template/compress.c:1-104
 *   inverse path                    Z/src/template/decode.c:9-165,
 *                                   Z/src/template/decode{1,2,3}.c,
 *                                   Z/src/template/decompress.c
 *   bit stream (LSB-first u64)      Z/src/inline/bitstream.c:195-373
 *   stream_flush / returned size    Z/src/zfp.c:603-630
 *   full header (magic, field       Z/src/zfp.c:661-719, zfp_field_metadata
 *   metadata, mode)                 :158-182, zfp_field_set_metadata
 *                                   :254-275, zfp_stream_mode :305-345,
 *                                   zfp_stream_set_mode :461-498
 *   int32 / int64 blocks            Z/src/template/encode.c:154-185 (no
 *                                   exponent, whole budget, maxprec 64),
 *                                   decode.c:116-135; zfp 0.5.0 codes them
 *                                   one block at a time
 *                                   (zfp_encode_block_int32_<d>), so arrays
 *                                   use the same block order and, for
 *                                   partial blocks, the same pad rule as
 *                                   the float path
 *
 * Parity is pinned two ways (see tests/test_oracle.py): against a build of
 * the reference's own zfp sources (oracle/_ref, built by oracle/Makefile in
 * a checkout that has the reference) and against committed golden streams in
 * tests/golden that were produced by that build.
 *
 * Defined behaviour where zfp 0.5.0 relies on C undefined behaviour: when a
 * block's largest magnitude is so small that the quantisation scale
 * 2^(P-2-emax) overflows to +inf (f32: emax < -97, f64: emax < -961), zfp
 * casts +-inf / NaN to an integer.  This restatement performs the IEEE-754
 * saturating conversion (+inf -> INT_MAX, -inf -> INT_MIN, NaN -> 0), which is
 * what the reference computes on AArch64 hosts and what CUDA's cvt.rzi does.
 * An x86-64 build of zfp 0.5.0 yields INT_MIN for every value instead.
 * Non-finite inputs (inf, NaN) are outside the codec's domain.
 *
 * The multi-threaded entry points split the block sequence into chunks of a
 * multiple of 64 blocks, so every chunk starts on a 64-bit word boundary of
 * the fixed-rate stream; output is byte-identical to the serial path.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define GZO_INT32 1  /* zfp_type_int32  (Z/inc/zfp.h:107-113) */
#define GZO_INT64 2  /* zfp_type_int64 */
#define GZO_FLOAT 3  /* zfp_type_float */
#define GZO_DOUBLE 4 /* zfp_type_double */
#define GZO_IS_INT(t) ((t) == GZO_INT32 || (t) == GZO_INT64)
#define GZO_MIN_EXP (-1074)

/* ---------------------------------------------------------------- bits --- */

typedef struct {
  uint64_t* words; /* word array */
  size_t pos;      /* next word index */
  uint64_t acc;    /* pending bits (LSB first) */
  unsigned fill;   /* number of pending bits, < 64 */
} wbits;

static void w_init(wbits* w, uint64_t* words, size_t bitoff) {
  /* bitoff is a multiple of 64 for every caller */
  w->words = words;
  w->pos = bitoff / 64;
  w->acc = 0;
  w->fill = 0;
}

/* append the low n (0..64) bits of v */
static void w_put(wbits* w, uint64_t v, unsigned n) {
  if (n == 0) return;
  if (n < 64) v &= ((uint64_t)1 << n) - 1;
  w->acc |= v << w->fill;
  if (w->fill + n >= 64) {
    w->words[w->pos++] = w->acc;
    unsigned used = 64 - w->fill; /* bits of v consumed by that word */
    w->acc = used < 64 ? v >> used : 0;
    w->fill = w->fill + n - 64;
  } else {
    w->fill += n;
  }
}

static void w_zeros(wbits* w, size_t n) {
  while (n >= 64) { w_put(w, 0, 64); n -= 64; }
  w_put(w, 0, (unsigned)n);
}

static void w_flush(wbits* w) {
  if (w->fill) { w->words[w->pos++] = w->acc; w->acc = 0; w->fill = 0; }
}

typedef struct {
  const uint64_t* words;
  size_t bit; /* absolute bit position of the next bit */
} rbits;

static uint64_t r_get(rbits* r, unsigned n) {
  if (n == 0) return 0;
  size_t wi = r->bit / 64;
  unsigned sh = (unsigned)(r->bit % 64);
  uint64_t v = r->words[wi] >> sh;
  if (sh && sh + n > 64) v |= r->words[wi + 1] << (64 - sh);
  r->bit += n;
  if (n < 64) v &= ((uint64_t)1 << n) - 1;
  return v;
}

/* --------------------------------------------------------- permutations --- */

/* sequency order of the coefficients: sort (i,j,k) by i+j+k, then by
   i^2+j^2+k^2; the exact tie order is that of Z/src/template/codec3.c:4-88 and
   codec2.c:4-30 and is reproduced here as index tables */
static const unsigned char PERM1[4] = {0, 1, 2, 3};
static const unsigned char PERM2[16] = {0, 1, 4, 5, 2, 8, 6, 9, 3, 12, 10, 7, 13, 11, 14, 15};
static const unsigned char PERM3[64] = {
    0,  1,  4,  16, 20, 17, 5,  2,  8,  32, 21, 6,  18, 24, 9,  33,
    36, 3,  12, 48, 22, 25, 37, 40, 34, 10, 7,  19, 28, 13, 49, 52,
    41, 38, 26, 23, 29, 53, 11, 35, 44, 14, 50, 56, 42, 27, 39, 45,
    30, 54, 57, 60, 51, 15, 43, 46, 58, 61, 55, 31, 62, 59, 47, 63};

static const unsigned char* perm_for(int dims) {
  return dims == 1 ? PERM1 : dims == 2 ? PERM2 : PERM3;
}

/* ------------------------------------------------------------ lifting ---- */

/* Lifting steps in wrap-around integer arithmetic; ">>" is the arithmetic
   shift of zfp's signed Int (Z/src/template/encode.c:77-103,
   decode.c:28-54).  Wrapping only matters for streams that do not come from
   the encoder, where zfp's signed overflow is undefined in C. */
#define ADD64(a, b) ((int64_t)((uint64_t)(a) + (uint64_t)(b)))
#define SUB64(a, b) ((int64_t)((uint64_t)(a) - (uint64_t)(b)))
#define SHL64(a) ((int64_t)((uint64_t)(a) << 1))
#define ADD32(a, b) ((int32_t)((uint32_t)(a) + (uint32_t)(b)))
#define SUB32(a, b) ((int32_t)((uint32_t)(a) - (uint32_t)(b)))
#define SHL32(a) ((int32_t)((uint32_t)(a) << 1))

static void lift_fwd(int64_t* p, int s) {
  int64_t x = p[0], y = p[s], z = p[2 * s], w = p[3 * s];
  x = ADD64(x, w); x >>= 1; w = SUB64(w, x);
  z = ADD64(z, y); z >>= 1; y = SUB64(y, z);
  x = ADD64(x, z); x >>= 1; z = SUB64(z, x);
  w = ADD64(w, y); w >>= 1; y = SUB64(y, w);
  w = ADD64(w, y >> 1); y = SUB64(y, w >> 1);
  p[0] = x; p[s] = y; p[2 * s] = z; p[3 * s] = w;
}

static void lift_inv(int64_t* p, int s) {
  int64_t x = p[0], y = p[s], z = p[2 * s], w = p[3 * s];
  y = ADD64(y, w >> 1); w = SUB64(w, y >> 1);
  y = ADD64(y, w); w = SHL64(w); w = SUB64(w, y);
  z = ADD64(z, x); x = SHL64(x); x = SUB64(x, z);
  y = ADD64(y, z); z = SHL64(z); z = SUB64(z, y);
  w = ADD64(w, x); x = SHL64(x); x = SUB64(x, w);
  p[0] = x; p[s] = y; p[2 * s] = z; p[3 * s] = w;
}

static void lift_fwd32(int32_t* p, int s) {
  int32_t x = p[0], y = p[s], z = p[2 * s], w = p[3 * s];
  x = ADD32(x, w); x >>= 1; w = SUB32(w, x);
  z = ADD32(z, y); z >>= 1; y = SUB32(y, z);
  x = ADD32(x, z); x >>= 1; z = SUB32(z, x);
  w = ADD32(w, y); w >>= 1; y = SUB32(y, w);
  w = ADD32(w, y >> 1); y = SUB32(y, w >> 1);
  p[0] = x; p[s] = y; p[2 * s] = z; p[3 * s] = w;
}

static void lift_inv32(int32_t* p, int s) {
  int32_t x = p[0], y = p[s], z = p[2 * s], w = p[3 * s];
  y = ADD32(y, w >> 1); w = SUB32(w, y >> 1);
  y = ADD32(y, w); w = SHL32(w); w = SUB32(w, y);
  z = ADD32(z, x); x = SHL32(x); x = SUB32(x, z);
  y = ADD32(y, z); z = SHL32(z); z = SUB32(z, y);
  w = ADD32(w, x); x = SHL32(x); x = SUB32(x, w);
  p[0] = x; p[s] = y; p[2 * s] = z; p[3 * s] = w;
}

/* the 1D/2D/3D transforms: x lines (stride 1), then y (stride 4), then z
   (stride 16); the inverse runs z, y, x */
static void xform(void* blk, int dims, int wide, int inverse) {
  int n = 1 << (2 * dims);
  int lines = n / 4;
  int axis, a, l;
  for (a = 0; a < dims; a++) {
    axis = inverse ? dims - 1 - a : a;
    int stride = 1 << (2 * axis);
    for (l = 0; l < lines; l++) {
      /* l enumerates the coordinates other than `axis` */
      int lo = l % stride;
      int hi = l / stride;
      int base = lo + hi * stride * 4;
      if (wide) {
        int64_t* p = (int64_t*)blk + base;
        if (inverse) lift_inv(p, stride); else lift_fwd(p, stride);
      } else {
        int32_t* p = (int32_t*)blk + base;
        if (inverse) lift_inv32(p, stride); else lift_fwd32(p, stride);
      }
    }
  }
}

/* ------------------------------------------------------------- params ---- */

typedef struct {
  int type, dims;
  unsigned nx, ny, nz; /* per-axis sizes (1 for unused axes) */
  unsigned bx, by, bz; /* blocks per axis */
  unsigned maxbits;
  /* the rest of zfp_stream's parameters (Z/inc/zfp.h:129-135); fixed rate
     as zfp_stream_set_rate leaves them: minbits = maxbits, maxprec = P,
     minexp = ZFP_MIN_EXP */
  unsigned minbits, maxprec;
  int minexp;
  int P;      /* bits per integer: 32 or 64 */
  int ebits;  /* exponent bits: 8 or 11 */
  int ebias;  /* 127 or 1023 */
  long long sx, sy, sz; /* element strides (zfp_field sx/sy/sz, 0 = contiguous) */
} params;

/* zfp_stream_set_rate, wra = 0 (Z/src/zfp.c:405-430): floor(4^d rate + 0.5)
   bits per block, raised to 1 + EBITS for float and double only */
unsigned gzo_maxbits(int type, int dims, double rate) {
  unsigned n = 1u << (2 * dims);
  unsigned bits = (unsigned)floor(n * rate + 0.5);
  unsigned lo = type == GZO_FLOAT ? 9u : type == GZO_DOUBLE ? 12u : 0u;
  return bits < lo ? lo : bits;
}

/* geometry and codec constants for `maxbits` bits per block */
static int setup_bits(params* p, int type, unsigned nx, unsigned ny, unsigned nz,
                      unsigned maxbits) {
  if (type != GZO_FLOAT && type != GZO_DOUBLE && !GZO_IS_INT(type)) return 0;
  if (nx == 0) return 0;
  p->dims = nz ? 3 : ny ? 2 : 1;
  if (nz && !ny) return 0;
  p->type = type;
  p->nx = nx; p->ny = ny ? ny : 1; p->nz = nz ? nz : 1;
  p->bx = (p->nx + 3) / 4; p->by = (p->ny + 3) / 4; p->bz = (p->nz + 3) / 4;
  p->maxbits = maxbits;
  if (p->maxbits == 0) return 0;
  p->P = type == GZO_FLOAT || type == GZO_INT32 ? 32 : 64;
  p->minbits = maxbits;
  p->maxprec = (unsigned)p->P;
  p->minexp = GZO_MIN_EXP;
  /* integer blocks carry no exponent (Z/src/template/encode.c:176-185) */
  p->ebits = type == GZO_FLOAT ? 8 : type == GZO_DOUBLE ? 11 : 0;
  p->ebias = p->ebits ? (1 << (p->ebits - 1)) - 1 : 0;
  p->sx = 1;
  p->sy = p->nx;
  p->sz = (long long)p->nx * p->ny;
  return 1;
}

static int setup(params* p, int type, unsigned nx, unsigned ny, unsigned nz, double rate) {
  return setup_bits(p, type, nx, ny, nz, gzo_maxbits(type, nz ? 3 : ny ? 2 : 1, rate));
}

static size_t scalar_bytes(const params* p) { return p->P == 32 ? 4 : 8; }

size_t gzo_stream_bytes(int type, unsigned nx, unsigned ny, unsigned nz, double rate) {
  params p;
  if (!setup(&p, type, nx, ny, nz, rate)) return 0;
  uint64_t blocks = (uint64_t)p.bx * p.by * p.bz;
  return (size_t)((blocks * p.maxbits + 63) / 64 * 8);
}

/* ------------------------------------------------------------- encoder --- */

/* IEEE-754 saturating float->int conversion (see the header comment) */
static int64_t sat_i64(double v) {
  if (v != v) return 0;
  if (v >= 9223372036854775808.0) return INT64_MAX;
  if (v < -9223372036854775808.0) return INT64_MIN;
  return (int64_t)v;
}
static int32_t sat_i32(float v) {
  if (v != v) return 0;
  if (v >= 2147483648.0f) return INT32_MAX;
  if (v < -2147483648.0f) return INT32_MIN;
  return (int32_t)v;
}

/* the embedded bit-plane coder; returns bits written (<= budget) */
static unsigned encode_planes(wbits* w, unsigned budget, int intprec, int kmin,
                              const uint64_t* u, int size) {
  unsigned bits = budget;
  int k = intprec, n = 0;
  while (bits && k-- > kmin) {
    uint64_t x = 0;
    int i;
    for (i = 0; i < size; i++) x |= ((u[i] >> k) & 1u) << i;
    /* first n bits of the plane go out verbatim */
    unsigned m = (unsigned)n < bits ? (unsigned)n : bits;
    bits -= m;
    w_put(w, x, m);
    x = m < 64 ? x >> m : 0;
    /* group tests: is anything left in the plane?  then a unary run up to
       the next one bit; a one in the last position is implied */
    while (n < size && bits) {
      bits--;
      unsigned any = x != 0;
      w_put(w, any, 1);
      if (!any) break;
      while (n < size - 1 && bits) {
        bits--;
        unsigned b = (unsigned)(x & 1u);
        w_put(w, b, 1);
        if (b) break;
        x >>= 1;
        n++;
      }
      x >>= 1;
      n++;
    }
  }
  return budget - bits;
}

/* lowest plane an integer block codes: P - maxprec (Z/src/template/
   encode.c:127, kmin) */
static int int_kmin(const params* p) {
  return (unsigned)p->P > p->maxprec ? p->P - (int)p->maxprec : 0;
}

/* the planes a floating-point block with exponent emax codes: precision()
   of Z/src/template/codec{1,2,3}.c, MIN(maxprec, MAX(0, emax - minexp +
   2 * (dims + 1))) */
static int float_precision(const params* p, int emax) {
  int prec = emax - p->minexp + 2 * p->dims + 2;
  if (prec < 0) prec = 0;
  if (prec > (int)p->maxprec) prec = (int)p->maxprec;
  if (prec > p->P) prec = p->P;
  return prec;
}

/* integer block: decorrelating transform, order, embedded coding of up to
   maxbits bits and maxprec planes, zero padding to minbits (encode_block
   for Int, Z/src/template/encode.c:154-171, called by
   zfp_encode_block_int32_<d> / int64, :176-185) */
static void encode_int_block(wbits* w, const params* p, const void* iblock) {
  int size = 1 << (2 * p->dims);
  int i;
  uint64_t u[64];
  const unsigned char* perm = perm_for(p->dims);
  if (p->P == 32) {
    int32_t q[64];
    memcpy(q, iblock, (size_t)size * 4);
    xform(q, p->dims, 0, 0);
    for (i = 0; i < size; i++)
      u[i] = (uint32_t)(((uint32_t)q[perm[i]] + 0xaaaaaaaau) ^ 0xaaaaaaaau);
  } else {
    int64_t q[64];
    memcpy(q, iblock, (size_t)size * 8);
    xform(q, p->dims, 1, 0);
    for (i = 0; i < size; i++)
      u[i] = ((uint64_t)q[perm[i]] + 0xaaaaaaaaaaaaaaaaull) ^ 0xaaaaaaaaaaaaaaaaull;
  }
  unsigned used = encode_planes(w, p->maxbits, p->P, int_kmin(p), u, size);
  if (used < p->minbits) w_zeros(w, p->minbits - used);
}

static void encode_block(wbits* w, const params* p, const void* fblock) {
  int size = 1 << (2 * p->dims);
  int i;
  if (GZO_IS_INT(p->type)) {
    encode_int_block(w, p, fblock);
    return;
  }
  /* largest magnitude -> common exponent (frexp convention) */
  int emax;
  if (p->type == GZO_FLOAT) {
    const float* f = (const float*)fblock;
    float mx = 0;
    for (i = 0; i < size; i++) { float a = fabsf(f[i]); if (mx < a) mx = a; }
    if (mx > 0) { int e; frexpf(mx, &e); emax = e < 1 - p->ebias ? 1 - p->ebias : e; }
    else emax = -p->ebias;
  } else {
    const double* f = (const double*)fblock;
    double mx = 0;
    for (i = 0; i < size; i++) { double a = fabs(f[i]); if (mx < a) mx = a; }
    if (mx > 0) { int e; frexp(mx, &e); emax = e < 1 - p->ebias ? 1 - p->ebias : e; }
    else emax = -p->ebias;
  }
  int prec = float_precision(p, emax);
  unsigned e = prec ? (unsigned)(emax + p->ebias) : 0;
  if (!e) {
    /* all-zero block (or nothing above minexp): one 0 bit, then zero
       padding up to minbits */
    w_zeros(w, p->minbits > 1 ? p->minbits : 1);
    return;
  }
  unsigned hbits = (unsigned)p->ebits + 1;
  w_put(w, 2 * (uint64_t)e + 1, hbits);
  uint64_t u[64];
  const unsigned char* perm = perm_for(p->dims);
  if (p->type == GZO_FLOAT) {
    int32_t q[64];
    const float* f = (const float*)fblock;
    float s = ldexpf(1.0f, p->P - 2 - emax);
    for (i = 0; i < size; i++) q[i] = sat_i32(s * f[i]);
    xform(q, p->dims, 0, 0);
    for (i = 0; i < size; i++)
      u[i] = (uint32_t)(((uint32_t)q[perm[i]] + 0xaaaaaaaau) ^ 0xaaaaaaaau);
  } else {
    int64_t q[64];
    const double* f = (const double*)fblock;
    double s = ldexp(1.0, p->P - 2 - emax);
    for (i = 0; i < size; i++) q[i] = sat_i64(s * f[i]);
    xform(q, p->dims, 1, 0);
    for (i = 0; i < size; i++)
      u[i] = ((uint64_t)q[perm[i]] + 0xaaaaaaaaaaaaaaaaull) ^ 0xaaaaaaaaaaaaaaaaull;
  }
  unsigned budget = p->maxbits - hbits;
  unsigned used = encode_planes(w, budget, p->P, p->P - prec, u, size);
  if (used + hbits < p->minbits) w_zeros(w, p->minbits - hbits - used);
}

/* pad rule of Z/src/template/encode.c:55-74 expressed as an index map */
static unsigned padmap(unsigned n, unsigned i) {
  static const unsigned char map[5][4] = {
      {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 1, 1, 0}, {0, 1, 2, 0}, {0, 1, 2, 3}};
  return map[n][i];
}

static void gather(const params* p, const void* data, unsigned bx, unsigned by, unsigned bz,
                   void* blk) {
  unsigned cx = p->nx - 4 * bx, cy = p->ny - 4 * by, cz = p->nz - 4 * bz;
  cx = cx > 4 ? 4 : cx; cy = cy > 4 ? 4 : cy; cz = cz > 4 ? 4 : cz;
  unsigned dz = p->dims == 3 ? 4 : 1, dy = p->dims >= 2 ? 4 : 1;
  unsigned x, y, z;
  for (z = 0; z < dz; z++)
    for (y = 0; y < dy; y++)
      for (x = 0; x < 4; x++) {
        size_t gx = 4 * bx + padmap(cx, x);
        size_t gy = p->dims >= 2 ? 4 * by + padmap(cy, y) : 0;
        size_t gz = p->dims == 3 ? 4 * bz + padmap(cz, z) : 0;
        long long idx = (long long)gx * p->sx + (long long)gy * p->sy + (long long)gz * p->sz;
        unsigned o = x + 4 * y + 16 * z;
        const size_t es = scalar_bytes(p);  /* memcpy: any scalar type, no aliasing */
        memcpy((char*)blk + o * es, (const char*)data + idx * es, es);
      }
}

/* ------------------------------------------------------------- decoder --- */

static unsigned decode_planes(rbits* r, unsigned budget, int intprec, int kmin, uint64_t* u,
                              int size) {
  unsigned bits = budget;
  int k = intprec, n = 0, i;
  for (i = 0; i < size; i++) u[i] = 0;
  while (bits && k-- > kmin) {
    unsigned m = (unsigned)n < bits ? (unsigned)n : bits;
    bits -= m;
    uint64_t x = r_get(r, m);
    while (n < size && bits) {
      bits--;
      if (!r_get(r, 1)) break;
      while (n < size - 1 && bits) {
        bits--;
        if (r_get(r, 1)) break;
        n++;
      }
      /* a one at position n: read, implied by position, or assumed when the
         budget ran out (Z/src/template/decode.c:94-98) */
      x += (uint64_t)1 << n;
      n++;
    }
    for (i = 0; x; i++, x >>= 1) u[i] += (x & 1u) << k;
  }
  return budget - bits;
}

/* inverse of encode_int_block (zfp_decode_block_int32_<d> / int64) */
static void decode_int_block(rbits* r, const params* p, void* iblock) {
  int size = 1 << (2 * p->dims);
  int i;
  size_t start = r->bit;
  uint64_t u[64];
  unsigned used = decode_planes(r, p->maxbits, p->P, int_kmin(p), u, size);
  r->bit = start + (used < p->minbits ? p->minbits : used);
  const unsigned char* perm = perm_for(p->dims);
  if (p->P == 32) {
    int32_t q[64];
    for (i = 0; i < size; i++)
      q[perm[i]] = (int32_t)(((uint32_t)u[i] ^ 0xaaaaaaaau) - 0xaaaaaaaau);
    xform(q, p->dims, 0, 1);
    memcpy(iblock, q, (size_t)size * 4);
  } else {
    int64_t q[64];
    for (i = 0; i < size; i++)
      q[perm[i]] = (int64_t)((u[i] ^ 0xaaaaaaaaaaaaaaaaull) - 0xaaaaaaaaaaaaaaaaull);
    xform(q, p->dims, 1, 1);
    memcpy(iblock, q, (size_t)size * 8);
  }
}

static void decode_block(rbits* r, const params* p, void* fblock) {
  int size = 1 << (2 * p->dims);
  int i;
  if (GZO_IS_INT(p->type)) {
    decode_int_block(r, p, fblock);
    return;
  }
  size_t start = r->bit;
  if (!r_get(r, 1)) {
    if (p->type == GZO_FLOAT) for (i = 0; i < size; i++) ((float*)fblock)[i] = 0;
    else for (i = 0; i < size; i++) ((double*)fblock)[i] = 0;
    r->bit = start + (p->minbits > 1 ? p->minbits : 1);
    return;
  }
  unsigned hbits = (unsigned)p->ebits + 1;
  int emax = (int)r_get(r, (unsigned)p->ebits) - p->ebias;
  int prec = float_precision(p, emax);
  uint64_t u[64];
  unsigned used = hbits + decode_planes(r, p->maxbits - hbits, p->P, p->P - prec, u, size);
  r->bit = start + (used < p->minbits ? p->minbits : used);
  const unsigned char* perm = perm_for(p->dims);
  if (p->type == GZO_FLOAT) {
    int32_t q[64];
    for (i = 0; i < size; i++)
      q[perm[i]] = (int32_t)(((uint32_t)u[i] ^ 0xaaaaaaaau) - 0xaaaaaaaau);
    xform(q, p->dims, 0, 1);
    float s = ldexpf(1.0f, emax - (p->P - 2));
    for (i = 0; i < size; i++) ((float*)fblock)[i] = s * (float)q[i];
  } else {
    int64_t q[64];
    for (i = 0; i < size; i++)
      q[perm[i]] = (int64_t)((u[i] ^ 0xaaaaaaaaaaaaaaaaull) - 0xaaaaaaaaaaaaaaaaull);
    xform(q, p->dims, 1, 1);
    double s = ldexp(1.0, emax - (p->P - 2));
    for (i = 0; i < size; i++) ((double*)fblock)[i] = s * (double)q[i];
  }
}

static void scatter(const params* p, void* data, unsigned bx, unsigned by, unsigned bz,
                    const void* blk) {
  unsigned cx = p->nx - 4 * bx, cy = p->ny - 4 * by, cz = p->nz - 4 * bz;
  cx = cx > 4 ? 4 : cx; cy = cy > 4 ? 4 : cy; cz = cz > 4 ? 4 : cz;
  if (p->dims < 3) cz = 1;
  if (p->dims < 2) cy = 1;
  unsigned x, y, z;
  for (z = 0; z < cz; z++)
    for (y = 0; y < cy; y++)
      for (x = 0; x < cx; x++) {
        long long idx = (long long)(4 * bx + x) * p->sx + (long long)(4 * by + y) * p->sy +
                        (long long)(4 * bz + z) * p->sz;
        unsigned o = x + 4 * y + 16 * z;
        const size_t es = scalar_bytes(p);
        memcpy((char*)data + idx * es, (const char*)blk + o * es, es);
      }
}

/* ------------------------------------------------------------- drivers --- */

typedef struct {
  const params* p;
  const void* data;
  void* out;
  uint64_t* stream;
  const uint64_t* istream;
  uint64_t b0, b1; /* block range [b0, b1) */
} job;

static void* encode_range(void* arg) {
  job* j = (job*)arg;
  const params* p = j->p;
  wbits w;
  w_init(&w, j->stream, (size_t)(j->b0 * p->maxbits));
  double blk[64];
  uint64_t b;
  for (b = j->b0; b < j->b1; b++) {
    unsigned bx = (unsigned)(b % p->bx);
    unsigned by = (unsigned)((b / p->bx) % p->by);
    unsigned bz = (unsigned)(b / ((uint64_t)p->bx * p->by));
    gather(p, j->data, bx, by, bz, blk);
    encode_block(&w, p, blk);
  }
  w_flush(&w);
  return 0;
}

static void* decode_range(void* arg) {
  job* j = (job*)arg;
  const params* p = j->p;
  rbits r;
  r.words = j->istream;
  r.bit = (size_t)(j->b0 * p->maxbits);
  double blk[64];
  uint64_t b;
  for (b = j->b0; b < j->b1; b++) {
    unsigned bx = (unsigned)(b % p->bx);
    unsigned by = (unsigned)((b / p->bx) % p->by);
    unsigned bz = (unsigned)(b / ((uint64_t)p->bx * p->by));
    decode_block(&r, p, blk);
    scatter(p, j->out, bx, by, bz, blk);
  }
  return 0;
}

static void run_jobs(const params* p, job* proto, uint64_t nblocks, int nthreads,
                     void* (*fn)(void*)) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  /* chunks of a multiple of 64 blocks start on word boundaries */
  uint64_t per = (nblocks + (uint64_t)nthreads - 1) / (uint64_t)nthreads;
  per = (per + 63) / 64 * 64;
  if (per == 0) per = 64;
  pthread_t th[256];
  job jobs[256];
  int t, started = 0;
  for (t = 0; t < nthreads; t++) {
    jobs[t] = *proto;
    jobs[t].b0 = per * (uint64_t)t;
    jobs[t].b1 = jobs[t].b0 + per;
    if (jobs[t].b0 >= nblocks) break;
    if (jobs[t].b1 > nblocks) jobs[t].b1 = nblocks;
  }
  started = t;
  if (started == 1) { fn(&jobs[0]); return; }
  for (t = 0; t < started; t++) pthread_create(&th[t], 0, fn, &jobs[t]);
  for (t = 0; t < started; t++) pthread_join(th[t], 0);
  (void)p;
}

/* Compress a contiguous a[nz][ny][nx] array (ny = nz = 0 for 1D, nz = 0 for
   2D) at `rate` bits per value.  Returns the stream size in bytes (a whole
   number of 64-bit words), or 0 on a bad argument or short buffer. */
size_t gzo_compress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                    const void* data, void* stream, size_t capacity, int nthreads) {
  params p;
  if (!setup(&p, type, nx, ny, nz, rate)) return 0;
  size_t bytes = gzo_stream_bytes(type, nx, ny, nz, rate);
  if (capacity < bytes) return 0;
  uint64_t nblocks = (uint64_t)p.bx * p.by * p.bz;
  job proto;
  memset(&proto, 0, sizeof proto);
  proto.p = &p;
  proto.data = data;
  proto.stream = (uint64_t*)stream;
  run_jobs(&p, &proto, nblocks, nthreads, encode_range);
  return bytes;
}

/* Decompress a stream made by gzo_compress (or zfp 0.5.0 in fixed-rate mode)
   into a contiguous array.  Returns 1 on success, 0 on a bad argument. */
int gzo_decompress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                   const void* stream, size_t bytes, void* data, int nthreads) {
  params p;
  if (!setup(&p, type, nx, ny, nz, rate)) return 0;
  if (bytes < gzo_stream_bytes(type, nx, ny, nz, rate)) return 0;
  uint64_t nblocks = (uint64_t)p.bx * p.by * p.bz;
  job proto;
  memset(&proto, 0, sizeof proto);
  proto.p = &p;
  proto.out = data;
  proto.istream = (const uint64_t*)stream;
  run_jobs(&p, &proto, nblocks, nthreads, decode_range);
  return 1;
}

/* Strided fields (zfp_field sx/sy/sz; Z/src/template/compress.c,
   compress_strided / decompress_strided): value (x, y, z) at element
   x*sx + y*sy + z*sz of `data`, 0 meaning the contiguous stride. */
static void set_strides(params* p, long long sx, long long sy, long long sz) {
  p->sx = sx ? sx : 1;
  p->sy = sy ? sy : (long long)p->nx;
  p->sz = sz ? sz : (long long)p->nx * p->ny;
}

size_t gzo_compress_strided(int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                            long long sy, long long sz, double rate, const void* data,
                            void* stream, size_t capacity, int nthreads) {
  params p;
  if (!setup(&p, type, nx, ny, nz, rate)) return 0;
  set_strides(&p, sx, sy, sz);
  size_t bytes = gzo_stream_bytes(type, nx, ny, nz, rate);
  if (capacity < bytes) return 0;
  job proto;
  memset(&proto, 0, sizeof proto);
  proto.p = &p;
  proto.data = data;
  proto.stream = (uint64_t*)stream;
  run_jobs(&p, &proto, (uint64_t)p.bx * p.by * p.bz, nthreads, encode_range);
  return bytes;
}

int gzo_decompress_strided(int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                           long long sy, long long sz, double rate, const void* stream,
                           size_t bytes, void* data, int nthreads) {
  params p;
  if (!setup(&p, type, nx, ny, nz, rate)) return 0;
  set_strides(&p, sx, sy, sz);
  if (bytes < gzo_stream_bytes(type, nx, ny, nz, rate)) return 0;
  job proto;
  memset(&proto, 0, sizeof proto);
  proto.p = &p;
  proto.out = data;
  proto.istream = (const uint64_t*)stream;
  run_jobs(&p, &proto, (uint64_t)p.bx * p.by * p.bz, nthreads, decode_range);
  return 1;
}

/* ---------------------------------------------------------------- header --- */

/* zfp_write_header(zfp, field, ZFP_HEADER_FULL) for the parameters that
   zfp_stream_set_rate sets (minbits = maxbits, maxprec = the type's
   precision, minexp = ZFP_MIN_EXP): 'z' 'f' 'p' and ZFP_VERSION >> 4 in 8
   bits each; 52 bits of metadata (sizes minus one -- 48 bits in 1D, 24 per
   axis in 2D, 16 per axis in 3D -- then dims - 1 and type - 1 in 2 bits
   each); the mode in 12 bits (maxbits - 1) when maxprec reaches 64 and
   maxbits <= 2048, otherwise 64 bits holding minexp + 16495 (15 bits),
   maxprec - 1 (7), maxbits - 1 (15), minbits - 1 (15) and 0xfff (12).
   Returns the header length in bits, or 0 for sizes or a rate the header
   cannot record. */
static unsigned header_put(wbits* w, const params* p) {
  uint64_t meta, mode;
  unsigned mbits = 12;
  if (p->dims == 2 && (p->nx > (1u << 24) || p->ny > (1u << 24))) return 0;
  if (p->dims == 3 && (p->nx > (1u << 16) || p->ny > (1u << 16) || p->nz > (1u << 16))) return 0;
  /* zfp_stream_mode: the three 12-bit forms, else every parameter */
  if (p->minbits == p->maxbits && p->maxbits >= 1 && p->maxbits <= 2048 && p->maxprec >= 64 &&
      p->minexp <= GZO_MIN_EXP) {
    mode = p->maxbits - 1u;
  } else if (p->minbits == 0 && p->maxbits >= 4171 && p->maxprec >= 1 && p->maxprec <= 128 &&
             p->minexp <= GZO_MIN_EXP) {
    mode = p->maxprec + 2047u;
  } else if (p->minbits == 0 && p->maxbits >= 4171 && p->maxprec >= 64 &&
             p->minexp >= GZO_MIN_EXP && p->minexp <= 843) {
    mode = (uint64_t)(p->minexp + 3251);
  } else {
    /* the 64-bit form would clamp these: no header records them */
    if (p->minbits > 0x8000u || p->maxbits > 0x8000u || p->minexp + 16495 < 0 ||
        p->minexp + 16495 > 0x7fff)
      return 0;
    mbits = 64;
    mode = (uint64_t)(p->minexp + 16495);
    mode = mode << 7 | (uint64_t)(p->maxprec - 1);
    mode = mode << 15 | (uint64_t)(p->maxbits - 1);
    mode = mode << 15 | (uint64_t)(p->minbits ? p->minbits - 1 : 0);
    mode = mode << 12 | 0xfffu;
  }
  w_put(w, 'z', 8);
  w_put(w, 'f', 8);
  w_put(w, 'p', 8);
  w_put(w, 0x05, 8);
  if (p->dims == 1)
    meta = p->nx - 1u;
  else if (p->dims == 2)
    meta = (uint64_t)(p->ny - 1u) << 24 | (p->nx - 1u);
  else
    meta = (uint64_t)(p->nz - 1u) << 32 | (uint64_t)(p->ny - 1u) << 16 | (p->nx - 1u);
  meta = meta << 4 | (uint64_t)(p->dims - 1) << 2 | (uint64_t)(p->type - 1);
  w_put(w, meta, 52);
  w_put(w, mode, mbits);
  return 32 + 52 + mbits;
}

static size_t headed_bytes(const params* p, unsigned header_bits) {
  uint64_t blocks = (uint64_t)p->bx * p->by * p->bz;
  return (size_t)((header_bits + blocks * p->maxbits + 63) / 64 * 8);
}

/* Header bits a stream of this field and rate starts with (0 if none fits) */
unsigned gzo_header_bits(int type, unsigned nx, unsigned ny, unsigned nz, double rate) {
  params p;
  uint64_t scratch[3];
  wbits w;
  if (!setup(&p, type, nx, ny, nz, rate)) return 0;
  w_init(&w, scratch, 0);
  return header_put(&w, &p);
}

/* The header, then every block right after it, one thread (the blocks do
   not start on word boundaries).  Returns the stream size in bytes. */
size_t gzo_compress_headed(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                           const void* data, void* stream, size_t capacity) {
  params p;
  uint64_t scratch[3];
  wbits w;
  unsigned hb;
  size_t bytes;
  uint64_t b, nblocks;
  double blk[64];
  if (!setup(&p, type, nx, ny, nz, rate)) return 0;
  w_init(&w, scratch, 0);
  hb = header_put(&w, &p);
  if (!hb) return 0;
  bytes = headed_bytes(&p, hb);
  if (capacity < bytes) return 0;
  w_init(&w, (uint64_t*)stream, 0);
  header_put(&w, &p);
  nblocks = (uint64_t)p.bx * p.by * p.bz;
  for (b = 0; b < nblocks; b++) {
    unsigned bx = (unsigned)(b % p.bx);
    unsigned by = (unsigned)((b / p.bx) % p.by);
    unsigned bz = (unsigned)(b / ((uint64_t)p.bx * p.by));
    gather(&p, data, bx, by, bz, blk);
    encode_block(&w, &p, blk);
  }
  w_flush(&w);
  return bytes;
}

/* zfp_read_header(ZFP_HEADER_FULL): returns the header bits, 0 for a bad
   magic or a short buffer, -1 for a stream in a mode other than the fixed
   rate zfp_stream_set_rate sets.  ny = 0 (1D) and nz = 0 (1D, 2D) as in
   the rest of this file's entry points. */
long gzo_read_header(const void* stream, size_t bytes, int* type, unsigned* nx, unsigned* ny,
                     unsigned* nz, unsigned* maxbits) {
  uint64_t words[3] = {0, 0, 0};
  rbits r;
  uint64_t meta, mode;
  int dims, t;
  long bits = 32 + 52 + 12;
  memcpy(words, stream, bytes < sizeof words ? bytes : sizeof words);
  if (bytes * 8 < (size_t)bits) return 0;
  r.words = words;
  r.bit = 0;
  if (r_get(&r, 8) != 'z' || r_get(&r, 8) != 'f' || r_get(&r, 8) != 'p' || r_get(&r, 8) != 0x05)
    return 0;
  meta = r_get(&r, 52);
  t = (int)(meta & 3) + 1;
  dims = (int)(meta >> 2 & 3) + 1;
  meta >>= 4;
  *ny = *nz = 0;
  if (dims == 1) {
    if ((meta & 0xffffffffffffull) >= 0xffffffffull) return -1;
    *nx = (unsigned)(meta & 0xffffffffffffull) + 1u;
  } else if (dims == 2) {
    *nx = (unsigned)(meta & 0xffffff) + 1u;
    *ny = (unsigned)(meta >> 24 & 0xffffff) + 1u;
  } else if (dims == 3) {
    *nx = (unsigned)(meta & 0xffff) + 1u;
    *ny = (unsigned)(meta >> 16 & 0xffff) + 1u;
    *nz = (unsigned)(meta >> 32 & 0xffff) + 1u;
  } else {
    return -1;
  }
  *type = t;
  mode = r_get(&r, 12);
  if (mode < 4095) {
    if (mode >= 2048) return -1; /* fixed precision or fixed accuracy */
    *maxbits = (unsigned)mode + 1u;
  } else {
    unsigned minbits, maxprec, P = t == GZO_FLOAT || t == GZO_INT32 ? 32u : 64u;
    int minexp;
    bits = 32 + 52 + 64;
    if (bytes * 8 < (size_t)bits) return 0;
    mode += r_get(&r, 52) << 12;
    minbits = (unsigned)(mode >> 12 & 0x7fff) + 1u;
    *maxbits = (unsigned)(mode >> 27 & 0x7fff) + 1u;
    maxprec = (unsigned)(mode >> 42 & 0x7f) + 1u;
    minexp = (int)(mode >> 49 & 0x7fff) - 16495;
    if (minbits != *maxbits || maxprec < P || minexp != GZO_MIN_EXP) return -1;
  }
  return bits;
}

/* Decode a headed stream into `data` (capacity data_bytes); 1 on success */
int gzo_decompress_headed(const void* stream, size_t bytes, void* data, size_t data_bytes) {
  params p;
  rbits r;
  int type;
  unsigned nx, ny, nz, maxbits;
  uint64_t b, nblocks;
  double blk[64];
  long hb = gzo_read_header(stream, bytes, &type, &nx, &ny, &nz, &maxbits);
  if (hb <= 0) return 0;
  if (!setup_bits(&p, type, nx, ny, nz, maxbits)) return 0;
  if (maxbits < 1u + (unsigned)p.ebits) return 0;
  if (bytes < headed_bytes(&p, (unsigned)hb)) return 0;
  if (data_bytes < (size_t)p.nx * p.ny * p.nz * scalar_bytes(&p)) return 0;
  r.words = (const uint64_t*)stream;
  r.bit = (size_t)hb;
  nblocks = (uint64_t)p.bx * p.by * p.bz;
  for (b = 0; b < nblocks; b++) {
    unsigned bx = (unsigned)(b % p.bx);
    unsigned by = (unsigned)((b / p.bx) % p.by);
    unsigned bz = (unsigned)(b / ((uint64_t)p.bx * p.by));
    decode_block(&r, &p, blk);
    scatter(&p, data, bx, by, bz, blk);
  }
  return 1;
}

/* ---------------------------------------------------------- block access --- */

/* One listed block as a one-block field of its tile: extents from zfp's
   partial-block shape code (two bits per axis, x lowest, each 4 minus the
   extent; Z/array/zfpcodecd.h:5-75), values at strides 1, 4, 16. */
static int tile_params(params* p, int type, int dims, unsigned shape, unsigned maxbits) {
  unsigned cx = 4 - (shape & 3), cy = 4 - (shape >> 2 & 3), cz = 4 - (shape >> 4 & 3);
  if (!setup_bits(p, type, cx, dims >= 2 ? cy : 0, dims >= 3 ? cz : 0, maxbits)) return 0;
  p->sx = 1;
  p->sy = 4;
  p->sz = 16;
  return 1;
}

/* zfp_decode_block_* / zfp_decode_partial_block_strided_* at bit
   index[i] * maxbits (stream_rseek, Z/src/inline/bitstream.c:309-322), into
   tile i; a partial block writes only its valid values.  Indices past the
   stream are skipped.  Returns 1, or 0 on a bad argument. */
int gzo_decode_blocks(int type, int dims, unsigned maxbits, const void* stream, size_t bytes,
                      const unsigned long long* index, const unsigned char* shape, size_t count,
                      void* tiles) {
  size_t i, es = type == GZO_FLOAT || type == GZO_INT32 ? 4 : 8;
  size_t slots = bytes / 8 * 64 / (maxbits ? maxbits : 1);
  double blk[64];
  for (i = 0; i < count; i++) {
    params p;
    rbits r;
    if (!tile_params(&p, type, dims, shape ? shape[i] : 0u, maxbits)) return 0;
    if (index[i] >= slots) continue;
    r.words = (const uint64_t*)stream;
    r.bit = (size_t)(index[i] * maxbits);
    decode_block(&r, &p, blk);
    scatter(&p, (char*)tiles + i * ((size_t)1 << (2 * dims)) * es, 0, 0, 0, blk);
  }
  return 1;
}

/* zfp_encode_block_* / zfp_encode_partial_block_strided_* of tile i into
   the slot of index[i], keeping every other bit of the stream (zfp's own
   stream_wseek + stream_flush zero the rest of the slot's last word,
   Z/src/inline/bitstream.c:89-96; that agrees with this for word-aligned
   slots).  Indices past the stream are skipped. */
int gzo_encode_blocks(int type, int dims, unsigned maxbits, const void* tiles,
                      const unsigned long long* index, const unsigned char* shape, size_t count,
                      void* stream, size_t bytes) {
  size_t i, es = type == GZO_FLOAT || type == GZO_INT32 ? 4 : 8;
  size_t nwords = bytes / 8, slots = nwords * 64 / (maxbits ? maxbits : 1);
  uint64_t* words = (uint64_t*)stream;
  uint64_t* tmp = (uint64_t*)calloc(maxbits / 64 + 3, 8);
  double blk[64];
  if (!tmp) return 0;
  for (i = 0; i < count; i++) {
    params p;
    wbits w;
    uint64_t pos, end, k;
    unsigned off;
    if (!tile_params(&p, type, dims, shape ? shape[i] : 0u, maxbits)) {
      free(tmp);
      return 0;
    }
    if (index[i] >= slots) continue;
    pos = index[i] * maxbits;
    end = pos + maxbits;
    off = (unsigned)(pos % 64);
    /* code the block into tmp, at the slot's offset within its first word */
    memset(tmp, 0, (maxbits / 64 + 3) * 8);
    w_init(&w, tmp, 0);
    w_put(&w, 0, off);
    gather(&p, (const char*)tiles + i * ((size_t)1 << (2 * dims)) * es, 0, 0, 0, blk);
    encode_block(&w, &p, blk);
    w_flush(&w);
    /* replace the slot's bits, word by word */
    for (k = pos / 64; k * 64 < end; k++) {
      uint64_t lo = k * 64 < pos ? pos - k * 64 : 0;
      uint64_t hi = end - k * 64 < 64 ? end - k * 64 : 64;
      uint64_t mask = (hi >= 64 ? ~0ull : ((1ull << hi) - 1)) & ~((1ull << lo) - 1);
      words[k] = (words[k] & ~mask) | (tmp[k - pos / 64] & mask);
    }
  }
  free(tmp);
  return 1;
}

/* ------------------------------------------------ general stream params --- */

/* zfp_stream_set_precision (Z/src/zfp.c:432-441) and
   zfp_stream_set_accuracy (:443-458): blocks of up to ZFP_MAX_BITS = 4171
   bits and no minimum, coded down to a number of planes or to an absolute
   exponent */
void gzo_mode_precision(int type, unsigned precision, unsigned* minbits, unsigned* maxbits,
                        unsigned* maxprec, int* minexp) {
  unsigned P = type == GZO_FLOAT || type == GZO_INT32 ? 32 : 64;
  *minbits = 0;
  *maxbits = 4171;
  *maxprec = precision ? (precision < P ? precision : P) : P;
  *minexp = GZO_MIN_EXP;
}

void gzo_mode_accuracy(int type, double tolerance, unsigned* minbits, unsigned* maxbits,
                       unsigned* maxprec, int* minexp) {
  int emin = GZO_MIN_EXP;
  if (tolerance > 0) {
    frexp(tolerance, &emin); /* tolerance = x * 2^emin, 0.5 <= x < 1 */
    emin--;
  }
  *minbits = 0;
  *maxbits = 4171;
  *maxprec = type == GZO_FLOAT || type == GZO_INT32 ? 32 : 64;
  *minexp = emin;
}

static int setup_params(params* p, int type, unsigned nx, unsigned ny, unsigned nz,
                        unsigned minbits, unsigned maxbits, unsigned maxprec, int minexp) {
  /* zfp_stream_set_params' checks (Z/src/zfp.c:499-510), and room for the
     block header that every nonzero floating-point block writes */
  if (minbits > maxbits || maxprec == 0 || maxprec > 64) return 0;
  if (!setup_bits(p, type, nx, ny, nz, maxbits)) return 0;
  if (maxbits < (unsigned)p->ebits + 1) return 0;
  p->minbits = minbits;
  p->maxprec = maxprec;
  p->minexp = minexp;
  return 1;
}

/* the most bits a block can take: zfp_stream_maximum_size's per-block bound
   (Z/src/zfp.c:368-397) */
static unsigned block_bound(const params* p) {
  unsigned values = 1u << (2 * p->dims);
  unsigned prec = p->maxprec < (unsigned)p->P ? p->maxprec : (unsigned)p->P;
  unsigned b = 1 + (unsigned)p->ebits + values - 1 + values * prec;
  if (b > p->maxbits) b = p->maxbits;
  if (b < p->minbits) b = p->minbits;
  return b;
}

size_t gzo_bound_params(int type, unsigned nx, unsigned ny, unsigned nz, unsigned minbits,
                        unsigned maxbits, unsigned maxprec, int minexp) {
  params p;
  if (!setup_params(&p, type, nx, ny, nz, minbits, maxbits, maxprec, minexp)) return 0;
  return (size_t)(((uint64_t)p.bx * p.by * p.bz * block_bound(&p) + 63) / 64 * 8);
}

/* zfp_compress with these parameters: every block right after the
   previous one, in zfp's block order, then a flush to a whole word.  The
   start bit of every block goes to offsets[] when it is given.  Returns
   the stream size in bytes, 0 on a bad argument or a buffer smaller than
   the bound above. */
size_t gzo_compress_params(int type, unsigned nx, unsigned ny, unsigned nz, unsigned minbits,
                           unsigned maxbits, unsigned maxprec, int minexp, const void* data,
                           void* stream, size_t capacity, unsigned long long* offsets) {
  params p;
  wbits w;
  uint64_t b, nblocks, pos = 0;
  double blk[64];
  if (!setup_params(&p, type, nx, ny, nz, minbits, maxbits, maxprec, minexp)) return 0;
  if (capacity < gzo_bound_params(type, nx, ny, nz, minbits, maxbits, maxprec, minexp)) return 0;
  w_init(&w, (uint64_t*)stream, 0);
  nblocks = (uint64_t)p.bx * p.by * p.bz;
  for (b = 0; b < nblocks; b++) {
    unsigned bx = (unsigned)(b % p.bx);
    unsigned by = (unsigned)((b / p.bx) % p.by);
    unsigned bz = (unsigned)(b / ((uint64_t)p.bx * p.by));
    if (offsets) offsets[b] = pos;
    gather(&p, data, bx, by, bz, blk);
    encode_block(&w, &p, blk);
    pos = (uint64_t)w.pos * 64 + w.fill;
  }
  w_flush(&w);
  return (size_t)((pos + 63) / 64 * 8);
}

/* zfp_decompress with these parameters; offsets[] (optional) receives every
   block's start bit.  Returns 1, or 0 on a bad argument or a stream that
   ends before its last block. */
int gzo_decompress_params(int type, unsigned nx, unsigned ny, unsigned nz, unsigned minbits,
                          unsigned maxbits, unsigned maxprec, int minexp, const void* stream,
                          size_t bytes, void* data, unsigned long long* offsets) {
  params p;
  rbits r;
  uint64_t b, nblocks;
  double blk[64];
  uint64_t* padded;
  if (!setup_params(&p, type, nx, ny, nz, minbits, maxbits, maxprec, minexp)) return 0;
  /* read through a copy with zero words after the end, as many as one
     block can span (4171 bits) and the word a bit reader looks ahead */
  padded = (uint64_t*)calloc(bytes / 8 + 70, 8);
  if (!padded) return 0;
  memcpy(padded, stream, bytes / 8 * 8);
  r.words = padded;
  r.bit = 0;
  nblocks = (uint64_t)p.bx * p.by * p.bz;
  for (b = 0; b < nblocks && r.bit <= bytes / 8 * 64; b++) {
    unsigned bx = (unsigned)(b % p.bx);
    unsigned by = (unsigned)((b / p.bx) % p.by);
    unsigned bz = (unsigned)(b / ((uint64_t)p.bx * p.by));
    if (offsets) offsets[b] = r.bit;
    decode_block(&r, &p, blk);
    scatter(&p, data, bx, by, bz, blk);
  }
  free(padded);
  return b == nblocks && r.bit <= bytes / 8 * 64;
}


/* zfp_read_header's field and parameters for every mode (zfp_stream_set_mode,
   Z/src/zfp.c:461-498).  Returns the header bits, 0 for a bad magic, a short
   buffer or a field zfp 0.5.0 cannot hold. */
long gzo_read_header_params(const void* stream, size_t bytes, int* type, unsigned* nx,
                            unsigned* ny, unsigned* nz, unsigned* minbits, unsigned* maxbits,
                            unsigned* maxprec, int* minexp) {
  uint64_t words[3] = {0, 0, 0};
  rbits r;
  uint64_t meta, mode;
  int dims;
  long bits = 32 + 52 + 12;
  memcpy(words, stream, bytes < sizeof words ? bytes : sizeof words);
  if (bytes * 8 < (size_t)bits) return 0;
  r.words = words;
  r.bit = 0;
  if (r_get(&r, 8) != 'z' || r_get(&r, 8) != 'f' || r_get(&r, 8) != 'p' || r_get(&r, 8) != 0x05)
    return 0;
  meta = r_get(&r, 52);
  *type = (int)(meta & 3) + 1;
  dims = (int)(meta >> 2 & 3) + 1;
  meta >>= 4;
  *ny = *nz = 0;
  if (dims == 1) {
    if ((meta & 0xffffffffffffull) >= 0xffffffffull) return 0;
    *nx = (unsigned)(meta & 0xffffffffffffull) + 1u;
  } else if (dims == 2) {
    *nx = (unsigned)(meta & 0xffffff) + 1u;
    *ny = (unsigned)(meta >> 24 & 0xffffff) + 1u;
  } else if (dims == 3) {
    *nx = (unsigned)(meta & 0xffff) + 1u;
    *ny = (unsigned)(meta >> 16 & 0xffff) + 1u;
    *nz = (unsigned)(meta >> 32 & 0xffff) + 1u;
  } else {
    return 0;
  }
  mode = r_get(&r, 12);
  if (mode < 2048) {
    *minbits = *maxbits = (unsigned)mode + 1u;
    *maxprec = 64;
    *minexp = GZO_MIN_EXP;
  } else if (mode < 2176) {
    *minbits = 0;
    *maxbits = 4171;
    *maxprec = (unsigned)mode - 2047u;
    *minexp = GZO_MIN_EXP;
  } else if (mode < 4095) {
    *minbits = 0;
    *maxbits = 4171;
    *maxprec = 64;
    *minexp = (int)mode - 3251;
  } else {
    bits = 32 + 52 + 64;
    if (bytes * 8 < (size_t)bits) return 0;
    mode += r_get(&r, 52) << 12;
    *minbits = (unsigned)(mode >> 12 & 0x7fff) + 1u;
    *maxbits = (unsigned)(mode >> 27 & 0x7fff) + 1u;
    *maxprec = (unsigned)(mode >> 42 & 0x7f) + 1u;
    *minexp = (int)(mode >> 49 & 0x7fff) - 16495;
  }
  return bits;
}

/* The header of these parameters, then the blocks (zfp_write_header, then
   zfp_compress with them).  Returns the stream size in bytes, 0 on a bad
   argument, parameters no header records, or a short buffer. */
size_t gzo_compress_params_headed(int type, unsigned nx, unsigned ny, unsigned nz,
                                  unsigned minbits, unsigned maxbits, unsigned maxprec,
                                  int minexp, const void* data, void* stream, size_t capacity) {
  params p;
  uint64_t scratch[3];
  wbits w;
  unsigned hb;
  uint64_t b, nblocks, pos;
  double blk[64];
  if (!setup_params(&p, type, nx, ny, nz, minbits, maxbits, maxprec, minexp)) return 0;
  w_init(&w, scratch, 0);
  hb = header_put(&w, &p);
  if (!hb) return 0;
  if (capacity < gzo_bound_params(type, nx, ny, nz, minbits, maxbits, maxprec, minexp) + 24)
    return 0;
  w_init(&w, (uint64_t*)stream, 0);
  header_put(&w, &p);
  nblocks = (uint64_t)p.bx * p.by * p.bz;
  for (b = 0; b < nblocks; b++) {
    unsigned bx = (unsigned)(b % p.bx);
    unsigned by = (unsigned)((b / p.bx) % p.by);
    unsigned bz = (unsigned)(b / ((uint64_t)p.bx * p.by));
    gather(&p, data, bx, by, bz, blk);
    encode_block(&w, &p, blk);
  }
  pos = (uint64_t)w.pos * 64 + w.fill;
  w_flush(&w);
  return (size_t)((pos + 63) / 64 * 8);
}
