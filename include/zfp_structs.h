/*
 * zfp_structs.h -- cuZFP-compatible stream / field records and helpers for
 * the GB300 codec (libgzfp.so).
 *
 * Drop-in for src/cuZFP/zfp_structs.h: the same names, fields and helper
 * signatures in namespace cuZFP, so code written against cuZFP compiles
 * unchanged.  Rate semantics follow zfp 0.5.0 (zfp_stream_set_rate with
 * wra = 0, zfp-0.5.0/src/zfp.c:405-430): cuZFP's copy rounded 3D block sizes
 * up to a multiple of 64 bits (zfp_structs.h:64-69), which changes nothing
 * for integer rates; the codec accepts either block size.
 */
#ifndef GZFP_ZFP_STRUCTS_H
#define GZFP_ZFP_STRUCTS_H

#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdlib>

#include "gzfp.h"

#define ZFP_MAX_PREC 64         /* maximum precision supported */
#define ZFP_MIN_EXP -1074       /* minimum floating-point base-2 exponent */
#define ZFP_MAX_BITS 4171       /* maximum number of bits per block */
#define ZFP_MIN_BITS 0          /* minimum number of bits per block */
#define ZFP_HEADER_MAX_BITS 148 /* max number of header bits */

typedef unsigned long long Word;

namespace cuZFP {

typedef struct {
  unsigned int minbits;
  unsigned int maxbits;
  unsigned int maxprec;
  int minexp;
  Word* stream; /* host or device buffer of compressed words */
} zfp_stream;

typedef enum {
  zfp_type_none = 0,
  zfp_type_int32 = GZFP_TYPE_INT32,
  zfp_type_int64 = GZFP_TYPE_INT64,
  zfp_type_float = GZFP_TYPE_FLOAT,
  zfp_type_double = GZFP_TYPE_DOUBLE
} zfp_type;

typedef struct {
  zfp_type type;              /* scalar type */
  unsigned int nx, ny, nz;    /* sizes (zero for unused dimensions) */
  int sx, sy, sz;             /* strides in values (0: contiguous a[nz][ny][nx]) */
  void* data;                 /* host or device pointer to the array */
} zfp_field;

static inline unsigned int zfp_field_dimensionality(const zfp_field* field) {
  return field->nx ? field->ny ? field->nz ? 3 : 2 : 1 : 0;
}

/* fixed-rate mode: bits per block for `rate` bits per value; returns the
   rate actually used */
static inline double stream_set_rate(zfp_stream* zfp, double rate, zfp_type type,
                                     unsigned int dims) {
  unsigned int bits = gzfp_rate_to_maxbits((int)type, dims, rate);
  zfp->minbits = bits;
  zfp->maxbits = bits;
  zfp->maxprec = ZFP_MAX_PREC;
  zfp->minexp = ZFP_MIN_EXP;
  return (double)bits / (double)(1u << (2 * dims));
}

/* zfp's fixed-precision and fixed-accuracy settings (zfp 0.5.0,
   zfp_stream_set_precision / zfp_stream_set_accuracy, src/zfp.c:432-458);
   not in cuZFP, which is fixed-rate only.  Return the precision, or the
   tolerance actually used. */
static inline unsigned int zfp_stream_set_precision(zfp_stream* zfp, unsigned int precision,
                                                    zfp_type type) {
  gzfp_mode m;
  if (gzfp_mode_precision((int)type, precision, &m) != GZFP_OK) return 0;
  zfp->minbits = m.minbits;
  zfp->maxbits = m.maxbits;
  zfp->maxprec = m.maxprec;
  zfp->minexp = m.minexp;
  return m.maxprec;
}

static inline double zfp_stream_set_accuracy(zfp_stream* zfp, double tolerance, zfp_type type) {
  gzfp_mode m;
  if (gzfp_mode_accuracy((int)type, tolerance, &m) != GZFP_OK) return 0.0;
  zfp->minbits = m.minbits;
  zfp->maxbits = m.maxbits;
  zfp->maxprec = m.maxprec;
  zfp->minexp = m.minexp;
  return tolerance > 0 ? std::ldexp(1.0, m.minexp) : 0.0;
}

static inline zfp_field* zfp_field_alloc() {
  zfp_field* f = (zfp_field*)std::malloc(sizeof(zfp_field));
  if (f) {
    f->type = zfp_type_none;
    f->nx = f->ny = f->nz = 0;
    f->sx = f->sy = f->sz = 0;
    f->data = 0;
  }
  return f;
}

static inline zfp_field* zfp_field_1d(void* data, zfp_type type, unsigned int nx) {
  zfp_field* f = zfp_field_alloc();
  if (f) { f->type = type; f->nx = nx; f->data = data; }
  return f;
}

static inline zfp_field* zfp_field_2d(void* data, zfp_type type, unsigned int nx,
                                      unsigned int ny) {
  zfp_field* f = zfp_field_alloc();
  if (f) { f->type = type; f->nx = nx; f->ny = ny; f->data = data; }
  return f;
}

static inline zfp_field* zfp_field_3d(void* data, zfp_type type, unsigned int nx,
                                      unsigned int ny, unsigned int nz) {
  zfp_field* f = zfp_field_alloc();
  if (f) { f->type = type; f->nx = nx; f->ny = ny; f->nz = nz; f->data = data; }
  return f;
}

static inline void zfp_field_free(zfp_field* field) { std::free(field); }

static inline zfp_stream* zfp_stream_open(Word* stream) {
  zfp_stream* zfp = (zfp_stream*)std::malloc(sizeof(zfp_stream));
  if (zfp) {
    zfp->stream = stream;
    zfp->minbits = ZFP_MIN_BITS;
    zfp->maxbits = ZFP_MAX_BITS;
    zfp->maxprec = ZFP_MAX_PREC;
    zfp->minexp = ZFP_MIN_EXP;
  }
  return zfp;
}

static inline void zfp_stream_close(zfp_stream* zfp) { std::free(zfp); }

static inline unsigned int type_precision(zfp_type type) {
  switch (type) {
    case zfp_type_int32: return CHAR_BIT * (unsigned int)sizeof(int);
    case zfp_type_int64: return CHAR_BIT * (unsigned int)sizeof(long long int);
    case zfp_type_float: return CHAR_BIT * (unsigned int)sizeof(float);
    case zfp_type_double: return CHAR_BIT * (unsigned int)sizeof(double);
    default: return 0;
  }
}

template <typename T> static inline zfp_type get_zfp_type() { return zfp_type_none; }
template <> inline zfp_type get_zfp_type<int>() { return zfp_type_int32; }
template <> inline zfp_type get_zfp_type<long long int>() { return zfp_type_int64; }
template <> inline zfp_type get_zfp_type<float>() { return zfp_type_float; }
template <> inline zfp_type get_zfp_type<double>() { return zfp_type_double; }

static inline size_t zfp_type_size(zfp_type type) {
  switch (type) {
    case zfp_type_int32: return sizeof(int);
    case zfp_type_int64: return sizeof(long long int);
    case zfp_type_float: return sizeof(float);
    case zfp_type_double: return sizeof(double);
    default: return 0;
  }
}

/* worst-case stream bytes for `field` under the stream's settings
   (zfp_stream_maximum_size) */
static inline size_t zfp_stream_maximum_size(const zfp_stream* zfp, const zfp_field* field) {
  unsigned int dims = zfp_field_dimensionality(field);
  if (!dims) return 0;
  unsigned int values = 1u << (2 * dims);
  unsigned int prec = type_precision(field->type);
  unsigned int ebits = field->type == zfp_type_float ? 8u : field->type == zfp_type_double ? 11u : 0u;
  unsigned int maxbits = 1 + ebits + values - 1 + values * (zfp->maxprec < prec ? zfp->maxprec : prec);
  if (maxbits > zfp->maxbits) maxbits = zfp->maxbits;
  if (maxbits < zfp->minbits) maxbits = zfp->minbits;
  size_t mx = ((field->nx ? field->nx : 1) + 3) / 4;
  size_t my = ((field->ny ? field->ny : 1) + 3) / 4;
  size_t mz = ((field->nz ? field->nz : 1) + 3) / 4;
  size_t blocks = mx * my * mz;
  return ((ZFP_HEADER_MAX_BITS + blocks * maxbits + 63) & ~(size_t)63) / CHAR_BIT;
}

}  // namespace cuZFP

#endif /* GZFP_ZFP_STRUCTS_H */
