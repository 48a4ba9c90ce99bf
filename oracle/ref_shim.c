/*
 * ref_shim.c -- flat C entry points over the reference's own zfp 0.5.0 API.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together
 * with the unmodified zfp sources vendored by cuZFP
 * (src/thirdparty_builtin/zfp-0.5.0/src/*.c) into oracle/_ref/libzfpref.so.
 * The shim follows the fixed-rate call sequence of the zfp test driver
 * (Z/tests/testzfp.cpp:92-178): zfp_stream_set_rate(..., wra = 0),
 * zfp_stream_maximum_size, stream_open, zfp_compress / zfp_decompress.
 */
#include <stddef.h>
#include "zfp.h"

static zfp_field* make_field(int type, unsigned nx, unsigned ny, unsigned nz, void* data) {
  if (nz) return zfp_field_3d(data, (zfp_type)type, nx, ny, nz);
  if (ny) return zfp_field_2d(data, (zfp_type)type, nx, ny);
  return zfp_field_1d(data, (zfp_type)type, nx);
}

size_t zref_compress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                     const void* data, void* buffer, size_t capacity) {
  zfp_field* field = make_field(type, nx, ny, nz, (void*)data);
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_rate(zfp, rate, (zfp_type)type, zfp_field_dimensionality(field), 0);
  size_t bytes = 0;
  if (zfp_stream_maximum_size(zfp, field) <= capacity) {
    bitstream* s = stream_open(buffer, capacity);
    zfp_stream_set_bit_stream(zfp, s);
    zfp_stream_rewind(zfp);
    bytes = zfp_compress(zfp, field);
    stream_close(s);
  }
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return bytes;
}

size_t zref_maximum_size(int type, unsigned nx, unsigned ny, unsigned nz, double rate) {
  zfp_field* field = make_field(type, nx, ny, nz, NULL);
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_rate(zfp, rate, (zfp_type)type, zfp_field_dimensionality(field), 0);
  size_t m = zfp_stream_maximum_size(zfp, field);
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return m;
}

int zref_decompress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                    const void* buffer, size_t bytes, void* out) {
  zfp_field* field = make_field(type, nx, ny, nz, out);
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_rate(zfp, rate, (zfp_type)type, zfp_field_dimensionality(field), 0);
  bitstream* s = stream_open((void*)buffer, bytes);
  zfp_stream_set_bit_stream(zfp, s);
  zfp_stream_rewind(zfp);
  int ok = zfp_decompress(zfp, field);
  stream_close(s);
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return ok;
}

unsigned zref_set_rate_bits(int type, unsigned dims, double rate) {
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_rate(zfp, rate, (zfp_type)type, dims, 0);
  unsigned b = zfp->maxbits;
  zfp_stream_close(zfp);
  return b;
}

/* Integer arrays.  zfp 0.5.0's zfp_compress takes float and double fields
 * only (Z/src/zfp.c:618-624); its integer codec is the per-block API
 * zfp_encode_block_int32_<d> / zfp_encode_block_int64_<d> and the matching
 * decoders (Z/inc/zfp.h:452-521), with the rate set by zfp_stream_set_rate
 * as for floating point.  These drive that API over a contiguous array whose
 * sizes are multiples of 4, block by block in zfp_compress's order (x
 * fastest, then y, then z; Z/src/template/compress.c), and flush the stream
 * to a 64-bit word as zfp_compress does (Z/src/zfp.c:627-629). */
static void int_block_io(int type, int dims, unsigned nx, unsigned ny, unsigned nz,
                         unsigned bx, unsigned by, unsigned bz, void* data, void* blk,
                         int to_block) {
  const size_t es = type == zfp_type_int32 ? 4 : 8;
  unsigned x, y, z;
  unsigned dz = dims == 3 ? 4 : 1, dy = dims >= 2 ? 4 : 1;
  for (z = 0; z < dz; z++)
    for (y = 0; y < dy; y++)
      for (x = 0; x < 4; x++) {
        size_t idx = (4 * bx + x) + (size_t)nx * ((4 * by + y) + (size_t)ny * (4 * bz + z));
        char* a = (char*)data + idx * es;
        char* b = (char*)blk + (x + 4 * y + 16 * z) * es;
        size_t i;
        for (i = 0; i < es; i++) {
          if (to_block) b[i] = a[i];
          else a[i] = b[i];
        }
      }
}

static void int_block_codec(zfp_stream* zfp, int type, int dims, void* blk, int encode) {
  if (type == zfp_type_int32) {
    int32* b = (int32*)blk;
    if (encode) {
      if (dims == 1) zfp_encode_block_int32_1(zfp, b);
      else if (dims == 2) zfp_encode_block_int32_2(zfp, b);
      else zfp_encode_block_int32_3(zfp, b);
    } else {
      if (dims == 1) zfp_decode_block_int32_1(zfp, b);
      else if (dims == 2) zfp_decode_block_int32_2(zfp, b);
      else zfp_decode_block_int32_3(zfp, b);
    }
  } else {
    int64* b = (int64*)blk;
    if (encode) {
      if (dims == 1) zfp_encode_block_int64_1(zfp, b);
      else if (dims == 2) zfp_encode_block_int64_2(zfp, b);
      else zfp_encode_block_int64_3(zfp, b);
    } else {
      if (dims == 1) zfp_decode_block_int64_1(zfp, b);
      else if (dims == 2) zfp_decode_block_int64_2(zfp, b);
      else zfp_decode_block_int64_3(zfp, b);
    }
  }
}

static size_t int_array(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                        void* data, void* buffer, size_t capacity, int encode, int headed) {
  const int dims = nz ? 3 : ny ? 2 : 1;
  const unsigned NY = ny ? ny : 1, NZ = nz ? nz : 1;
  if ((type != zfp_type_int32 && type != zfp_type_int64) || nx % 4 ||
      (dims >= 2 && NY % 4) || (dims == 3 && NZ % 4))
    return 0;
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_rate(zfp, rate, (zfp_type)type, (uint)dims, 0);
  const size_t blocks = (size_t)(nx / 4) * (dims >= 2 ? NY / 4 : 1) * (dims == 3 ? NZ / 4 : 1);
  size_t hbits = 0;
  bitstream* s = stream_open(buffer, capacity);
  zfp_stream_set_bit_stream(zfp, s);
  zfp_stream_rewind(zfp);
  if (headed && capacity >= 3 * sizeof(uint64)) {
    /* the header of the field this array is, then its blocks */
    zfp_field* f = make_field(type, nx, ny, nz, data);
    hbits = encode ? zfp_write_header(zfp, f, ZFP_HEADER_FULL)
                   : zfp_read_header(zfp, f, ZFP_HEADER_FULL);
    zfp_field_free(f);
  }
  const size_t bytes = (hbits + blocks * zfp->maxbits + 63) / 64 * 8;
  if (bytes > capacity || (headed && !hbits)) {
    stream_close(s);
    zfp_stream_close(zfp);
    return 0;
  }
  int64 blk[64];
  unsigned bx, by, bz;
  for (bz = 0; bz < (dims == 3 ? NZ / 4 : 1); bz++)
    for (by = 0; by < (dims >= 2 ? NY / 4 : 1); by++)
      for (bx = 0; bx < nx / 4; bx++) {
        if (encode) int_block_io(type, dims, nx, NY, NZ, bx, by, bz, data, blk, 1);
        int_block_codec(zfp, type, dims, blk, encode);
        if (!encode) int_block_io(type, dims, nx, NY, NZ, bx, by, bz, data, blk, 0);
      }
  if (encode) stream_flush(s);
  const size_t used = encode ? stream_size(s) : bytes;
  stream_close(s);
  zfp_stream_close(zfp);
  return used;
}

size_t zref_compress_int(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                         const void* data, void* buffer, size_t capacity) {
  return int_array(type, nx, ny, nz, rate, (void*)data, buffer, capacity, 1, 0);
}

int zref_decompress_int(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                        const void* buffer, size_t bytes, void* out) {
  return int_array(type, nx, ny, nz, rate, out, (void*)buffer, bytes, 0, 0) != 0;
}

/* Strided fields through zfp_field_set_stride_<d> (Z/src/zfp.c:230-252):
   zfp_compress and zfp_decompress then take their strided paths. */
static zfp_field* make_strided(int type, unsigned nx, unsigned ny, unsigned nz, int sx, int sy,
                               int sz, void* data) {
  zfp_field* f = make_field(type, nx, ny, nz, data);
  if (nz) zfp_field_set_stride_3d(f, sx, sy, sz);
  else if (ny) zfp_field_set_stride_2d(f, sx, sy);
  else zfp_field_set_stride_1d(f, sx);
  return f;
}

size_t zref_compress_strided(int type, unsigned nx, unsigned ny, unsigned nz, int sx, int sy,
                             int sz, double rate, const void* data, void* buffer,
                             size_t capacity) {
  zfp_field* field = make_strided(type, nx, ny, nz, sx, sy, sz, (void*)data);
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_rate(zfp, rate, (zfp_type)type, zfp_field_dimensionality(field), 0);
  size_t bytes = 0;
  if (zfp_stream_maximum_size(zfp, field) <= capacity) {
    bitstream* s = stream_open(buffer, capacity);
    zfp_stream_set_bit_stream(zfp, s);
    zfp_stream_rewind(zfp);
    bytes = zfp_compress(zfp, field);
    stream_close(s);
  }
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return bytes;
}

int zref_decompress_strided(int type, unsigned nx, unsigned ny, unsigned nz, int sx, int sy,
                            int sz, double rate, const void* buffer, size_t bytes, void* out) {
  zfp_field* field = make_strided(type, nx, ny, nz, sx, sy, sz, out);
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_rate(zfp, rate, (zfp_type)type, zfp_field_dimensionality(field), 0);
  bitstream* s = stream_open((void*)buffer, bytes);
  zfp_stream_set_bit_stream(zfp, s);
  zfp_stream_rewind(zfp);
  int ok = zfp_decompress(zfp, field);
  stream_close(s);
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return ok;
}

/* Headed streams, the sequence of zfp's command-line tool with -h
   (Z/utils/zfp.c:378-427): zfp_write_header(ZFP_HEADER_FULL) and then
   zfp_compress on the same bit stream, so the first block follows the
   header bits directly; zfp_read_header then zfp_decompress to read one
   back.  Integer arrays take the per-block path above after the header. */
size_t zref_compress_headed(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                            const void* data, void* buffer, size_t capacity) {
  if (type == zfp_type_int32 || type == zfp_type_int64)
    return int_array(type, nx, ny, nz, rate, (void*)data, buffer, capacity, 1, 1);
  zfp_field* field = make_field(type, nx, ny, nz, (void*)data);
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_rate(zfp, rate, (zfp_type)type, zfp_field_dimensionality(field), 0);
  size_t bytes = 0;
  if (zfp_stream_maximum_size(zfp, field) <= capacity) {
    bitstream* s = stream_open(buffer, capacity);
    zfp_stream_set_bit_stream(zfp, s);
    zfp_stream_rewind(zfp);
    if (zfp_write_header(zfp, field, ZFP_HEADER_FULL)) bytes = zfp_compress(zfp, field);
    stream_close(s);
  }
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return bytes;
}

/* Parse a header with zfp_read_header; returns its bits (0 if zfp rejects
   it) and the field and mode it records. */
size_t zref_read_header(const void* buffer, size_t bytes, int* type, unsigned* nx, unsigned* ny,
                        unsigned* nz, unsigned* minbits, unsigned* maxbits, unsigned* maxprec,
                        int* minexp) {
  zfp_field* field = zfp_field_alloc();
  zfp_stream* zfp = zfp_stream_open(NULL);
  bitstream* s = stream_open((void*)buffer, bytes);
  zfp_stream_set_bit_stream(zfp, s);
  zfp_stream_rewind(zfp);
  size_t bits = zfp_read_header(zfp, field, ZFP_HEADER_FULL);
  *type = (int)field->type;
  *nx = field->nx;
  *ny = field->ny;
  *nz = field->nz;
  zfp_stream_params(zfp, minbits, maxbits, maxprec, minexp);
  stream_close(s);
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return bits;
}

/* zfp_read_header, then zfp_decompress into `out` (float and double) */
int zref_decompress_headed(const void* buffer, size_t bytes, void* out) {
  zfp_field* field = zfp_field_alloc();
  zfp_stream* zfp = zfp_stream_open(NULL);
  bitstream* s = stream_open((void*)buffer, bytes);
  zfp_stream_set_bit_stream(zfp, s);
  zfp_stream_rewind(zfp);
  int ok = 0;
  if (zfp_read_header(zfp, field, ZFP_HEADER_FULL)) {
    zfp_field_set_pointer(field, out);
    ok = zfp_decompress(zfp, field);
  }
  stream_close(s);
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return ok;
}

/* Integer arrays of the given sizes: zfp_read_header, then the blocks */
int zref_decompress_headed_int(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                               const void* buffer, size_t bytes, void* out) {
  return int_array(type, nx, ny, nz, rate, out, (void*)buffer, bytes, 0, 1) != 0;
}

/* Random access through the per-block API (Z/inc/zfp.h:452-521), the way
   zfp's compressed arrays fetch and write back blocks
   (Z/array/zfparray3.h:225-255): stream_rseek / stream_wseek to
   index * maxbits, one zfp_{en,de}code_{,partial_}block_* call, and after
   an encode stream_flush.  The stream parameters are those
   zfp_stream_set_rate leaves (zfp_stream_set_params, Z/src/zfp.c:500-511).
   zfp 0.5.0 has no partial-block calls for integer blocks: those return 0. */
static void float_block(zfp_stream* zfp, int dims, float* t, unsigned shape, int encode) {
  uint nx = 4 - (shape & 3u), ny = 4 - (shape >> 2 & 3u), nz = 4 - (shape >> 4 & 3u);
  if (encode && !shape) {
    if (dims == 1) zfp_encode_block_float_1(zfp, t);
    else if (dims == 2) zfp_encode_block_float_2(zfp, t);
    else zfp_encode_block_float_3(zfp, t);
  } else if (encode) {
    if (dims == 1) zfp_encode_partial_block_strided_float_1(zfp, t, nx, 1);
    else if (dims == 2) zfp_encode_partial_block_strided_float_2(zfp, t, nx, ny, 1, 4);
    else zfp_encode_partial_block_strided_float_3(zfp, t, nx, ny, nz, 1, 4, 16);
  } else if (!shape) {
    if (dims == 1) zfp_decode_block_float_1(zfp, t);
    else if (dims == 2) zfp_decode_block_float_2(zfp, t);
    else zfp_decode_block_float_3(zfp, t);
  } else {
    if (dims == 1) zfp_decode_partial_block_strided_float_1(zfp, t, nx, 1);
    else if (dims == 2) zfp_decode_partial_block_strided_float_2(zfp, t, nx, ny, 1, 4);
    else zfp_decode_partial_block_strided_float_3(zfp, t, nx, ny, nz, 1, 4, 16);
  }
}

static void double_block(zfp_stream* zfp, int dims, double* t, unsigned shape, int encode) {
  uint nx = 4 - (shape & 3u), ny = 4 - (shape >> 2 & 3u), nz = 4 - (shape >> 4 & 3u);
  if (encode && !shape) {
    if (dims == 1) zfp_encode_block_double_1(zfp, t);
    else if (dims == 2) zfp_encode_block_double_2(zfp, t);
    else zfp_encode_block_double_3(zfp, t);
  } else if (encode) {
    if (dims == 1) zfp_encode_partial_block_strided_double_1(zfp, t, nx, 1);
    else if (dims == 2) zfp_encode_partial_block_strided_double_2(zfp, t, nx, ny, 1, 4);
    else zfp_encode_partial_block_strided_double_3(zfp, t, nx, ny, nz, 1, 4, 16);
  } else if (!shape) {
    if (dims == 1) zfp_decode_block_double_1(zfp, t);
    else if (dims == 2) zfp_decode_block_double_2(zfp, t);
    else zfp_decode_block_double_3(zfp, t);
  } else {
    if (dims == 1) zfp_decode_partial_block_strided_double_1(zfp, t, nx, 1);
    else if (dims == 2) zfp_decode_partial_block_strided_double_2(zfp, t, nx, ny, 1, 4);
    else zfp_decode_partial_block_strided_double_3(zfp, t, nx, ny, nz, 1, 4, 16);
  }
}

static int block_io(zfp_stream* zfp, int type, int dims, void* tile, unsigned shape, int encode) {
  if (type == zfp_type_float) float_block(zfp, dims, (float*)tile, shape, encode);
  else if (type == zfp_type_double) double_block(zfp, dims, (double*)tile, shape, encode);
  else if (shape) return 0;
  else int_block_codec(zfp, type, dims, tile, encode);
  return 1;
}

static int blocks(int type, int dims, unsigned maxbits, void* tiles,
                  const unsigned long long* index, const unsigned char* shape, size_t count,
                  void* buffer, size_t bytes, int encode) {
  const size_t es = type == zfp_type_float || type == zfp_type_int32 ? 4 : 8;
  const uint prec = es == 4 ? 32 : 64;
  zfp_stream* zfp = zfp_stream_open(NULL);
  bitstream* s = stream_open(buffer, bytes);
  size_t i;
  int ok = zfp_stream_set_params(zfp, maxbits, maxbits, prec, ZFP_MIN_EXP);
  zfp_stream_set_bit_stream(zfp, s);
  for (i = 0; ok && i < count; i++) {
    void* tile = (char*)tiles + i * ((size_t)1 << (2 * dims)) * es;
    if (encode) stream_wseek(s, (size_t)(index[i] * maxbits));
    else stream_rseek(s, (size_t)(index[i] * maxbits));
    ok = block_io(zfp, type, dims, tile, shape ? shape[i] : 0u, encode);
    if (encode) stream_flush(s);
  }
  stream_close(s);
  zfp_stream_close(zfp);
  return ok;
}

int zref_encode_blocks(int type, int dims, unsigned maxbits, const void* tiles,
                       const unsigned long long* index, const unsigned char* shape, size_t count,
                       void* buffer, size_t bytes) {
  return blocks(type, dims, maxbits, (void*)tiles, index, shape, count, buffer, bytes, 1);
}

int zref_decode_blocks(int type, int dims, unsigned maxbits, const void* buffer, size_t bytes,
                       const unsigned long long* index, const unsigned char* shape, size_t count,
                       void* tiles) {
  return blocks(type, dims, maxbits, tiles, index, shape, count, (void*)buffer, bytes, 0);
}

/* zfp's general parameters (zfp_stream_set_params, Z/src/zfp.c:499-510;
   fixed precision and fixed accuracy are two settings of them,
   zfp_stream_set_precision / _accuracy, :432-458): zfp_compress and
   zfp_decompress for float and double fields; integer arrays (whole blocks
   only) through the per-block API in zfp's block order.  Blocks follow one
   another at their own lengths. */
static size_t params_array(int type, unsigned nx, unsigned ny, unsigned nz, unsigned minbits,
                           unsigned maxbits, unsigned maxprec, int minexp, void* data,
                           void* buffer, size_t capacity, int encode) {
  const int dims = nz ? 3 : ny ? 2 : 1;
  const unsigned NY = ny ? ny : 1, NZ = nz ? nz : 1;
  zfp_field* field = make_field(type, nx, ny, nz, data);
  zfp_stream* zfp = zfp_stream_open(NULL);
  size_t result = 0;
  if (zfp_stream_set_params(zfp, minbits, maxbits, maxprec, minexp) &&
      (!encode || zfp_stream_maximum_size(zfp, field) <= capacity)) {
    bitstream* s = stream_open(buffer, capacity);
    zfp_stream_set_bit_stream(zfp, s);
    zfp_stream_rewind(zfp);
    if (type == zfp_type_float || type == zfp_type_double) {
      result = encode ? zfp_compress(zfp, field) : (size_t)zfp_decompress(zfp, field);
    } else if (!(nx % 4 || (dims >= 2 && NY % 4) || (dims == 3 && NZ % 4))) {
      int64 blk[64];
      unsigned bx, by, bz;
      for (bz = 0; bz < (dims == 3 ? NZ / 4 : 1); bz++)
        for (by = 0; by < (dims >= 2 ? NY / 4 : 1); by++)
          for (bx = 0; bx < nx / 4; bx++) {
            if (encode) int_block_io(type, dims, nx, NY, NZ, bx, by, bz, data, blk, 1);
            int_block_codec(zfp, type, dims, blk, encode);
            if (!encode) int_block_io(type, dims, nx, NY, NZ, bx, by, bz, data, blk, 0);
          }
      if (encode) stream_flush(s);
      result = encode ? stream_size(s) : 1;
    }
    stream_close(s);
  }
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return result;
}

size_t zref_compress_params(int type, unsigned nx, unsigned ny, unsigned nz, unsigned minbits,
                            unsigned maxbits, unsigned maxprec, int minexp, const void* data,
                            void* buffer, size_t capacity) {
  return params_array(type, nx, ny, nz, minbits, maxbits, maxprec, minexp, (void*)data, buffer,
                      capacity, 1);
}

int zref_decompress_params(int type, unsigned nx, unsigned ny, unsigned nz, unsigned minbits,
                           unsigned maxbits, unsigned maxprec, int minexp, const void* buffer,
                           size_t bytes, void* out) {
  return params_array(type, nx, ny, nz, minbits, maxbits, maxprec, minexp, out, (void*)buffer,
                      bytes, 0) != 0;
}

static void stream_params(const zfp_stream* zfp, unsigned* minbits, unsigned* maxbits,
                          unsigned* maxprec, int* minexp) {
  *minbits = zfp->minbits;
  *maxbits = zfp->maxbits;
  *maxprec = zfp->maxprec;
  *minexp = zfp->minexp;
}

void zref_set_precision(int type, unsigned precision, unsigned* minbits, unsigned* maxbits,
                        unsigned* maxprec, int* minexp) {
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_precision(zfp, precision, (zfp_type)type);
  stream_params(zfp, minbits, maxbits, maxprec, minexp);
  zfp_stream_close(zfp);
}

void zref_set_accuracy(int type, double tolerance, unsigned* minbits, unsigned* maxbits,
                       unsigned* maxprec, int* minexp) {
  zfp_stream* zfp = zfp_stream_open(NULL);
  zfp_stream_set_accuracy(zfp, tolerance, (zfp_type)type);
  stream_params(zfp, minbits, maxbits, maxprec, minexp);
  zfp_stream_close(zfp);
}

/* zfp_write_header(ZFP_HEADER_FULL) with these parameters, then
   zfp_compress on the same bit stream (float and double fields). */
size_t zref_compress_params_headed(int type, unsigned nx, unsigned ny, unsigned nz,
                                   unsigned minbits, unsigned maxbits, unsigned maxprec,
                                   int minexp, const void* data, void* buffer, size_t capacity) {
  zfp_field* field = make_field(type, nx, ny, nz, (void*)data);
  zfp_stream* zfp = zfp_stream_open(NULL);
  size_t bytes = 0;
  if (zfp_stream_set_params(zfp, minbits, maxbits, maxprec, minexp) &&
      zfp_stream_maximum_size(zfp, field) <= capacity) {
    bitstream* s = stream_open(buffer, capacity);
    zfp_stream_set_bit_stream(zfp, s);
    zfp_stream_rewind(zfp);
    if (zfp_write_header(zfp, field, ZFP_HEADER_FULL)) bytes = zfp_compress(zfp, field);
    stream_close(s);
  }
  zfp_stream_close(zfp);
  zfp_field_free(field);
  return bytes;
}
