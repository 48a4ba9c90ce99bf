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
