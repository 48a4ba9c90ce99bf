// gzfp_header_api.cu -- zfp 0.5.0's stream header (gzfp_write_header*,
// gzfp_read_header*, headed compression and decompression; include/gzfp.h).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "gzfp.h"
#include "gzfp_host.h"
#include "gzfp_launch.h"

using namespace gzfp_host;

// ------------------------------------------------------------------ headers
// zfp 0.5.0's full header (zfp_write_header / zfp_read_header with
// ZFP_HEADER_FULL, Z/src/zfp.c:661-719): a 32-bit magic, 52 bits of field
// metadata (zfp_field_metadata / zfp_field_set_metadata, :158-182 and
// :254-275) and the stream parameters in 12 or 64 bits (zfp_stream_mode /
// zfp_stream_set_mode, :305-345 and :461-498).
namespace {

constexpr unsigned kMagicBits = 32, kMetaBits = 52, kModeShortBits = 12, kModeLongBits = 64;
constexpr uint64_t kModeShortMax = (1u << kModeShortBits) - 2;  // ZFP_MODE_SHORT_MAX
constexpr int kMinExp = -1074;                                    // ZFP_MIN_EXP
constexpr unsigned kMaxBitsZfp = 4171;                            // ZFP_MAX_BITS
constexpr int kMinExpBias = 16495;  // minexp offset of the long mode form
constexpr unsigned kLongField = 0x8000;  // largest minbits / maxbits the long form records

// up to 192 bits, LSB first in 64-bit words (the stream's own layout)
struct HeaderWords {
  uint64_t w[3] = {0, 0, 0};
  unsigned n = 0;
  void put(uint64_t v, unsigned bits) {  // bits <= 64
    if (bits < 64) v &= (1ull << bits) - 1;
    const unsigned i = n >> 6, o = n & 63;
    w[i] |= v << o;
    if (o && o + bits > 64) w[i + 1] |= v >> (64 - o);
    n += bits;
  }
  uint64_t get(unsigned& pos, unsigned bits) const {  // bits <= 64
    const unsigned i = pos >> 6, o = pos & 63;
    uint64_t v = w[i] >> o;
    if (o && o + bits > 64) v |= w[i + 1] << (64 - o);
    pos += bits;
    return bits < 64 ? v & ((1ull << bits) - 1) : v;
  }
};

// Field sizes a header records: 48 bits of nx - 1 in 1D, 24 bits per axis
// in 2D, 16 bits per axis in 3D (zfp_field_metadata, Z/src/zfp.c:158-182).
bool header_sizes_fit(int dims, unsigned nx, unsigned ny, unsigned nz) {
  if (dims == 2) return nx <= (1u << 24) && ny <= (1u << 24);
  if (dims == 3) return nx <= (1u << 16) && ny <= (1u << 16) && nz <= (1u << 16);
  return true;
}

// zfp_stream_mode: the 12-bit forms for fixed rate (maxbits - 1), fixed
// precision (maxprec + 2047) and fixed accuracy (minexp + 3251), else the
// 64-bit form holding every parameter.
uint64_t mode_code(const gzfp_mode& m, unsigned& bits) {
  bits = kModeShortBits;
  if (m.minbits == m.maxbits && m.maxbits >= 1 && m.maxbits <= 2048 && m.maxprec >= 64 &&
      m.minexp <= kMinExp)
    return m.maxbits - 1;
  if (m.minbits == 0 && m.maxbits >= kMaxBitsZfp && m.maxprec >= 1 && m.maxprec <= 128 &&
      m.minexp <= kMinExp)
    return m.maxprec + 2047;
  if (m.minbits == 0 && m.maxbits >= kMaxBitsZfp && m.maxprec >= 64 && m.minexp >= kMinExp &&
      m.minexp <= 843)
    return (uint64_t)(m.minexp + 3251);
  bits = kModeLongBits;
  auto clamp1 = [](unsigned v, unsigned hi) { return (v < 1 ? 1 : v > hi ? hi : v) - 1; };
  const int e = m.minexp + kMinExpBias;
  uint64_t code = (uint64_t)(e < 0 ? 0 : e > 0x7fff ? 0x7fff : e);
  code = (code << 7) | clamp1(m.maxprec, 0x80);
  code = (code << 15) | clamp1(m.maxbits, kLongField);
  code = (code << 15) | clamp1(m.minbits, kLongField);
  return (code << 12) | 0xfff;
}

int build_header_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode& m,
                      HeaderWords& h) {
  gzfp::Geom g;
  int dims;
  int st = check_mode(type, nx, ny, nz, &m, g, dims);
  if (st) return st;
  if (!header_sizes_fit(dims, nx, ny, nz))
    return fail(GZFP_ERR_ARG, "field sizes beyond what a zfp header records");
  unsigned mbits;
  const uint64_t code = mode_code(m, mbits);
  // the long form clamps: refuse parameters it would record differently
  if (mbits == kModeLongBits &&
      (m.minbits > kLongField || m.maxbits > kLongField || m.minexp + kMinExpBias < 0 ||
       m.minexp + kMinExpBias > 0x7fff))
    return fail(GZFP_ERR_ARG, "parameters beyond what a zfp header records");
  h.put('z', 8);
  h.put('f', 8);
  h.put('p', 8);
  h.put(5, 8);  // ZFP_VERSION >> 4 for 0.5.0
  uint64_t meta = dims == 1   ? (uint64_t)(nx - 1)
                  : dims == 2 ? ((uint64_t)(ny - 1) << 24) | (nx - 1)
                              : ((((uint64_t)(nz - 1) << 16) | (ny - 1)) << 16) | (nx - 1);
  meta = (meta << 4) | ((uint64_t)(dims - 1) << 2) | (uint64_t)(type - 1);
  h.put(meta, kMetaBits);
  h.put(code, mbits);
  return GZFP_OK;
}

// Parse a header into the field and the stream parameters
// (zfp_stream_set_mode); checks that the parameters can code a stream.
int parse_header_mode(const HeaderWords& h, size_t avail_bits, int* type, unsigned* nx,
                      unsigned* ny, unsigned* nz, gzfp_mode* m, size_t* header_bits) {
  if (avail_bits < kMagicBits + kMetaBits + kModeShortBits)
    return fail(GZFP_ERR_ARG, "stream shorter than a zfp header");
  unsigned pos = 0;
  if (h.get(pos, 8) != 'z' || h.get(pos, 8) != 'f' || h.get(pos, 8) != 'p' || h.get(pos, 8) != 5)
    return fail(GZFP_ERR_ARG, "no zfp 0.5.0 header (magic mismatch)");
  uint64_t meta = h.get(pos, kMetaBits);
  const int t = (int)(meta & 3) + 1;
  const int dims = (int)((meta >> 2) & 3) + 1;
  meta >>= 4;
  unsigned x, y = 0, z = 0;
  if (dims == 1) {
    const uint64_t n = (meta & 0xffffffffffffull) + 1;
    if (n > 0xffffffffull) return fail(GZFP_ERR_UNSUPPORTED, "1D field of 2^32 values or more");
    x = (unsigned)n;
  } else if (dims == 2) {
    x = (unsigned)(meta & 0xffffff) + 1;
    y = (unsigned)((meta >> 24) & 0xffffff) + 1;
  } else if (dims == 3) {
    x = (unsigned)(meta & 0xffff) + 1;
    y = (unsigned)((meta >> 16) & 0xffff) + 1;
    z = (unsigned)((meta >> 32) & 0xffff) + 1;
  } else {
    return fail(GZFP_ERR_UNSUPPORTED, "4D field (not part of zfp 0.5.0)");
  }
  uint64_t code = h.get(pos, kModeShortBits);
  gzfp_mode md;
  if (code <= kModeShortMax) {
    if (code < 2048)
      md = gzfp_mode{(unsigned)code + 1, (unsigned)code + 1, 64, kMinExp};
    else if (code < 2176)
      md = gzfp_mode{0, kMaxBitsZfp, (unsigned)code - 2047, kMinExp};
    else
      md = gzfp_mode{0, kMaxBitsZfp, 64, (int)code - 3251};
  } else {
    if (avail_bits < kMagicBits + kMetaBits + kModeLongBits)
      return fail(GZFP_ERR_ARG, "stream shorter than a zfp header");
    code |= h.get(pos, kModeLongBits - kModeShortBits) << kModeShortBits;
    md.minbits = (unsigned)((code >> 12) & 0x7fff) + 1;
    md.maxbits = (unsigned)((code >> 27) & 0x7fff) + 1;
    md.maxprec = (unsigned)((code >> 42) & 0x7f) + 1;
    md.minexp = (int)((code >> 49) & 0x7fff) - kMinExpBias;
  }
  gzfp::Geom g;
  int d;
  if (check_mode(t, x, y, z, &md, g, d))
    return fail(GZFP_ERR_UNSUPPORTED, "header parameters this codec cannot decode");
  *type = t;
  *nx = x;
  *ny = y;
  *nz = z;
  *m = md;
  *header_bits = pos;
  return GZFP_OK;
}

// the header at the start of a host or device stream (for a device stream:
// a copy of its first words after the work queued on `s`)
int stream_header(const void* stream, size_t bytes, cudaStream_t s, HeaderWords& h) {
  const size_t hb = bytes < sizeof h.w ? bytes : sizeof h.w;
  if (is_device_pointer(stream)) {
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h.w, stream, hb, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_fail(e, "cudaMemcpyAsync(header D2H)");
  } else {
    memcpy(h.w, stream, hb);
  }
  return GZFP_OK;
}

}  // namespace

extern "C" {

int gzfp_write_header_mode(int type, unsigned nx, unsigned ny, unsigned nz,
                           const gzfp_mode* mode, void* header, size_t capacity,
                           size_t* header_bits) {
  clear_error();
  if (!mode || !header) return fail(GZFP_ERR_ARG, "null pointer");
  HeaderWords h;
  int st = build_header_mode(type, nx, ny, nz, *mode, h);
  if (st) return st;
  const size_t bytes = (h.n + 7) / 8;
  if (capacity < bytes) return fail(GZFP_ERR_CAPACITY, "header buffer too small");
  memcpy(header, h.w, bytes);
  if (header_bits) *header_bits = h.n;
  return GZFP_OK;
}

int gzfp_write_header(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                      void* header, size_t capacity, size_t* header_bits) {
  clear_error();
  // the parameters zfp_stream_set_rate leaves
  const gzfp_mode m{maxbits, maxbits, precision_bits(type), kMinExp};
  return gzfp_write_header_mode(type, nx, ny, nz, &m, header, capacity, header_bits);
}

int gzfp_read_header_mode(const void* header, size_t bytes, int* type, unsigned* nx,
                          unsigned* ny, unsigned* nz, gzfp_mode* mode, size_t* header_bits) {
  clear_error();
  if (!header || !type || !nx || !ny || !nz || !mode || !header_bits)
    return fail(GZFP_ERR_ARG, "null pointer");
  HeaderWords h;
  memcpy(h.w, header, bytes < sizeof h.w ? bytes : sizeof h.w);
  return parse_header_mode(h, bytes * 8, type, nx, ny, nz, mode, header_bits);
}

int gzfp_read_header(const void* header, size_t bytes, int* type, unsigned* nx, unsigned* ny,
                     unsigned* nz, unsigned* maxbits, size_t* header_bits) {
  gzfp_mode m;
  int st = gzfp_read_header_mode(header, bytes, type, nx, ny, nz, &m, header_bits);
  if (st) return st;
  if (!maxbits) return fail(GZFP_ERR_ARG, "null pointer");
  if (!fixed_rate_mode(*type, &m))
    return fail(GZFP_ERR_UNSUPPORTED, "stream in a mode other than fixed rate (see gzfp_read_header_mode)");
  *maxbits = m.maxbits;
  return GZFP_OK;
}

int gzfp_compress_headed(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                         const void* data, void* stream, size_t capacity, size_t* out_bytes,
                         void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  if (!make_geom(nx, ny, nz, g, dims)) return fail(GZFP_ERR_ARG, "bad dimensions");
  gzfp_mode m;
  int st = gzfp_mode_rate(type, (unsigned)dims, rate, &m);
  if (st) return st;
  return gzfp_compress_mode_headed(type, nx, ny, nz, &m, data, stream, capacity, out_bytes,
                                   nullptr, cuda_stream);
}

int gzfp_compress_mode_headed(int type, unsigned nx, unsigned ny, unsigned nz,
                              const gzfp_mode* mode, const void* data, void* stream,
                              size_t capacity, size_t* out_bytes, unsigned long long* offsets,
                              void* cuda_stream) {
  clear_error();
  if (!mode) return fail(GZFP_ERR_ARG, "null mode");
  HeaderWords h;
  int st = build_header_mode(type, nx, ny, nz, *mode, h);
  if (st) return st;
  return compress_mode_impl(type, nx, ny, nz, mode, data, stream, capacity, out_bytes, offsets,
                            cuda_stream, h.w, h.n);
}

int gzfp_decompress_headed(const void* stream, size_t bytes, void* data, size_t data_bytes,
                           void* cuda_stream) {
  clear_error();
  if (!stream || !data) return fail(GZFP_ERR_ARG, "null pointer");
  HeaderWords h;
  int st = stream_header(stream, bytes, (cudaStream_t)cuda_stream, h);
  if (st) return st;
  int type;
  unsigned nx, ny, nz;
  gzfp_mode m;
  size_t header_bits;
  if ((st = parse_header_mode(h, bytes * 8, &type, &nx, &ny, &nz, &m, &header_bits))) return st;
  const uint64_t values = (uint64_t)nx * (ny ? ny : 1) * (nz ? nz : 1);
  if (data_bytes < values * scalar_size(type))
    return fail(GZFP_ERR_CAPACITY, "output buffer smaller than the field in the header");
  return decompress_mode_impl(type, nx, ny, nz, &m, stream, bytes, nullptr, data, cuda_stream,
                              header_bits);
}

}  // extern "C"

