// host_codec.cpp -- test-only host build of the per-thread kernel code.
//
// Compiles cuzfp_gb300/csrc/gzfp_array.cuh (the exact per-block code that the
// CUDA kernels run, one block per thread) for the CPU and runs it block by
// block, so the CPU test suite can compare the kernel logic with the oracle
// without a GPU.  It is never part of the product library.
#include <stddef.h>
#include <stdint.h>
#include <string.h>
#include <math.h>

#include "../../cuzfp_gb300/csrc/gzfp_array.cuh"

namespace {

struct HostWords {
  uint64_t* out;       // writer target (pre-zeroed)
  const uint64_t* in;  // reader source
  uint64_t n;          // words available
  void store(uint64_t i, uint64_t v) { out[i] = v; }
  void merge(uint64_t i, uint64_t v) { out[i] |= v; }
  uint64_t load(uint64_t i) const { return i < n ? in[i] : 0; }
};

bool geom(unsigned nx, unsigned ny, unsigned nz, gzfp::Geom& g, int& dims) {
  if (!nx || (nz && !ny)) return false;
  dims = nz ? 3 : ny ? 2 : 1;
  g = gzfp::make_geom_blocks(nx, ny ? ny : 1, nz ? nz : 1);
  g.vec = (nx % 4 == 0);  // memcpy rows on the host: only the index math matters
  return true;
}

// types: 1 int32, 2 int64, 3 float, 4 double (zfp_type)
unsigned maxbits_for(int type, int dims, double rate) {
  unsigned bits = (unsigned)floor((1 << (2 * dims)) * rate + 0.5);
  unsigned lo = type == 3 ? 9u : type == 4 ? 12u : 0u;
  return bits < lo ? lo : bits;
}

template <typename T>
void enc_t(int dims, const void* data, const gzfp::Geom& g, unsigned maxbits, uint64_t* out,
           uint64_t words);
template <typename T>
void dec_t(int dims, const uint64_t* in, uint64_t words, const gzfp::Geom& g, unsigned maxbits,
           void* data);

template <int D, typename T>
void enc(const void* data, const gzfp::Geom& g, unsigned maxbits, uint64_t* out, uint64_t words) {
  HostWords w{out, nullptr, words};
  gzfp::LocalPlanes ps;
  for (uint64_t b = 0; b < g.nblocks; b++)
    gzfp::encode_one<D, T>((const T*)data, g, b, maxbits, w, ps);
}

template <int D, typename T>
void dec(const uint64_t* in, uint64_t words, const gzfp::Geom& g, unsigned maxbits, void* data) {
  HostWords w{nullptr, in, words};
  gzfp::LocalPlanes ps;
  for (uint64_t b = 0; b < g.nblocks; b++)
    gzfp::decode_one<D, T>((T*)data, g, b, maxbits, w, ps);
}

template <typename T>
void enc_t(int dims, const void* data, const gzfp::Geom& g, unsigned maxbits, uint64_t* out,
           uint64_t words) {
  if (dims == 1) enc<1, T>(data, g, maxbits, out, words);
  if (dims == 2) enc<2, T>(data, g, maxbits, out, words);
  if (dims == 3) enc<3, T>(data, g, maxbits, out, words);
}

template <typename T>
void dec_t(int dims, const uint64_t* in, uint64_t words, const gzfp::Geom& g, unsigned maxbits,
           void* data) {
  if (dims == 1) dec<1, T>(in, words, g, maxbits, data);
  if (dims == 2) dec<2, T>(in, words, g, maxbits, data);
  if (dims == 3) dec<3, T>(in, words, g, maxbits, data);
}

}  // namespace

extern "C" size_t hc_compress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                              const void* data, uint64_t* out, size_t cap) {
  gzfp::Geom g;
  int dims;
  if (!geom(nx, ny, nz, g, dims) || type < 1 || type > 4) return 0;
  unsigned maxbits = maxbits_for(type, dims, rate);
  if (!maxbits) return 0;
  uint64_t words = (g.nblocks * maxbits + 63) / 64;
  if (cap < words * 8) return 0;
  memset(out, 0, words * 8);
  if (type == 1) enc_t<int32_t>(dims, data, g, maxbits, out, words);
  if (type == 2) enc_t<int64_t>(dims, data, g, maxbits, out, words);
  if (type == 3) enc_t<float>(dims, data, g, maxbits, out, words);
  if (type == 4) enc_t<double>(dims, data, g, maxbits, out, words);
  return words * 8;
}

extern "C" int hc_decompress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                             const uint64_t* in, size_t bytes, void* data) {
  gzfp::Geom g;
  int dims;
  if (!geom(nx, ny, nz, g, dims) || type < 1 || type > 4) return 0;
  unsigned maxbits = maxbits_for(type, dims, rate);
  if (!maxbits) return 0;
  uint64_t words = bytes / 8;
  if (type == 1) dec_t<int32_t>(dims, in, words, g, maxbits, data);
  if (type == 2) dec_t<int64_t>(dims, in, words, g, maxbits, data);
  if (type == 3) dec_t<float>(dims, in, words, g, maxbits, data);
  if (type == 4) dec_t<double>(dims, in, words, g, maxbits, data);
  return 1;
}

namespace {

template <int D, typename T>
uint64_t walk(const uint64_t* in, uint64_t words, uint64_t nblocks, const gzfp::General& mode,
              uint64_t* offsets) {
  HostWords w{nullptr, in, words};
  uint64_t pos = 0;
  for (uint64_t b = 0; b < nblocks; b++) {
    offsets[b] = pos;
    gzfp::BitReader<HostWords> r(w, pos);
    pos += gzfp::block_bits<D, T>(r, mode);
  }
  return pos;
}

template <typename T>
uint64_t walk_t(int dims, const uint64_t* in, uint64_t words, uint64_t nblocks,
                const gzfp::General& mode, uint64_t* offsets) {
  if (dims == 1) return walk<1, T>(in, words, nblocks, mode, offsets);
  if (dims == 2) return walk<2, T>(in, words, nblocks, mode, offsets);
  return walk<3, T>(in, words, nblocks, mode, offsets);
}

}  // namespace

// The start bit of every block of a general-mode stream (zfp's minbits,
// maxbits, maxprec, minexp) by the kernels' block-length parse
// (gzfp::block_bits), as the device index walks it; returns the bit after
// the last block, 0 on bad arguments.
extern "C" uint64_t hc_block_offsets(int type, unsigned nx, unsigned ny, unsigned nz,
                                     unsigned minbits, unsigned maxbits, unsigned maxprec,
                                     int minexp, const uint64_t* in, size_t bytes,
                                     uint64_t* offsets) {
  gzfp::Geom g;
  int dims;
  if (!geom(nx, ny, nz, g, dims) || type < 1 || type > 4) return 0;
  const gzfp::General mode{minbits, maxbits, maxprec, minexp};
  const uint64_t words = bytes / 8;
  if (type == 1) return walk_t<int32_t>(dims, in, words, g.nblocks, mode, offsets);
  if (type == 2) return walk_t<int64_t>(dims, in, words, g.nblocks, mode, offsets);
  if (type == 3) return walk_t<float>(dims, in, words, g.nblocks, mode, offsets);
  return walk_t<double>(dims, in, words, g.nblocks, mode, offsets);
}

namespace {

// General-mode coding block after block (the per-block code of the mode
// kernels, encode_block_mode / decode_block_mode): each block's bits follow
// the previous block's at once, as zfp writes them.
template <int D, typename T>
uint64_t enc_general(const void* data, const gzfp::Geom& g, const gzfp::General& mode,
                     uint64_t* out, uint64_t words) {
  typedef typename gzfp::FT<T>::UInt UInt;
  HostWords w{out, nullptr, words};
  gzfp::LocalPlanes ps;
  uint64_t pos = 0;
  for (uint64_t b = 0; b < g.nblocks; b++) {
    uint32_t ix, iy, iz;
    gzfp::block_coords(g, b, ix, iy, iz);
    UInt raw[1 << (2 * D)];
    gzfp::gather<D, T>((const T*)data, g, ix, iy, iz, raw);
    gzfp::BitWriter<HostWords> bw(w, pos, mode.maxbits);
    pos += gzfp::encode_block_mode<D, T>(raw, mode, bw, ps);
    bw.finish();
  }
  return pos;
}

template <int D, typename T>
uint64_t dec_general(const uint64_t* in, uint64_t words, const gzfp::Geom& g,
                     const gzfp::General& mode, void* data) {
  typedef typename gzfp::FT<T>::UInt UInt;
  HostWords w{nullptr, in, words};
  gzfp::LocalPlanes ps;
  uint64_t pos = 0;
  for (uint64_t b = 0; b < g.nblocks; b++) {
    uint32_t ix, iy, iz;
    gzfp::block_coords(g, b, ix, iy, iz);
    gzfp::BitReader<HostWords> r(w, pos);
    UInt raw[1 << (2 * D)];
    pos += gzfp::decode_block_mode<D, T>(r, mode, raw, ps);
    gzfp::scatter<D, T>((T*)data, g, ix, iy, iz, raw);
  }
  return pos;
}

template <typename T>
uint64_t general_t(bool decode, int dims, const void* data, const gzfp::Geom& g,
                   const gzfp::General& mode, uint64_t* words, uint64_t nwords) {
  if (decode) {
    if (dims == 1) return dec_general<1, T>(words, nwords, g, mode, (void*)data);
    if (dims == 2) return dec_general<2, T>(words, nwords, g, mode, (void*)data);
    return dec_general<3, T>(words, nwords, g, mode, (void*)data);
  }
  if (dims == 1) return enc_general<1, T>(data, g, mode, words, nwords);
  if (dims == 2) return enc_general<2, T>(data, g, mode, words, nwords);
  return enc_general<3, T>(data, g, mode, words, nwords);
}

uint64_t general(bool decode, int type, unsigned nx, unsigned ny, unsigned nz, unsigned minbits,
                 unsigned maxbits, unsigned maxprec, int minexp, const void* data,
                 uint64_t* words, size_t bytes) {
  gzfp::Geom g;
  int dims;
  if (!geom(nx, ny, nz, g, dims) || type < 1 || type > 4) return 0;
  const gzfp::General mode{minbits, maxbits, maxprec, minexp};
  if (!decode) memset(words, 0, bytes);
  const uint64_t n = bytes / 8;
  if (type == 1) return general_t<int32_t>(decode, dims, data, g, mode, words, n);
  if (type == 2) return general_t<int64_t>(decode, dims, data, g, mode, words, n);
  if (type == 3) return general_t<float>(decode, dims, data, g, mode, words, n);
  return general_t<double>(decode, dims, data, g, mode, words, n);
}

}  // namespace

// General-mode compression into a zeroed buffer of `bytes` (at least the
// stream's size); returns the stream's bits, 0 on bad arguments.
extern "C" uint64_t hc_compress_params(int type, unsigned nx, unsigned ny, unsigned nz,
                                       unsigned minbits, unsigned maxbits, unsigned maxprec,
                                       int minexp, const void* data, uint64_t* out,
                                       size_t bytes) {
  return general(false, type, nx, ny, nz, minbits, maxbits, maxprec, minexp, data, out, bytes);
}

// General-mode decompression; returns the bits read, 0 on bad arguments.
extern "C" uint64_t hc_decompress_params(int type, unsigned nx, unsigned ny, unsigned nz,
                                         unsigned minbits, unsigned maxbits, unsigned maxprec,
                                         int minexp, const uint64_t* in, size_t bytes,
                                         void* data) {
  return general(true, type, nx, ny, nz, minbits, maxbits, maxprec, minexp, data,
                 (uint64_t*)in, bytes);
}

namespace {

template <int D, typename T>
void enc_aligned(const void* data, const gzfp::Geom& g, unsigned maxbits, uint64_t* out,
                 uint64_t words) {
  HostWords w{out, nullptr, words};
  gzfp::LocalPlanes ps;
  for (uint64_t b = 0; b < g.nblocks; b++)
    gzfp::encode_one<D, T, true>((const T*)data, g, b, maxbits, w, ps);
}

template <typename T>
void aligned_t(int dims, const void* data, const gzfp::Geom& g, unsigned maxbits, uint64_t* out,
               uint64_t words) {
  if (dims == 1) enc_aligned<1, T>(data, g, maxbits, out, words);
  if (dims == 2) enc_aligned<2, T>(data, g, maxbits, out, words);
  if (dims == 3) enc_aligned<3, T>(data, g, maxbits, out, words);
}

}  // namespace

// hc_compress through the encoder's aligned writer (whole words stored, no
// shared words merged), as the GPU kernels use it for blocks of whole 64-bit
// words; 0 when the rate's blocks are not whole words.  The output is
// filled with ones first, so a word the writer skips shows.
extern "C" size_t hc_compress_aligned(int type, unsigned nx, unsigned ny, unsigned nz,
                                      double rate, const void* data, uint64_t* out,
                                      size_t cap) {
  gzfp::Geom g;
  int dims;
  if (!geom(nx, ny, nz, g, dims) || type < 1 || type > 4) return 0;
  const unsigned maxbits = maxbits_for(type, dims, rate);
  if (!maxbits || maxbits % 64) return 0;
  const uint64_t words = g.nblocks * maxbits / 64;
  if (cap < words * 8) return 0;
  memset(out, 0xff, words * 8);
  if (type == 1) aligned_t<int32_t>(dims, data, g, maxbits, out, words);
  if (type == 2) aligned_t<int64_t>(dims, data, g, maxbits, out, words);
  if (type == 3) aligned_t<float>(dims, data, g, maxbits, out, words);
  if (type == 4) aligned_t<double>(dims, data, g, maxbits, out, words);
  return words * 8;
}

namespace {

template <int D, typename T>
void strided(bool decode, void* data, const gzfp::Geom& g, unsigned maxbits, uint64_t* words,
             uint64_t nwords) {
  HostWords w{decode ? nullptr : words, decode ? words : nullptr, nwords};
  gzfp::LocalPlanes ps;
  for (uint64_t b = 0; b < g.nblocks; b++) {
    if (decode)
      gzfp::decode_one<D, T>((T*)data, g, b, maxbits, w, ps);
    else
      gzfp::encode_one<D, T>((const T*)data, g, b, maxbits, w, ps);
  }
}

template <typename T>
void strided_t(bool decode, int dims, void* data, const gzfp::Geom& g, unsigned maxbits,
               uint64_t* words, uint64_t nwords) {
  if (dims == 1) strided<1, T>(decode, data, g, maxbits, words, nwords);
  if (dims == 2) strided<2, T>(decode, data, g, maxbits, words, nwords);
  if (dims == 3) strided<3, T>(decode, data, g, maxbits, words, nwords);
}

// a strided field: `data` is the address of value (0, 0, 0), value (x, y, z)
// at data + x sx + y sy + z sz elements (signed strides, 0 = contiguous)
size_t strided_call(bool decode, int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                    long long sy, long long sz, double rate, void* data, uint64_t* words,
                    size_t bytes) {
  gzfp::Geom g;
  int dims;
  if (!geom(nx, ny, nz, g, dims) || type < 1 || type > 4) return 0;
  g.sx = sx ? sx : 1;
  g.sy = sy ? sy : (long long)nx;
  g.sz = sz ? sz : (long long)nx * (ny ? ny : 1);
  g.vec = 0;  // value by value: only the index arithmetic matters on the host
  const unsigned maxbits = maxbits_for(type, dims, rate);
  const uint64_t nwords = (g.nblocks * maxbits + 63) / 64;
  if (bytes < nwords * 8) return 0;
  if (!decode) memset(words, 0, nwords * 8);
  if (type == 1) strided_t<int32_t>(decode, dims, data, g, maxbits, words, nwords);
  if (type == 2) strided_t<int64_t>(decode, dims, data, g, maxbits, words, nwords);
  if (type == 3) strided_t<float>(decode, dims, data, g, maxbits, words, nwords);
  if (type == 4) strided_t<double>(decode, dims, data, g, maxbits, words, nwords);
  return nwords * 8;
}

}  // namespace

// hc_compress / hc_decompress of a strided field (zfp_field sx/sy/sz)
extern "C" size_t hc_compress_strided(int type, unsigned nx, unsigned ny, unsigned nz,
                                      long long sx, long long sy, long long sz, double rate,
                                      const void* data, uint64_t* out, size_t cap) {
  return strided_call(false, type, nx, ny, nz, sx, sy, sz, rate, (void*)data, out, cap);
}
extern "C" size_t hc_decompress_strided(int type, unsigned nx, unsigned ny, unsigned nz,
                                        long long sx, long long sy, long long sz, double rate,
                                        const uint64_t* in, size_t bytes, void* data) {
  return strided_call(true, type, nx, ny, nz, sx, sy, sz, rate, data, (uint64_t*)in, bytes);
}
