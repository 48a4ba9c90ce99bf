// gzfp_modes_api.cu -- zfp's general coding modes (fixed precision, fixed
// accuracy, any stream parameters) in the C ABI (include/gzfp.h): argument
// checks, the per-device scratch, staging of host buffers, and the launches
// of gzfp_modes_*.cu.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "gzfp.h"
#include "gzfp_host.h"
#include "gzfp_launch.h"

using namespace gzfp_host;

namespace gzfp_host {

// Device buffers of the general-mode calls on one device, grown on demand
// and kept for the life of the process.
struct ModeSpace {
  std::mutex mu;
  void* scratch = nullptr;  size_t scratch_cap = 0;   // one slot per block
  void* lengths = nullptr;  size_t lengths_cap = 0;
  void* offsets = nullptr;  size_t offsets_cap = 0;
  void* sums = nullptr;     size_t sums_cap = 0;      // scan partials + total; walk end
  void* field = nullptr;    size_t field_cap = 0;     // staged host field
  void* stream = nullptr;   size_t stream_cap = 0;    // staged host stream
  void* index = nullptr;    size_t index_cap = 0;     // parallel index: lists and per-segment state
  void* pieces = nullptr;   size_t pieces_cap = 0;    // parallel index: the true chain's pieces
};
ModeSpace g_mode[kMaxDevices];

int mode_space(ModeSpace*& ms) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (device < 0 || device >= kMaxDevices) return fail(GZFP_ERR_CUDA, "device index out of range");
  ms = &g_mode[device];
  return GZFP_OK;
}

unsigned precision_bits(int type) {
  return type == GZFP_TYPE_FLOAT || type == GZFP_TYPE_INT32 ? 32 : 64;
}

// zfp_stream_set_params' checks (zfp-0.5.0/src/zfp.c:499-510), plus room
// for the header of a floating-point block and this library's block limit
int check_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* m,
               gzfp::Geom& g, int& dims) {
  if (!m) return fail(GZFP_ERR_ARG, "null mode");
  if (!known_type(type)) return fail(GZFP_ERR_ARG, "unknown scalar type");
  if (!make_geom(nx, ny, nz, g, dims))
    return fail(GZFP_ERR_ARG, "bad dimensions (nx must be > 0; nz > 0 needs ny > 0; under 2^32 blocks)");
  if (m->minbits > m->maxbits || m->maxprec == 0 || m->maxprec > 64)
    return fail(GZFP_ERR_ARG, "bad mode (minbits > maxbits, or maxprec outside 1..64)");
  if (m->maxbits < (unsigned)ebits_of(type) + 1 || m->maxbits > kMaxBitsLimit)
    return fail(GZFP_ERR_ARG, "bits per block out of range");
  return GZFP_OK;
}

// parameters whose blocks are exactly the fixed-rate path's
bool fixed_rate_mode(int type, const gzfp_mode* m) {
  const bool ints = type == GZFP_TYPE_INT32 || type == GZFP_TYPE_INT64;
  return m->minbits == m->maxbits && m->maxprec >= precision_bits(type) &&
         (ints || m->minexp == -1074);
}

gzfp::General general_of(const gzfp_mode* m) {
  return gzfp::General{m->minbits, m->maxbits, m->maxprec, m->minexp};
}

uint32_t mode_block_bound(int type, int dims, const gzfp_mode* m) {
  return gzfp::block_bound_host(dims, (int)precision_bits(type), ebits_of(type), general_of(m));
}

cudaError_t encode_mode_launch(int type, int dims, const void* in, const gzfp::Geom& g,
                               const gzfp::General& mode, uint64_t* scratch, uint32_t slot_words,
                               uint32_t* lengths, cudaStream_t s) {
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return gzfp::launch_encode_mode<float>(dims, (const float*)in, g, mode, scratch, slot_words, lengths, s);
    case GZFP_TYPE_DOUBLE:
      return gzfp::launch_encode_mode<double>(dims, (const double*)in, g, mode, scratch, slot_words, lengths, s);
    case GZFP_TYPE_INT32:
      return gzfp::launch_encode_mode<int32_t>(dims, (const int32_t*)in, g, mode, scratch, slot_words, lengths, s);
    default:
      return gzfp::launch_encode_mode<int64_t>(dims, (const int64_t*)in, g, mode, scratch, slot_words, lengths, s);
  }
}

cudaError_t decode_mode_launch(int type, int dims, const uint64_t* in, uint64_t nwords,
                               const unsigned long long* offsets, const gzfp::Geom& g,
                               const gzfp::General& mode, void* out, cudaStream_t s) {
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return gzfp::launch_decode_mode<float>(dims, in, nwords, offsets, g, mode, (float*)out, s);
    case GZFP_TYPE_DOUBLE:
      return gzfp::launch_decode_mode<double>(dims, in, nwords, offsets, g, mode, (double*)out, s);
    case GZFP_TYPE_INT32:
      return gzfp::launch_decode_mode<int32_t>(dims, in, nwords, offsets, g, mode, (int32_t*)out, s);
    default:
      return gzfp::launch_decode_mode<int64_t>(dims, in, nwords, offsets, g, mode, (int64_t*)out, s);
  }
}

cudaError_t index_launch(int type, int dims, const uint64_t* in, uint64_t nwords, uint64_t nblocks,
                         const gzfp::General& mode, uint64_t first, unsigned long long* offsets,
                         unsigned long long* end, cudaStream_t s) {
  switch (type) {
    case GZFP_TYPE_FLOAT:
      return gzfp::launch_index_blocks<float>(dims, in, nwords, nblocks, mode, first, offsets, end, s);
    case GZFP_TYPE_DOUBLE:
      return gzfp::launch_index_blocks<double>(dims, in, nwords, nblocks, mode, first, offsets, end, s);
    case GZFP_TYPE_INT32:
      return gzfp::launch_index_blocks<int32_t>(dims, in, nwords, nblocks, mode, first, offsets, end, s);
    default:
      return gzfp::launch_index_blocks<int64_t>(dims, in, nwords, nblocks, mode, first, offsets, end, s);
  }
}

// The block starts of a device stream by the parallel index
// (gzfp_modes.cuh): walkers over segments of the stream, joined where their
// chains merge.  Returns false, with nothing written that counts, when a
// list overflows or a chain does not merge; the caller then walks serially.
bool parallel_index(ModeSpace& ms, int type, int dims, const uint64_t* words, uint64_t nwords,
                    uint64_t nblocks, const gzfp::General& mode, uint64_t first,
                    uint64_t& end_bit, cudaStream_t s, cudaError_t& err) {
  err = cudaSuccess;
  const uint64_t total = nwords * 64;
  if (nblocks < 4096 || first >= total) return false;  // short streams: the serial walk
  gzfp::IndexJob j{};
  j.in = words;
  j.nwords = nwords;
  j.mode = mode;
  j.first = first;
  j.nseg = (uint32_t)std::min<uint64_t>(4096, nblocks / 1024);
  j.seg_bits = (total - first + j.nseg - 1) / j.nseg;
  j.cap = (uint32_t)(4 * ((nblocks + j.nseg - 1) / j.nseg) + 256);
  j.ext_cap = 16384;
  const size_t nseg = j.nseg;
  const size_t bytes = (nseg * j.cap + 7 * nseg) * 8;
  if ((err = reserve(ms.index, ms.index_cap, bytes))) return false;
  j.lists = (unsigned long long*)ms.index;
  j.counts = j.lists + nseg * j.cap;
  j.exits = j.counts + nseg;
  j.info = j.exits + nseg;
  auto walk = [&](bool extend) {
    switch (type) {
      case GZFP_TYPE_FLOAT: return gzfp::launch_index_walk<float>(dims, j, extend, s);
      case GZFP_TYPE_DOUBLE: return gzfp::launch_index_walk<double>(dims, j, extend, s);
      case GZFP_TYPE_INT32: return gzfp::launch_index_walk<int32_t>(dims, j, extend, s);
      default: return gzfp::launch_index_walk<int64_t>(dims, j, extend, s);
    }
  };
  std::vector<unsigned long long> state(6 * nseg);  // counts, info (exits are not needed)
  if ((err = walk(false)) || (err = walk(true)) ||
      (err = cudaMemcpyAsync(state.data(), j.counts, nseg * 8, cudaMemcpyDeviceToHost, s)) ||
      (err = cudaMemcpyAsync(state.data() + 2 * nseg, j.info, 4 * nseg * 8,
                             cudaMemcpyDeviceToHost, s)) ||
      (err = cudaStreamSynchronize(s)))
    return false;
  const unsigned long long* counts = state.data();
  const unsigned long long* info = state.data() + 2 * nseg;
  // follow the true chain from segment 0 (whose walker starts at block 0)
  std::vector<gzfp::IndexPiece> pieces;
  if (!gzfp::index_pieces(nseg, j.cap, counts, info, nblocks, pieces)) return false;
  if ((err = reserve(ms.pieces, ms.pieces_cap, pieces.size() * sizeof(gzfp::IndexPiece))) ||
      (err = reserve(ms.offsets, ms.offsets_cap, (size_t)nblocks * 8)) ||
      (err = reserve(ms.sums, ms.sums_cap, 64)) ||
      (err = cudaMemcpyAsync(ms.pieces, pieces.data(), pieces.size() * sizeof(gzfp::IndexPiece),
                             cudaMemcpyHostToDevice, s)))
    return false;
  const gzfp::IndexPiece* dp = (const gzfp::IndexPiece*)ms.pieces;
  unsigned long long* off = (unsigned long long*)ms.offsets;
  unsigned long long* endp = (unsigned long long*)ms.sums;
  const uint32_t np = (uint32_t)pieces.size();
  switch (type) {
    case GZFP_TYPE_FLOAT: err = gzfp::launch_index_assemble<float>(dims, j, dp, np, off, nblocks, endp, s); break;
    case GZFP_TYPE_DOUBLE: err = gzfp::launch_index_assemble<double>(dims, j, dp, np, off, nblocks, endp, s); break;
    case GZFP_TYPE_INT32: err = gzfp::launch_index_assemble<int32_t>(dims, j, dp, np, off, nblocks, endp, s); break;
    default: err = gzfp::launch_index_assemble<int64_t>(dims, j, dp, np, off, nblocks, endp, s); break;
  }
  unsigned long long end = 0;
  if (err || (err = cudaMemcpyAsync(&end, endp, 8, cudaMemcpyDeviceToHost, s)) ||
      (err = cudaStreamSynchronize(s)))  // also keeps `pieces` alive for its copy
    return false;
  end_bit = end;
  return true;
}

// Walk the blocks of a device stream into ms.offsets; *end_bit = the bit
// after the last block: the parallel index, or one thread walking every
// block when that cannot join its pieces.  Synchronises `s`.
int walk_blocks(ModeSpace& ms, int type, int dims, const uint64_t* words, uint64_t nwords,
                const gzfp::Geom& g, const gzfp::General& mode, uint64_t first, uint64_t& end_bit,
                cudaStream_t s) {
  cudaError_t e;
  if (parallel_index(ms, type, dims, words, nwords, g.nblocks, mode, first, end_bit, s, e))
    return GZFP_OK;
  if (e) return cuda_fail(e, "parallel block index");
  if ((e = reserve(ms.offsets, ms.offsets_cap, (size_t)g.nblocks * 8)) ||
      (e = reserve(ms.sums, ms.sums_cap, 64)))
    return cuda_fail(e, "cudaMalloc(block offsets)");
  if ((e = index_launch(type, dims, words, nwords, g.nblocks, mode, first,
                        (unsigned long long*)ms.offsets, (unsigned long long*)ms.sums, s)))
    return cuda_fail(e, "block walk launch");
  unsigned long long end = 0;
  if ((e = cudaMemcpyAsync(&end, ms.sums, 8, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "block walk");
  end_bit = end;
  return GZFP_OK;
}

}  // namespace gzfp_host

extern "C" {

int gzfp_mode_rate(int type, unsigned dims, double rate, gzfp_mode* mode) {
  clear_error();
  if (!mode) return fail(GZFP_ERR_ARG, "null mode");
  const unsigned b = gzfp_rate_to_maxbits(type, dims, rate);
  if (!b) return fail(GZFP_ERR_ARG, "bad type, dimensionality or rate");
  *mode = gzfp_mode{b, b, precision_bits(type), -1074};
  return GZFP_OK;
}

int gzfp_mode_precision(int type, unsigned precision, gzfp_mode* mode) {
  clear_error();
  if (!mode) return fail(GZFP_ERR_ARG, "null mode");
  if (!known_type(type)) return fail(GZFP_ERR_ARG, "unknown scalar type");
  const unsigned P = precision_bits(type);
  *mode = gzfp_mode{0, 4171, precision ? (precision < P ? precision : P) : P, -1074};
  return GZFP_OK;
}

int gzfp_mode_accuracy(int type, double tolerance, gzfp_mode* mode) {
  clear_error();
  if (!mode) return fail(GZFP_ERR_ARG, "null mode");
  if (!known_type(type)) return fail(GZFP_ERR_ARG, "unknown scalar type");
  if (isnan(tolerance)) return fail(GZFP_ERR_ARG, "tolerance is NaN");
  int emin = -1074;
  if (tolerance > 0) {
    frexp(tolerance, &emin);  // tolerance = x * 2^emin with 0.5 <= x < 1
    emin--;
  }
  *mode = gzfp_mode{0, 4171, precision_bits(type), emin};
  return GZFP_OK;
}

size_t gzfp_mode_maximum_size(int type, unsigned nx, unsigned ny, unsigned nz,
                              const gzfp_mode* mode) {
  gzfp::Geom g;
  int dims;
  if (check_mode(type, nx, ny, nz, mode, g, dims)) return 0;
  return (size_t)((g.nblocks * mode_block_bound(type, dims, mode) + 63) / 64 * 8);
}

}  // extern "C"

namespace gzfp_host {

// A general-mode compression; with `header` (hbits bits in whole words)
// the stream starts with it and the blocks follow directly.
int compress_mode_impl(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                       const void* data, void* stream, size_t capacity, size_t* out_bytes,
                       unsigned long long* offsets, void* cuda_stream, const uint64_t* header,
                       unsigned hbits) {
  gzfp::Geom g;
  int dims;
  int st = check_mode(type, nx, ny, nz, mode, g, dims);
  if (st) return st;
  if (!data || !stream) return fail(GZFP_ERR_ARG, "null pointer");
  cudaStream_t s = (cudaStream_t)cuda_stream;
  cudaError_t e;
  if (fixed_rate_mode(type, mode)) {
    st = header ? strided_call(false, type, nx, ny, nz, 0, 0, 0, mode->maxbits, (void*)data,
                               (uint64_t*)stream, capacity, out_bytes, cuda_stream, hbits, header,
                               (hbits + 63) / 64)
                : gzfp_compress_bits(type, nx, ny, nz, mode->maxbits, data, stream, capacity,
                                     out_bytes, cuda_stream);
    if (st || !offsets) return st;
    if (is_device_pointer(offsets)) {
      if ((e = gzfp::launch_fixed_offsets(offsets, g.nblocks, hbits, mode->maxbits, s)))
        return cuda_fail(e, "offsets kernel launch");
    } else {
      for (uint64_t b = 0; b < g.nblocks; b++) offsets[b] = hbits + b * mode->maxbits;
    }
    return GZFP_OK;
  }
  if (out_bytes) *out_bytes = 0;
  if (g.nblocks == 0) return GZFP_OK;
  ModeSpace* msp;
  if ((st = mode_space(msp))) return st;
  ModeSpace& ms = *msp;
  std::lock_guard<std::mutex> lock(ms.mu);
  const size_t S = scalar_size(type);
  const gzfp::General gm = general_of(mode);
  const uint32_t slot_words = (mode_block_bound(type, dims, mode) + 63) / 64;
  const uint64_t m = gzfp::scan_sums_count(g.nblocks);
  const bool dev_data = is_device_pointer(data), dev_stream = is_device_pointer(stream);
  const bool dev_offsets = offsets && is_device_pointer(offsets);
  // one slot of slack after the last: a slot holds the most bits any block
  // can take, and the slack keeps even a longer block inside the buffer
  if ((e = reserve(ms.scratch, ms.scratch_cap, (size_t)((g.nblocks + 1) * slot_words * 8))) ||
      (e = reserve(ms.lengths, ms.lengths_cap, (size_t)g.nblocks * 4)) ||
      (e = reserve(ms.offsets, ms.offsets_cap, (size_t)g.nblocks * 8)) ||
      (e = reserve(ms.sums, ms.sums_cap, (size_t)(m + 1) * 8)))
    return cuda_fail(e, "cudaMalloc(general-mode scratch)");
  const void* din = data;
  const size_t field_bytes = (size_t)g.nx * g.ny * g.nz * S;
  if (!dev_data) {
    if ((e = reserve(ms.field, ms.field_cap, field_bytes)))
      return cuda_fail(e, "cudaMalloc(field staging)");
    if ((e = cudaMemcpyAsync(ms.field, data, field_bytes, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "cudaMemcpyAsync(field H2D)");
    din = ms.field;
  }
  gzfp::Geom gv = g;
  gv.vec = rows_vectorizable(din, nx, type);
  if ((e = encode_mode_launch(type, dims, din, gv, gm, (uint64_t*)ms.scratch, slot_words,
                              (uint32_t*)ms.lengths, s)))
    return cuda_fail(e, "encode kernel launch");
  if ((e = gzfp::launch_scan_lengths((const uint32_t*)ms.lengths, g.nblocks, hbits,
                                     (uint64_t*)ms.sums, (unsigned long long*)ms.offsets, s)))
    return cuda_fail(e, "scan kernel launch");
  unsigned long long total = 0;
  if ((e = cudaMemcpyAsync(&total, (uint64_t*)ms.sums + m, 8, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "encode");
  const size_t bytes = (size_t)((hbits + total + 63) / 64 * 8);
  if (out_bytes) *out_bytes = bytes;
  if (capacity < bytes) return fail(GZFP_ERR_CAPACITY, "stream buffer smaller than the compressed size");
  uint64_t* dstream = (uint64_t*)stream;
  if (!dev_stream) {
    if ((e = reserve(ms.stream, ms.stream_cap, bytes))) return cuda_fail(e, "cudaMalloc(stream staging)");
    dstream = (uint64_t*)ms.stream;
  }
  st = GZFP_OK;
  if ((e = cudaMemsetAsync(dstream, 0, bytes, s)) ||
      (header && (e = cudaMemcpyAsync(dstream, header, (hbits + 63) / 64 * 8,
                                      cudaMemcpyHostToDevice, s))) ||
      (e = gzfp::launch_place_blocks((const uint64_t*)ms.scratch, slot_words,
                                     (const uint32_t*)ms.lengths,
                                     (const unsigned long long*)ms.offsets, g.nblocks, dstream, s)))
    st = cuda_fail(e, "block placement");
  if (!st && !dev_stream && (e = cudaMemcpyAsync(stream, dstream, bytes, cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(stream D2H)");
  if (!st && offsets &&
      (e = cudaMemcpyAsync(offsets, ms.offsets, (size_t)g.nblocks * 8,
                           dev_offsets ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(offsets)");
  const cudaError_t es = cudaStreamSynchronize(s);  // the scratch is reused by the next call
  if (!st && es) st = cuda_fail(es, "cudaStreamSynchronize");
  return st;
}

// A general-mode decompression whose first block starts at bit `first`.
int decompress_mode_impl(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                         const void* stream, size_t bytes, const unsigned long long* offsets,
                         void* data, void* cuda_stream, uint64_t first) {
  gzfp::Geom g;
  int dims;
  int st = check_mode(type, nx, ny, nz, mode, g, dims);
  if (st) return st;
  if (!stream || !data) return fail(GZFP_ERR_ARG, "null pointer");
  if (fixed_rate_mode(type, mode))
    return first ? strided_call(true, type, nx, ny, nz, 0, 0, 0, mode->maxbits, data,
                                (uint64_t*)stream, bytes, nullptr, cuda_stream, first)
                 : gzfp_decompress_bits(type, nx, ny, nz, mode->maxbits, stream, bytes, data,
                                        cuda_stream);
  if (g.nblocks == 0) return GZFP_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  ModeSpace* msp;
  if ((st = mode_space(msp))) return st;
  ModeSpace& ms = *msp;
  std::lock_guard<std::mutex> lock(ms.mu);
  cudaError_t e;
  const uint64_t nwords = bytes / 8;
  const gzfp::General gm = general_of(mode);
  const size_t field_bytes = (size_t)g.nx * g.ny * g.nz * scalar_size(type);
  const bool dev_stream = is_device_pointer(stream), dev_data = is_device_pointer(data);
  bool staged = !dev_stream || !dev_data;
  const uint64_t* dw = (const uint64_t*)stream;
  if (!dev_stream) {
    if ((e = reserve(ms.stream, ms.stream_cap, nwords ? nwords * 8 : 8)) ||
        (e = cudaMemcpyAsync(ms.stream, stream, nwords * 8, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "stream staging");
    dw = (const uint64_t*)ms.stream;
  }
  const unsigned long long* doff = offsets;
  if (!offsets) {
    uint64_t end = 0;
    if ((st = walk_blocks(ms, type, dims, dw, nwords, g, gm, first, end, s))) return st;
    if (end > nwords * 64) return fail(GZFP_ERR_ARG, "stream shorter than its blocks");
    doff = (const unsigned long long*)ms.offsets;
  } else if (!is_device_pointer(offsets)) {
    if ((e = reserve(ms.offsets, ms.offsets_cap, (size_t)g.nblocks * 8)) ||
        (e = cudaMemcpyAsync(ms.offsets, offsets, (size_t)g.nblocks * 8, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "offsets staging");
    doff = (const unsigned long long*)ms.offsets;
    staged = true;
  }
  void* dout = data;
  if (!dev_data) {
    if ((e = reserve(ms.field, ms.field_cap, field_bytes))) return cuda_fail(e, "cudaMalloc(field staging)");
    dout = ms.field;
  }
  gzfp::Geom gv = g;
  gv.vec = rows_vectorizable(dout, nx, type);
  st = GZFP_OK;
  if ((e = decode_mode_launch(type, dims, dw, nwords, doff, gv, gm, dout, s)))
    st = cuda_fail(e, "decode kernel launch");
  if (!st && !dev_data && (e = cudaMemcpyAsync(data, dout, field_bytes, cudaMemcpyDeviceToHost, s)))
    st = cuda_fail(e, "cudaMemcpyAsync(field D2H)");
  if (staged || !offsets) {  // staging buffers and the walk's offsets are reused by the next call
    const cudaError_t es = cudaStreamSynchronize(s);
    if (!st && es) st = cuda_fail(es, "cudaStreamSynchronize");
  }
  return st;
}

}  // namespace gzfp_host

extern "C" {

int gzfp_compress_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                       const void* data, void* stream, size_t capacity, size_t* out_bytes,
                       unsigned long long* offsets, void* cuda_stream) {
  clear_error();
  return compress_mode_impl(type, nx, ny, nz, mode, data, stream, capacity, out_bytes, offsets,
                            cuda_stream, nullptr, 0);
}

int gzfp_decompress_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                         const void* stream, size_t bytes, const unsigned long long* offsets,
                         void* data, void* cuda_stream) {
  clear_error();
  return decompress_mode_impl(type, nx, ny, nz, mode, stream, bytes, offsets, data, cuda_stream,
                              0);
}

int gzfp_index_blocks(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                      const void* stream, size_t bytes, unsigned long long* offsets,
                      void* cuda_stream) {
  clear_error();
  gzfp::Geom g;
  int dims;
  int st = check_mode(type, nx, ny, nz, mode, g, dims);
  if (st) return st;
  if (!stream || !offsets) return fail(GZFP_ERR_ARG, "null pointer");
  if (g.nblocks == 0) return GZFP_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  ModeSpace* msp;
  if ((st = mode_space(msp))) return st;
  ModeSpace& ms = *msp;
  std::lock_guard<std::mutex> lock(ms.mu);
  cudaError_t e;
  const uint64_t nwords = bytes / 8;
  const uint64_t* dw = (const uint64_t*)stream;
  if (!is_device_pointer(stream)) {
    if ((e = reserve(ms.stream, ms.stream_cap, nwords ? nwords * 8 : 8)) ||
        (e = cudaMemcpyAsync(ms.stream, stream, nwords * 8, cudaMemcpyHostToDevice, s)))
      return cuda_fail(e, "stream staging");
    dw = (const uint64_t*)ms.stream;
  }
  uint64_t end = 0;
  if ((st = walk_blocks(ms, type, dims, dw, nwords, g, general_of(mode), 0, end, s))) return st;
  if (end > nwords * 64) return fail(GZFP_ERR_ARG, "stream shorter than its blocks");
  if ((e = cudaMemcpyAsync(offsets, ms.offsets, (size_t)g.nblocks * 8,
                           is_device_pointer(offsets) ? cudaMemcpyDeviceToDevice
                                                      : cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "cudaMemcpyAsync(offsets)");
  return GZFP_OK;
}

}  // extern "C"

