// cuzfp_compat.cu -- cuZFP::compress / cuZFP::decompress (include/cuZFP.h)
// over the C ABI, for C++ callers written against cuZFP
// (src/cuZFP/cuZFP.cu:174-269).  The calls are synchronous, as in cuZFP:
// work is queued on the legacy default stream, which is then synchronised.
#include <cuda_runtime.h>

#include "cuZFP.h"

namespace cuZFP {
namespace {
thread_local int g_status = GZFP_OK;

// cuZFP codes every stream as fixed rate, whatever the zfp_stream holds;
// here the stream's four parameters are honoured: fixed rate through the
// fixed-rate path, other settings (fixed precision, fixed accuracy) through
// zfp's general mode.  Strided fields (which cuZFP codes as contiguous) are
// coded through their strides, as zfp does -- in fixed-rate mode.
int check(const zfp_stream* zfp, const zfp_field* f) {
  if (!zfp || !f) return GZFP_ERR_ARG;
  return GZFP_OK;
}

bool strided(const zfp_field* f) { return f->sx || f->sy || f->sz; }

gzfp_mode mode_of(const zfp_stream* zfp) {
  return gzfp_mode{zfp->minbits, zfp->maxbits, zfp->maxprec, zfp->minexp};
}

// minbits == maxbits: every block has its fixed slot
bool fixed_slots(const zfp_stream* zfp) { return zfp->minbits == zfp->maxbits; }

// the parameters of fixed-rate coding (zfp_stream_set_rate, or cuZFP's
// stream_set_rate): the only ones the strided path takes
bool fixed_rate(const zfp_stream* zfp, const zfp_field* f) {
  const bool ints = f->type == zfp_type_int32 || f->type == zfp_type_int64;
  return fixed_slots(zfp) && zfp->maxprec >= type_precision(f->type) &&
         (ints || zfp->minexp == ZFP_MIN_EXP);
}
}  // namespace

int last_status() { return g_status; }

size_t compress(zfp_stream* zfp, zfp_field* field) {
  g_status = check(zfp, field);
  if (g_status != GZFP_OK) return 0;
  size_t bytes = 0;
  const size_t cap = zfp_stream_maximum_size(zfp, field);
  const gzfp_mode m = mode_of(zfp);
  if (strided(field) && !fixed_rate(zfp, field))
    g_status = GZFP_ERR_UNSUPPORTED;  // strided fields take the fixed-rate path only
  else if (strided(field))
    g_status = gzfp_compress_strided((int)field->type, field->nx, field->ny, field->nz, field->sx,
                                     field->sy, field->sz, zfp->maxbits, field->data, zfp->stream,
                                     cap, &bytes, nullptr);
  else
    g_status = gzfp_compress_mode((int)field->type, field->nx, field->ny, field->nz, &m,
                                  field->data, zfp->stream, cap, &bytes, nullptr, nullptr);
  if (g_status == GZFP_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) g_status = GZFP_ERR_CUDA;
  return g_status == GZFP_OK ? bytes : 0;
}

void decompress(zfp_stream* zfp, zfp_field* field) {
  g_status = check(zfp, field);
  if (g_status != GZFP_OK) return;
  const gzfp_mode m = mode_of(zfp);
  // fixed slots: the exact stream size; otherwise the buffer is taken to be
  // zfp_stream_maximum_size bytes, as cuZFP's callers allocate it, and the
  // blocks are found by walking them
  const size_t bytes =
      fixed_slots(zfp)
          ? gzfp_stream_size((int)field->type, field->nx, field->ny, field->nz, zfp->maxbits)
          : zfp_stream_maximum_size(zfp, field);
  if (strided(field) && !fixed_rate(zfp, field))
    g_status = GZFP_ERR_UNSUPPORTED;
  else if (strided(field))
    g_status = gzfp_decompress_strided((int)field->type, field->nx, field->ny, field->nz,
                                       field->sx, field->sy, field->sz, zfp->maxbits, zfp->stream,
                                       bytes, field->data, nullptr);
  else
    g_status = gzfp_decompress_mode((int)field->type, field->nx, field->ny, field->nz, &m,
                                    zfp->stream, bytes, nullptr, field->data, nullptr);
  if (g_status == GZFP_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) g_status = GZFP_ERR_CUDA;
}

}  // namespace cuZFP
