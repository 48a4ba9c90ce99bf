// cuzfp_compat.cu -- cuZFP::compress / cuZFP::decompress (include/cuZFP.h)
// over the C ABI, for C++ callers written against cuZFP
// (src/cuZFP/cuZFP.cu:174-269).  The calls are synchronous, as in cuZFP:
// work is queued on the legacy default stream, which is then synchronised.
#include <cuda_runtime.h>

#include "cuZFP.h"

namespace cuZFP {
namespace {
thread_local int g_status = GZFP_OK;

// cuZFP honours only fixed-rate streams; other modes are reported instead
// of being silently ignored.  Strided fields (which cuZFP codes as
// contiguous) are coded through their strides, as zfp does.
int check(const zfp_stream* zfp, const zfp_field* f) {
  if (!zfp || !f) return GZFP_ERR_ARG;
  if (zfp->minbits != zfp->maxbits) return GZFP_ERR_UNSUPPORTED;
  return GZFP_OK;
}

bool strided(const zfp_field* f) { return f->sx || f->sy || f->sz; }
}  // namespace

int last_status() { return g_status; }

size_t compress(zfp_stream* zfp, zfp_field* field) {
  g_status = check(zfp, field);
  if (g_status != GZFP_OK) return 0;
  size_t bytes = 0;
  const size_t cap = zfp_stream_maximum_size(zfp, field);
  g_status = strided(field)
                 ? gzfp_compress_strided((int)field->type, field->nx, field->ny, field->nz,
                                         field->sx, field->sy, field->sz, zfp->maxbits, field->data,
                                         zfp->stream, cap, &bytes, nullptr)
                 : gzfp_compress_bits((int)field->type, field->nx, field->ny, field->nz,
                                      zfp->maxbits, field->data, zfp->stream, cap, &bytes, nullptr);
  if (g_status == GZFP_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) g_status = GZFP_ERR_CUDA;
  return g_status == GZFP_OK ? bytes : 0;
}

void decompress(zfp_stream* zfp, zfp_field* field) {
  g_status = check(zfp, field);
  if (g_status != GZFP_OK) return;
  size_t bytes = gzfp_stream_size((int)field->type, field->nx, field->ny, field->nz, zfp->maxbits);
  g_status = strided(field)
                 ? gzfp_decompress_strided((int)field->type, field->nx, field->ny, field->nz,
                                           field->sx, field->sy, field->sz, zfp->maxbits,
                                           zfp->stream, bytes, field->data, nullptr)
                 : gzfp_decompress_bits((int)field->type, field->nx, field->ny, field->nz,
                                        zfp->maxbits, zfp->stream, bytes, field->data, nullptr);
  if (g_status == GZFP_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) g_status = GZFP_ERR_CUDA;
}

}  // namespace cuZFP
