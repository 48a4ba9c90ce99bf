/*
 * cuZFP.h -- drop-in C++ entry points of the GB300 codec (libgzfp.so).
 *
 * Same declarations as cuZFP's src/cuZFP/cuZFP.h:9-10.  `compress` returns
 * the stream size in bytes and 0 on failure; `decompress` returns nothing,
 * as in cuZFP.  Both record failures in cuZFP::last_status() (a gzfp status
 * code, include/gzfp.h) and gzfp_last_error(), where cuZFP only printed them
 * (src/cuZFP/ErrorCheck.cu:11-19).  Buffers may be host or device memory;
 * the calls return with the results in place, like cuZFP's.
 *
 * cuZFP codes every stream at a fixed rate whatever its zfp_stream holds;
 * here all four parameters count: fixed rate (stream_set_rate) takes the
 * fixed-rate path, and zfp's other modes (zfp_stream_set_precision,
 * zfp_stream_set_accuracy in zfp_structs.h, or the fields set directly)
 * take its general mode.  A general-mode stream buffer is read as
 * zfp_stream_maximum_size bytes, the size cuZFP's callers allocate.
 * Strided fields are coded through their strides in fixed-rate mode.
 */
#ifndef GZFP_CUZFP_H
#define GZFP_CUZFP_H

#include <stddef.h>

#include "zfp_structs.h"

namespace cuZFP {

size_t compress(zfp_stream* stream, zfp_field* field);
void decompress(zfp_stream* stream, zfp_field* field);

/* status of the calling thread's last compress / decompress (GZFP_OK = 0) */
int last_status();

}  // namespace cuZFP

#endif /* GZFP_CUZFP_H */
