/*
 * cuZFP.h -- drop-in C++ entry points of the GB300 codec (libgzfp.so).
 *
 * Same declarations as cuZFP's src/cuZFP/cuZFP.h:9-10.  `compress` returns
 * the stream size in bytes and 0 on failure; `decompress` returns nothing,
 * as in cuZFP.  Both record failures in cuZFP::last_status() (a gzfp status
 * code, include/gzfp.h) and gzfp_last_error(), where cuZFP only printed them
 * (src/cuZFP/ErrorCheck.cu:11-19).  Buffers may be host or device memory;
 * the calls return with the results in place, like cuZFP's.
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
