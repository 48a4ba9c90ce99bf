/*
 * gzfp.h -- C ABI of the GB300 ZFP codec (libgzfp.so).
 *
 * Drop-in replacement for the compress / decompress path of cuZFP
 * (src/cuZFP/cuZFP.h:9-10, implemented in src/cuZFP/cuZFP.cu:174-269): the
 * same inputs -- array pointer, dimensions, scalar type and rate in bits per
 * value -- and the same fixed-rate stream as zfp 0.5.0's zfp_compress with
 * zfp_stream_set_rate(..., wra = 0), bit for bit.
 *
 * Plain C types only: pointers, sizes and an opaque CUDA stream handle
 * (a cudaStream_t passed as void*, NULL = the legacy default stream).
 * Every function returns a status code and never aborts.
 *
 * Pointers may be device or host memory, as in cuZFP (is_gpu_ptr,
 * src/cuZFP/pointers.cuh:12-22).  When both the array and the stream buffer
 * are device (or managed) memory the call is asynchronous on `cuda_stream`
 * and touches nothing else.  When either is host memory the library stages
 * it through a device workspace it owns, copies results back and
 * synchronises `cuda_stream` before returning.
 */
#ifndef GZFP_H
#define GZFP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* scalar types: the values of zfp_type (src/cuZFP/zfp_structs.h:31-37) */
#define GZFP_TYPE_INT32 1
#define GZFP_TYPE_INT64 2
#define GZFP_TYPE_FLOAT 3
#define GZFP_TYPE_DOUBLE 4

/* status codes */
#define GZFP_OK 0
#define GZFP_ERR_ARG 1         /* bad dimensions, type, rate, or null pointer */
#define GZFP_ERR_UNSUPPORTED 2 /* a field or mode this path does not handle */
#define GZFP_ERR_CAPACITY 3    /* output buffer smaller than needed */
#define GZFP_ERR_CUDA 4        /* a CUDA runtime call failed; see gzfp_last_error */

/* Library version, major * 10000 + minor * 100 + patch. */
int gzfp_version(void);

/* Static description of a status code. */
const char* gzfp_status_string(int status);

/* Detail of the last failure on the calling thread ("" if none). */
const char* gzfp_last_error(void);

/* Bits per block for `rate` bits per value on a `dims`-dimensional field:
   floor(4^dims * rate + 0.5), raised to 1 + exponent bits for float and
   double (integer blocks carry no exponent).  Replaces stream_set_rate
   (src/cuZFP/zfp_structs.h:46-76), computed as zfp 0.5.0's
   zfp_stream_set_rate with wra = 0 (zfp-0.5.0/src/zfp.c:405-430).  Returns 0
   for an unknown type, dims outside 1..3, or an integer rate of 0 bits. */
unsigned gzfp_rate_to_maxbits(int type, unsigned dims, double rate);

/* Exact size in bytes of the compressed stream: ceil(blocks * maxbits / 64)
   64-bit words (zfp_compress's return value, zfp-0.5.0/src/zfp.c:603-630).
   ny = 0 (and nz = 0) selects 1D, nz = 0 selects 2D.  0 on bad arguments. */
size_t gzfp_stream_size(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits);

/* Worst-case buffer size as computed by zfp_stream_maximum_size
   (src/cuZFP/zfp_structs.h:222-251) for a fixed-rate stream of `maxbits`
   bits per block; includes zfp's 148 header bits. */
size_t gzfp_maximum_size(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits);

/* Compress the contiguous array a[nz][ny][nx] at `rate` bits per value into
   `stream` (capacity bytes).  On success *out_bytes (if not NULL) receives
   the stream size.  Replaces cuZFP::compress (src/cuZFP/cuZFP.cu:174-210). */
int gzfp_compress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                  const void* data, void* stream, size_t capacity, size_t* out_bytes,
                  void* cuda_stream);

/* Decompress `bytes` bytes of `stream` into the contiguous array `data`.
   Replaces cuZFP::decompress (src/cuZFP/cuZFP.cu:212-269). */
int gzfp_decompress(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                    const void* stream, size_t bytes, void* data, void* cuda_stream);

/* As gzfp_compress / gzfp_decompress, with the block size given directly in
   bits (zfp_stream.maxbits), as cuZFP's internal::encode / internal::decode
   take it (src/cuZFP/cuZFP.cu:26-105).  Any maxbits >= 1 + exponent bits
   (9 for float, 12 for double, 1 for int32 and int64) up to 1<<20 is
   accepted.

   Integer fields (GZFP_TYPE_INT32 / INT64, cuZFP.cu:196-205) are coded as
   zfp 0.5.0's integer block codec codes them (zfp_encode_block_int32_<d>,
   zfp-0.5.0/src/template/encode.c:154-185): no exponent, the whole budget,
   all planes eligible.  zfp has no partial integer block API; partial edge
   blocks use its pad rule, as for floating point. */
int gzfp_compress_bits(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                       const void* data, void* stream, size_t capacity, size_t* out_bytes,
                       void* cuda_stream);
int gzfp_decompress_bits(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                         const void* stream, size_t bytes, void* data, void* cuda_stream);

/* Strided fields: value (x, y, z) at element x*sx + y*sy + z*sz of `data`,
   signed strides counted in values, 0 selecting the contiguous stride of
   that axis (1, nx, nx*ny) -- zfp_field's sx/sy/sz, as zfp 0.5.0 compresses
   them (zfp-0.5.0/src/template/compress.c, compress_strided).  cuZFP keeps
   these fields in its zfp_field (src/cuZFP/zfp_structs.h:39-44) but codes
   every field as contiguous.  The stream is the one zfp_compress writes for
   the strided field.  A host `data` pointer is staged as the whole span of
   values the strides reach; decompression into host memory reads that span
   first, so values between the field's are kept. */
int gzfp_compress_strided(int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                          long long sy, long long sz, unsigned maxbits, const void* data,
                          void* stream, size_t capacity, size_t* out_bytes, void* cuda_stream);
int gzfp_decompress_strided(int type, unsigned nx, unsigned ny, unsigned nz, long long sx,
                            long long sy, long long sz, unsigned maxbits, const void* stream,
                            size_t bytes, void* data, void* cuda_stream);

/* ------------------------------------------------------------ headers ---
   zfp 0.5.0's self-describing stream header (zfp_write_header /
   zfp_read_header with ZFP_HEADER_FULL, zfp-0.5.0/src/zfp.c:661-719): a
   32-bit magic ('z', 'f', 'p', codec 5), 52 bits of field metadata (scalar
   type, dimensionality and sizes: up to 2^32 - 1 values in 1D, 2^24 per
   axis in 2D, 2^16 per axis in 3D) and the fixed-rate mode in 12 bits
   (blocks up to 2048 bits) or 64 bits (up to 32768).  zfp_compress after
   zfp_write_header continues the same bit stream, so the first block starts
   right after the header: the stream zfp's command-line tool writes with -h.
   No counterpart in cuZFP, whose streams carry no header. */
#define GZFP_HEADER_MAX_BITS 148

/* Write the header into the host buffer `header` (capacity bytes; 24 are
   always enough); *header_bits receives its length in bits. */
int gzfp_write_header(int type, unsigned nx, unsigned ny, unsigned nz, unsigned maxbits,
                      void* header, size_t capacity, size_t* header_bits);

/* Parse a header from the host buffer `header`.  Streams in zfp's other
   modes (fixed precision or accuracy, expert parameters) are reported with
   GZFP_ERR_UNSUPPORTED. */
int gzfp_read_header(const void* header, size_t bytes, int* type, unsigned* nx, unsigned* ny,
                     unsigned* nz, unsigned* maxbits, size_t* header_bits);

/* Compress with a header in front, or decompress a stream that has one
   (the field's type and shape come from the header; `data_bytes` is the
   capacity of `data`).  Pointers may be host or device memory.
   gzfp_decompress_headed takes streams of every mode: a header naming
   fixed precision, fixed accuracy or other parameters (see "general
   modes" below) is decoded in that mode, its blocks found by the serial
   walk of gzfp_index_blocks. */
int gzfp_compress_headed(int type, unsigned nx, unsigned ny, unsigned nz, double rate,
                         const void* data, void* stream, size_t capacity, size_t* out_bytes,
                         void* cuda_stream);
int gzfp_decompress_headed(const void* stream, size_t bytes, void* data, size_t data_bytes,
                           void* cuda_stream);

/* ------------------------------------------------------- block access ---
   Random access to single blocks of a fixed-rate stream: zfp's per-block
   API (zfp_encode_block_* / zfp_decode_block_* and their partial-block
   forms, zfp-0.5.0/inc/zfp.h:452-521) over a list of blocks, as zfp's
   compressed arrays use it to fetch and write back cached blocks
   (zfp::array3::decode / encode, zfp-0.5.0/array/zfparray3.h:225-255).
   Block indices[i] occupies bits [indices[i] * maxbits, (indices[i] + 1) *
   maxbits) of the stream; tile i of `tiles` holds its 4^dims values, x
   fastest.  `shapes` (NULL: every block whole) holds zfp's partial-block
   codes, two bits per axis with x lowest, each 4 minus the block's extent
   along that axis: a partial block is encoded from its valid values with
   zfp's padding, and decoding one writes only those values of its tile.
   Encoding rewrites each listed slot in place and keeps every other bit of
   the stream; the indices of one call must be distinct.  Indices past the
   end of the stream are skipped.  Pointers may be host or device memory
   (host buffers, the stream included, are staged whole).
   No counterpart in cuZFP. */
int gzfp_decode_blocks(int type, unsigned dims, unsigned maxbits, const void* stream,
                       size_t bytes, const unsigned long long* indices,
                       const unsigned char* shapes, size_t count, void* tiles, void* cuda_stream);
int gzfp_encode_blocks(int type, unsigned dims, unsigned maxbits, const void* tiles,
                       const unsigned long long* indices, const unsigned char* shapes,
                       size_t count, void* stream, size_t bytes, void* cuda_stream);

/* ------------------------------------------------------ general modes ---
   zfp's other compression modes -- fixed precision, fixed accuracy, or any
   setting of its four stream parameters (zfp_stream_set_precision,
   zfp_stream_set_accuracy, zfp_stream_set_params; zfp-0.5.0/src/zfp.c:
   432-510) -- in which every block takes as many bits as it needs (at
   least minbits, at most maxbits) and follows the previous one directly.
   The stream is the one zfp_compress writes with those parameters.
   No counterpart in cuZFP, which is fixed-rate only
   (src/utils/cuda_zfp.cpp:350-354). */
typedef struct {
  unsigned minbits;  /* fewest bits per block */
  unsigned maxbits;  /* most bits per block */
  unsigned maxprec;  /* most bit planes per block, 1..64 */
  int minexp;        /* exponent of the lowest bit plane coded (floating point) */
} gzfp_mode;

/* The parameters zfp_stream_set_rate (wra = 0), zfp_stream_set_precision
   and zfp_stream_set_accuracy set. */
int gzfp_mode_rate(int type, unsigned dims, double rate, gzfp_mode* mode);
int gzfp_mode_precision(int type, unsigned precision, gzfp_mode* mode);
int gzfp_mode_accuracy(int type, double tolerance, gzfp_mode* mode);

/* Bytes a stream can take at most (zfp_stream_maximum_size without the
   header allowance); 0 for bad arguments. */
size_t gzfp_mode_maximum_size(int type, unsigned nx, unsigned ny, unsigned nz,
                              const gzfp_mode* mode);

/* Compress.  Every block is coded on the GPU into a scratch slot of its
   largest size, the start bits follow from a scan of the block lengths,
   and the blocks are moved into place: the call returns when the stream
   is complete (its size is only known then).  `offsets` (optional, host or
   device, one entry per block) receives every block's start bit; keep them
   to decode in parallel.  Fixed-rate parameters take the fixed-rate path. */
int gzfp_compress_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                       const void* data, void* stream, size_t capacity, size_t* out_bytes,
                       unsigned long long* offsets, void* cuda_stream);

/* Decompress.  With `offsets` every block decodes in parallel from its
   start bit; without, gzfp_index_blocks finds them first. */
int gzfp_decompress_mode(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                         const void* stream, size_t bytes, const unsigned long long* offsets,
                         void* data, void* cuda_stream);

/* Every block's start bit in a stream written with `mode` (by zfp or by
   gzfp_compress_mode), found by one GPU thread walking the blocks in
   order: its time grows with the number of blocks, not with the GPU. */
int gzfp_index_blocks(int type, unsigned nx, unsigned ny, unsigned nz, const gzfp_mode* mode,
                      const void* stream, size_t bytes, unsigned long long* offsets,
                      void* cuda_stream);

/* zfp's full header for any parameters (zfp_stream_mode's 12-bit forms
   for fixed rate, precision and accuracy, else its 64-bit form), and the
   header and parameters of a stream of any mode; gzfp_compress_mode_headed
   writes the header, then the blocks (offsets count from the stream's
   first bit). */
int gzfp_write_header_mode(int type, unsigned nx, unsigned ny, unsigned nz,
                           const gzfp_mode* mode, void* header, size_t capacity,
                           size_t* header_bits);
int gzfp_read_header_mode(const void* header, size_t bytes, int* type, unsigned* nx,
                          unsigned* ny, unsigned* nz, gzfp_mode* mode, size_t* header_bits);
int gzfp_compress_mode_headed(int type, unsigned nx, unsigned ny, unsigned nz,
                              const gzfp_mode* mode, const void* data, void* stream,
                              size_t capacity, size_t* out_bytes, unsigned long long* offsets,
                              void* cuda_stream);

/* ------------------------------------------------------------ batches ---
   Many arrays -- each with its own shape, scalar type, dimensionality and
   bits per block -- coded by one kernel per kind (dimensionality x scalar
   type) over a device-side work list of (array, chunk of blocks) items.  Every array's stream is the one
   gzfp_compress_bits would write.  Device pointers only; calls are
   asynchronous on `cuda_stream`.  No counterpart in cuZFP, which codes one
   array per call (src/cuZFP/cuZFP.cu:174-269). */

typedef struct {
  int type;               /* GZFP_TYPE_FLOAT, _DOUBLE, _INT32 or _INT64 */
  unsigned nx, ny, nz;    /* as gzfp_compress: ny = 0 for 1D, nz = 0 for 2D */
  unsigned maxbits;       /* bits per block (gzfp_rate_to_maxbits) */
  void* field;            /* device array: input of compress, output of decompress */
  void* stream;           /* device words: output of compress, input of decompress */
  size_t stream_capacity; /* bytes at `stream` */
} gzfp_batch_item;

/* Launch shape: threads per CTA (64, 128, 256); ctas_per_sm 0 (the default)
   for the grid kernel, one CTA per slice of threads blocks of a chunk, one
   block per thread, scheduled by the hardware; else the persistent kernel
   with that many resident CTAs per SM (capped at what fits), which claim
   chunks from a counter; blocks per thread per chunk (1, 2, 4); and, for
   the persistent kernel, whether the next chunk is claimed while the
   current one is coded (claim_ahead). */
typedef struct {
  int threads;
  int ctas_per_sm;
  int blocks_per_thread;
  int claim_ahead;
} gzfp_batch_config;

void gzfp_batch_default_config(gzfp_batch_config* cfg);

/* Detail of the last batch-path failure on the calling thread. */
const char* gzfp_batch_last_error(void);

/* One batch, built and launched now (cfg may be NULL for the default).  The
   library keeps one work list per device: a call first waits on the host
   until the previous call's kernel, on whatever stream, has finished with
   it, then queues its own work and returns. */
int gzfp_batch_compress(const gzfp_batch_item* items, int count, const gzfp_batch_config* cfg,
                        void* cuda_stream);
int gzfp_batch_decompress(const gzfp_batch_item* items, int count, const gzfp_batch_config* cfg,
                          void* cuda_stream);

/* A batch prepared once and captured in a CUDA graph (work list upload,
   zeroing, claim counter reset, per-kind kernels); each launch replays it
   on the same buffers. */
typedef struct gzfp_batch_plan gzfp_batch_plan;
int gzfp_batch_plan_create(const gzfp_batch_item* items, int count, int decompress,
                           const gzfp_batch_config* cfg, gzfp_batch_plan** plan);
int gzfp_batch_plan_launch(gzfp_batch_plan* plan, void* cuda_stream);
void gzfp_batch_plan_destroy(gzfp_batch_plan* plan);

/* Time every launch shape on this batch (graph replays, `repeats` each)
   and return the fastest in *best and its time in *best_ms. */
int gzfp_batch_autotune(const gzfp_batch_item* items, int count, int decompress, int repeats,
                        gzfp_batch_config* best, float* best_ms, void* cuda_stream);

/* ---------------------------------------------------- no-alloc batches ---
   gzfp_batch_compress / gzfp_batch_decompress (decompress = 0 / 1) with no
   memory allocated by the call: the work list (claim counter, array
   descriptors, chunk table) lives in a fixed device array compiled into the
   library, about 2.1 MiB per device.  No counterpart in cuZFP, which
   cudaMallocs and frees on every host-pointer call (src/cuZFP/cuZFP.cu:107-170).

   For callers that must not allocate: code running inside a device-memory
   allocator or its out-of-memory handler (an allocation there re-enters the
   allocator), programs whose caching allocator has already reserved nearly
   all device memory, and latency-bound loops that cannot afford cudaFree's
   device-wide synchronisation or a failed cudaMalloc in the middle of a step.

   Limits: at most GZFP_NOALLOC_MAX_ITEMS arrays and GZFP_NOALLOC_MAX_CHUNKS
   chunks of threads * blocks_per_thread zfp blocks (2^19 chunks of 128
   blocks = 2^26 blocks at the default shape); larger batches are rejected
   with GZFP_ERR_CAPACITY and a message naming the limit, before any GPU work.

   Set-up: every call looks up the array's device address in the current
   context (cudaGetSymbolAddress); with lazy module loading the first call on
   a device is also when the driver loads the module.  A call on a stream
   that is being captured into a CUDA graph is refused with GZFP_ERR_ARG
   before any work is queued.

   The call waits on the host for earlier work on `cuda_stream` (the
   descriptor upload is a pageable copy) and then queues its work
   asynchronously.  All calls on one device share the one work list:
   calls whose work overlaps on the device -- from different streams or
   threads without ordering between them -- race and give wrong streams.
   Calls in sequence on one stream are safe. */
#define GZFP_NOALLOC_MAX_ITEMS 1024
#define GZFP_NOALLOC_MAX_CHUNKS (1u << 19)
int gzfp_batch_run_noalloc(const gzfp_batch_item* items, int count, int decompress,
                           const gzfp_batch_config* cfg, void* cuda_stream);

/* ------------------------------------------------------------ serving ---
   A request server.  Compress and decompress requests of mixed shape,
   scalar type and rate arrive over time.  A request is admitted once the
   server's device-memory budget can hold its output.  Inputs stay resident
   in device memory; outputs live in a device arena of `budget_bytes`,
   allocated once per run, and are released when their request completes
   (optionally after a copy to a caller buffer).  Two modes:

   * slots (device_queue = 0; every scalar type and dimensionality): admitted requests are coded together by the batched
     path's kernels, and up to `max_inflight` batches run on the device at
     once, each on its own stream; a request that arrives while earlier
     batches run joins the next batch on a free slot.
   * device queue (device_queue = 1, the default; every scalar type and
     dimensionality): a persistent scheduler kernel stays on the device and drains a request
     table in pinned host memory that the GPU reads directly.  The host
     publishes an admitted request by writing its descriptor and raising the
     published count; the scheduler launches each published request, in
     order, as its own grid of the request's coder with a device-side
     launch, so a request that arrives while others run starts as soon as
     SMs free up, alongside them, with no host launch.  The request's last
     CTA marks it done in host memory.  Every wait of the scheduler is
     bounded: after `idle_exit_us` with nothing published it leaves, and the
     host starts a new one when new work is published.

   No counterpart in cuZFP, whose calls are synchronous and one array at a
   time (src/cuZFP/cuZFP.cu:174-269). */

#define GZFP_SERVE_COMPRESS 0
#define GZFP_SERVE_DECOMPRESS 1

typedef struct {
  int op;                /* GZFP_SERVE_COMPRESS or GZFP_SERVE_DECOMPRESS */
  int type;              /* GZFP_TYPE_FLOAT, _DOUBLE, _INT32 or _INT64 */
  unsigned nx, ny, nz;   /* as gzfp_compress */
  unsigned maxbits;      /* bits per block */
  const void* input;     /* device: the field (compress) or stream words (decompress) */
  void* copy_to;         /* device buffer that receives the output, or NULL */
  double arrival;        /* seconds after the start of the run */
} gzfp_serve_request;

typedef struct {
  double admitted;       /* seconds after the start: output memory granted, batch launched
                            (device queue: request published) */
  double completed;      /* seconds after the start: the request's batch finished
                            (device queue: its grid marked it done) */
  size_t output_bytes;
  int batch;             /* index of the batch (device queue: the publication) that ran it,
                            -1 if never run */
  int status;            /* GZFP_OK, or GZFP_ERR_CAPACITY for an output larger than the budget */
  double device_start;   /* device queue: device clock, seconds after the run's first CTA,
                            when the request's first CTA started (0 in slot mode) */
  double device_end;     /* device queue: the same, when its last CTA was done */
} gzfp_serve_result;

typedef struct {
  size_t budget_bytes;   /* device arena for request outputs */
  int max_batch;         /* requests per batch or publication (1..65535) */
  int max_inflight;      /* slot mode: batches on the device at once (1..8) */
  gzfp_batch_config compress_cfg;   /* slot mode: launch shapes (see gzfp_batch_autotune) */
  gzfp_batch_config decompress_cfg;
  int device_queue;      /* 0: slots; 1: device queue (the default) */
  unsigned idle_exit_us; /* device queue: the scheduler leaves after this long with nothing
                            published (1..10^7 us; default 2000) */
} gzfp_serve_config;

typedef struct {
  double wall;           /* seconds from the start to the last completion */
  int batches;           /* batches launched (device queue: publications) */
  double mean_batch;     /* requests per batch (device queue: per publication) */
  size_t peak_bytes;     /* largest arena use */
  double busy;           /* fraction of the run with at least one request on the device */
  int kernels;           /* kernels launched (slots: chunk tables and per-kind kernels;
                            device queue: schedulers and one grid per request) */
  double mean_inflight;  /* requests on the device when a request is admitted, itself
                            included, averaged over the admitted requests */
  int schedulers;        /* device queue: scheduler launches (0 in slot mode) */
} gzfp_serve_stats;

void gzfp_serve_default_config(gzfp_serve_config* cfg);

/* Serve `count` requests (any order; each is released at its arrival time
   on the host clock) and fill results[i] for reqs[i].  Returns after every
   request has completed.  The calling thread polls; the current device
   runs everything.  Failure details: gzfp_batch_last_error. */
int gzfp_serve_run(const gzfp_serve_request* reqs, int count, const gzfp_serve_config* cfg,
                   gzfp_serve_result* results, gzfp_serve_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* GZFP_H */
