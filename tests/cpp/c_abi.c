/* c_abi.c -- a plain C caller of include/gzfp.h (host buffers only, no CUDA
 * headers): fixed-rate round trip, a headed stream read back from its
 * header alone, fixed accuracy with and without block offsets, and random
 * access to one block.  Built and run by tests/test_cpp_dropin.py on a GPU
 * machine; prints "ok" on success. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gzfp.h"

#define NX 20
#define NY 17
#define NZ 9
#define N (NX * NY * NZ)

static int check(int st, const char* what) {
  if (st != GZFP_OK) printf("%s: %s (%s)\n", what, gzfp_status_string(st), gzfp_last_error());
  return st != GZFP_OK;
}

int main(void) {
  int fails = 0;
  size_t i, bytes;
  double* a = malloc(N * sizeof(double));
  double* b = malloc(N * sizeof(double));
  double* c = malloc(N * sizeof(double));
  for (i = 0; i < N; i++) a[i] = sin(0.1 * (double)i) + 0.001 * (double)(i % 7);

  /* fixed rate 16 */
  {
    unsigned mb = gzfp_rate_to_maxbits(GZFP_TYPE_DOUBLE, 3, 16.0);
    size_t cap = gzfp_stream_size(GZFP_TYPE_DOUBLE, NX, NY, NZ, mb);
    void* s = malloc(cap);
    fails += check(gzfp_compress(GZFP_TYPE_DOUBLE, NX, NY, NZ, 16.0, a, s, cap, &bytes, NULL),
                   "compress");
    fails += check(gzfp_decompress(GZFP_TYPE_DOUBLE, NX, NY, NZ, 16.0, s, bytes, b, NULL),
                   "decompress");
    for (i = 0; i < N; i++)
      if (fabs(a[i] - b[i]) > 1e-3) {
        fails++;
        break;
      }
    /* random access: block 5 alone equals its place in the field */
    {
      unsigned long long idx = 5;
      double tile[64];
      unsigned bx = (NX + 3) / 4;  /* block 5: (5 % bx, 5 / bx, 0) */
      unsigned x0 = 4 * (5 % bx), y0 = 4 * (5 / bx), x, y, z;
      fails += check(gzfp_decode_blocks(GZFP_TYPE_DOUBLE, 3, mb, s, bytes, &idx, NULL, 1, tile,
                                        NULL), "decode_blocks");
      for (z = 0; z < 4; z++)
        for (y = 0; y < 4; y++)
          for (x = 0; x < 4; x++)
            if (tile[x + 4 * y + 16 * z] != b[(x0 + x) + NX * ((y0 + y) + NY * z)]) fails++;
    }
    free(s);
  }

  /* a headed stream: type, shape and rate from the header */
  {
    size_t cap = gzfp_maximum_size(GZFP_TYPE_DOUBLE, NX, NY, NZ,
                                   gzfp_rate_to_maxbits(GZFP_TYPE_DOUBLE, 3, 12.0));
    void* s = malloc(cap);
    int type;
    unsigned x, y, z, mb;
    size_t hbits;
    fails += check(gzfp_compress_headed(GZFP_TYPE_DOUBLE, NX, NY, NZ, 12.0, a, s, cap, &bytes,
                                        NULL), "compress_headed");
    fails += check(gzfp_read_header(s, bytes, &type, &x, &y, &z, &mb, &hbits), "read_header");
    if (type != GZFP_TYPE_DOUBLE || x != NX || y != NY || z != NZ || hbits != 96) fails++;
    memset(c, 0, N * sizeof(double));
    fails += check(gzfp_decompress_headed(s, bytes, c, N * sizeof(double), NULL),
                   "decompress_headed");
    for (i = 0; i < N; i++)
      if (fabs(a[i] - c[i]) > 1e-2) {
        fails++;
        break;
      }
    free(s);
  }

  /* fixed accuracy: within the tolerance, decoded with and without offsets */
  {
    gzfp_mode m;
    size_t nb = (size_t)((NX + 3) / 4) * ((NY + 3) / 4) * ((NZ + 3) / 4), cap;
    unsigned long long* offs = malloc(nb * sizeof *offs);
    void* s;
    fails += check(gzfp_mode_accuracy(GZFP_TYPE_DOUBLE, 1e-6, &m), "mode_accuracy");
    cap = gzfp_mode_maximum_size(GZFP_TYPE_DOUBLE, NX, NY, NZ, &m);
    s = malloc(cap);
    fails += check(gzfp_compress_mode(GZFP_TYPE_DOUBLE, NX, NY, NZ, &m, a, s, cap, &bytes, offs,
                                      NULL), "compress_mode");
    fails += check(gzfp_decompress_mode(GZFP_TYPE_DOUBLE, NX, NY, NZ, &m, s, bytes, offs, b, NULL),
                   "decompress_mode");
    fails += check(gzfp_decompress_mode(GZFP_TYPE_DOUBLE, NX, NY, NZ, &m, s, bytes, NULL, c, NULL),
                   "decompress_mode (walk)");
    for (i = 0; i < N; i++)
      if (fabs(a[i] - b[i]) > 1e-6 || b[i] != c[i]) {
        fails++;
        break;
      }
    free(s);
    free(offs);
  }
  free(a);
  free(b);
  free(c);
  printf(fails ? "FAILED %d\n" : "ok\n", fails);
  return fails ? 1 : 0;
}
