// sanity.cpp -- C++ caller of the cuZFP drop-in header (include/cuZFP.h).
//
// Mirrors the checks of cuZFP's own gtest smoke tests: exact integer round
// trips at rate 8 for 1D (128 values), 2D (4x4) and 3D (16x8x4) float
// fields (src/tests/t_sanity_check_{1,2,3}.cpp) and the same 3D case with a
// device-resident stream (src/tests/t_cuda_mem.cu).  Built and run by
// tests/test_cpp_dropin.py on a GPU machine; prints "ok" on success.
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include <cuZFP.h>

using namespace cuZFP;

static int roundtrip(unsigned nx, unsigned ny, unsigned nz, bool device_stream) {
  const unsigned dims = nz ? 3 : ny ? 2 : 1;
  const size_t n = (size_t)nx * (ny ? ny : 1) * (nz ? nz : 1);
  std::vector<float> in(n), out(n, -1.0f);
  for (size_t i = 0; i < n; i++) in[i] = (float)i;
  zfp_field* f = dims == 3 ? zfp_field_3d(in.data(), zfp_type_float, nx, ny, nz)
               : dims == 2 ? zfp_field_2d(in.data(), zfp_type_float, nx, ny)
                           : zfp_field_1d(in.data(), zfp_type_float, nx);
  zfp_stream zfp;
  stream_set_rate(&zfp, 8, f->type, dims);
  size_t cap = zfp_stream_maximum_size(&zfp, f);
  std::vector<unsigned char> host(cap);
  void* dev = nullptr;
  if (device_stream) {
    if (cudaMalloc(&dev, cap) != cudaSuccess) return 1;
    zfp.stream = (Word*)dev;
  } else {
    zfp.stream = (Word*)host.data();
  }
  size_t bytes = compress(&zfp, f);
  if (bytes == 0 || last_status() != GZFP_OK) {
    std::printf("compress failed: %s\n", gzfp_last_error());
    return 1;
  }
  zfp_field* g = dims == 3 ? zfp_field_3d(out.data(), zfp_type_float, nx, ny, nz)
               : dims == 2 ? zfp_field_2d(out.data(), zfp_type_float, nx, ny)
                           : zfp_field_1d(out.data(), zfp_type_float, nx);
  decompress(&zfp, g);
  if (last_status() != GZFP_OK) {
    std::printf("decompress failed: %s\n", gzfp_last_error());
    return 1;
  }
  int bad = 0;
  for (size_t i = 0; i < n; i++)
    if ((int)i != (int)out[i]) bad++;
  zfp_field_free(f);
  zfp_field_free(g);
  if (dev) cudaFree(dev);
  if (bad) std::printf("%u x %u x %u: %d values differ\n", nx, ny, nz, bad);
  return bad ? 1 : 0;
}

int main() {
  int fails = 0;
  fails += roundtrip(128, 0, 0, false);
  fails += roundtrip(4, 4, 0, false);
  fails += roundtrip(16, 8, 4, false);
  fails += roundtrip(16, 8, 4, true);
  // a strided field is reported, not silently compressed
  std::vector<float> v(64, 1.0f);
  zfp_field* f = zfp_field_3d(v.data(), zfp_type_float, 4, 4, 4);
  f->sx = 2;
  zfp_stream zfp;
  stream_set_rate(&zfp, 8, f->type, 3);
  std::vector<unsigned char> buf(zfp_stream_maximum_size(&zfp, f));
  zfp.stream = (Word*)buf.data();
  if (compress(&zfp, f) != 0 || last_status() != GZFP_ERR_UNSUPPORTED) fails++;
  zfp_field_free(f);
  std::printf(fails ? "FAILED %d\n" : "ok\n", fails);
  return fails ? 1 : 0;
}
