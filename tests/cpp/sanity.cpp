// sanity.cpp -- C++ caller of the cuZFP drop-in header (include/cuZFP.h).
//
// Mirrors the checks of cuZFP's own gtest smoke tests: exact integer round
// trips at rate 8 for 1D (128 values), 2D (4x4) and 3D (16x8x4) float
// fields (src/tests/t_sanity_check_{1,2,3}.cpp) and the same 3D case with a
// device-resident stream (src/tests/t_cuda_mem.cu), plus a strided field and
// zfp's fixed-accuracy mode.  Built and run by
// tests/test_cpp_dropin.py on a GPU machine; prints "ok" on success.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
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
  // a strided field (every other value of a buffer) is coded through its
  // strides: the stream of its contiguous copy, decoded back in place
  {
    std::vector<float> v(128), c(64);
    for (int i = 0; i < 128; i++) v[i] = (float)((i * 37) % 101);
    for (int i = 0; i < 64; i++) c[i] = v[2 * i];
    zfp_field* fs = zfp_field_3d(v.data(), zfp_type_float, 4, 4, 4);
    fs->sx = 2;
    fs->sy = 8;
    fs->sz = 32;
    zfp_field* fc = zfp_field_3d(c.data(), zfp_type_float, 4, 4, 4);
    zfp_stream zs, zc;
    stream_set_rate(&zs, 8, fs->type, 3);
    stream_set_rate(&zc, 8, fc->type, 3);
    std::vector<unsigned char> bs(zfp_stream_maximum_size(&zs, fs)), bc(bs.size());
    zs.stream = (Word*)bs.data();
    zc.stream = (Word*)bc.data();
    const size_t ns = compress(&zs, fs), nc = compress(&zc, fc);
    if (!ns || ns != nc || std::memcmp(bs.data(), bc.data(), ns)) fails++;
    std::vector<float> back(128, -7.0f), cback(64);
    zfp_field* gs = zfp_field_3d(back.data(), zfp_type_float, 4, 4, 4);
    gs->sx = 2;
    gs->sy = 8;
    gs->sz = 32;
    decompress(&zs, gs);
    zfp_field* gc = zfp_field_3d(cback.data(), zfp_type_float, 4, 4, 4);
    decompress(&zc, gc);
    for (int i = 0; i < 64; i++)
      if (back[2 * i] != cback[i] || back[2 * i + 1] != -7.0f) {
        fails++;
        break;
      }
    zfp_field_free(fs);
    zfp_field_free(fc);
    zfp_field_free(gs);
    zfp_field_free(gc);
  }
  // zfp's fixed-accuracy mode through the same calls: the stream of
  // gzfp_compress_mode, decoded within the tolerance
  {
    const unsigned nx = 16, ny = 8, nz = 4, n = nx * ny * nz;
    std::vector<double> in(n), out(n, -1.0);
    for (unsigned i = 0; i < n; i++) in[i] = 0.01 * i + 0.5 * (i % 5);
    zfp_field* f = zfp_field_3d(in.data(), zfp_type_double, nx, ny, nz);
    zfp_stream zfp;
    zfp_stream_set_accuracy(&zfp, 1e-4, zfp_type_double);
    std::vector<unsigned char> buf(zfp_stream_maximum_size(&zfp, f)), ref(buf.size());
    zfp.stream = (Word*)buf.data();
    const size_t bytes = compress(&zfp, f);
    gzfp_mode m{zfp.minbits, zfp.maxbits, zfp.maxprec, zfp.minexp};
    size_t rbytes = 0;
    if (!bytes || gzfp_compress_mode(GZFP_TYPE_DOUBLE, nx, ny, nz, &m, in.data(), ref.data(),
                                     ref.size(), &rbytes, nullptr, nullptr) != GZFP_OK ||
        rbytes != bytes || std::memcmp(buf.data(), ref.data(), bytes))
      fails++;
    zfp_field* g = zfp_field_3d(out.data(), zfp_type_double, nx, ny, nz);
    decompress(&zfp, g);
    if (last_status() != GZFP_OK) fails++;
    for (unsigned i = 0; i < n; i++)
      if (out[i] - in[i] > 1e-4 || in[i] - out[i] > 1e-4) {
        fails++;
        break;
      }
    zfp_field_free(f);
    zfp_field_free(g);
  }
  std::printf(fails ? "FAILED %d\n" : "ok\n", fails);
  return fails ? 1 : 0;
}
