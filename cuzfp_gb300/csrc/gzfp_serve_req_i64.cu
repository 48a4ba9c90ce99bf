// Request grids of the device-queue server for int64_t arrays (1D, 2D, 3D;
// compress and decompress), launched from the device by the scheduler in
// gzfp_serve_queue.cu.  Relocatable device code.
#include "gzfp_serve_queue.cuh"

namespace gzfp {

__device__ cudaError_t queue_launch_i64(const QueueReq& r, uint32_t p, const QueueDev& q) {
  return queue_launch_t<int64_t>(r, p, q);
}

cudaError_t queue_setup_i64() { return queue_setup_t<int64_t>(); }

}  // namespace gzfp
