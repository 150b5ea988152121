// sg_batch_fp64.cu -- all-FP64 form of the batched gen loop.  Built with -fmad=false, as the
// single-problem FP64 form, so each history rounds exactly as SCONE's.
#include "sg_batch.cuh"

namespace sg {
template <>
cudaError_t launch_batch<double>(const BatchLaunch& L, bool dt, int grid, int block, cudaStream_t s) {
  return launch_batch_impl<double>(L, dt, grid, block, s);
}
template <>
int batch_occupancy<double>(int maxl, bool dt, int block) { return batch_occupancy_impl<double>(maxl, dt, block); }
}  // namespace sg
