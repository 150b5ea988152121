// sg_batch_mixed.cu -- mixed form of the batched gen loop: FP32 cross sections, distances and
// sampling; FP64 positions, coincidence tests and tally sums.
#include "sg_batch.cuh"

namespace sg {
template <>
cudaError_t launch_batch<float>(const BatchLaunch& L, bool dt, int grid, int block, cudaStream_t s) {
  return launch_batch_impl<float>(L, dt, grid, block, s);
}
template <>
int batch_occupancy<float>(int maxl, bool dt, int block) { return batch_occupancy_impl<float>(maxl, dt, block); }
}  // namespace sg
