// sg_batch_mixed_dt.cu -- the batched gen loop, mixed form, transportOperatorDT.
#include "sg_batch.cuh"

namespace sg {
template <>
cudaError_t launch_batch_op<float, OP_DT>(const BatchLaunch& L, int grid, int block, cudaStream_t s) {
  return launch_batch_unit<float, OP_DT>(L, grid, block, s);
}
template <>
int batch_occupancy_op<float, OP_DT>(int maxl, int lean, int block) {
  return batch_occupancy_unit<float, OP_DT>(maxl, lean != 0, block);
}
}  // namespace sg
