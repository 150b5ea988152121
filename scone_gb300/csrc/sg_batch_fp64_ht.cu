// sg_batch_fp64_ht.cu -- the batched gen loop, all-FP64 form, transportOperatorHT. Built with
// -fmad=false, as the single-problem FP64 form, so each history rounds exactly as SCONE's.
#include "sg_batch.cuh"

namespace sg {
template <>
cudaError_t launch_batch_op<double, OP_HT>(const BatchLaunch& L, int grid, int block, cudaStream_t s) {
  return launch_batch_unit<double, OP_HT>(L, grid, block, s);
}
template <>
int batch_occupancy_op<double, OP_HT>(int maxl, int lean, int block) {
  return batch_occupancy_unit<double, OP_HT>(maxl, lean != 0, block);
}
}  // namespace sg
