// sg_tr_ce_mixed_dt.cu -- history loop and event kernels, mixed form (FP32 cross sections, distances and sampling; FP64 energies, positions and tally sums),
// continuous-energy data (neutronCEstd), transportOperatorDT.
#include <algorithm>
#include "sg_dispatch.cuh"

namespace sg {
template <>
cudaError_t launch_kind_op<float, true, OP_DT>(int kind, const TransportArgs<float>& a, int maxl, size_t smem,
                                          cudaStream_t s, int* grid_out) {
  return launch_unit<float, true, OP_DT>(kind, a, maxl, smem, s, grid_out);
}
}  // namespace sg
