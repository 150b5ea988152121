// sg_tr_mg_mixed_st.cu -- history loop and event kernels, mixed form (FP32 cross sections, distances and sampling; FP64 positions, coincidence tests and tally sums),
// multigroup data (neutronMGstd), transportOperatorST.
#include <algorithm>
#include "sg_dispatch.cuh"

namespace sg {
template <>
cudaError_t launch_kind_op<float, false, OP_ST>(int kind, const TransportArgs<float>& a, int maxl, size_t smem,
                                          cudaStream_t s, int* grid_out) {
  return launch_unit<float, false, OP_ST>(kind, a, maxl, smem, s, grid_out);
}
}  // namespace sg
