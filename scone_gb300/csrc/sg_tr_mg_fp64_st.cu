// sg_tr_mg_fp64_st.cu -- history loop and event kernels, all-FP64 verification form,
// multigroup data (neutronMGstd), transportOperatorST. Built with -fmad=false so the arithmetic rounds
// exactly as SCONE's (no fused multiply-add).
#include <algorithm>
#include "sg_dispatch.cuh"

namespace sg {
template <>
cudaError_t launch_kind_op<double, false, OP_ST>(int kind, const TransportArgs<double>& a, int maxl, size_t smem,
                                          cudaStream_t s, int* grid_out) {
  return launch_unit<double, false, OP_ST>(kind, a, maxl, smem, s, grid_out);
}
}  // namespace sg
