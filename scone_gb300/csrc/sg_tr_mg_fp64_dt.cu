// sg_tr_mg_fp64_dt.cu -- history loop and event kernels, all-FP64 verification form,
// multigroup data (neutronMGstd), transportOperatorDT. Built with -fmad=false so the arithmetic rounds
// exactly as SCONE's (no fused multiply-add).
#include <algorithm>
#include "sg_dispatch.cuh"

namespace sg {
template <>
cudaError_t launch_kind_op<double, false, OP_DT>(int kind, const TransportArgs<double>& a, int maxl, size_t smem,
                                          cudaStream_t s, int* grid_out) {
  return launch_unit<double, false, OP_DT>(kind, a, maxl, smem, s, grid_out);
}
}  // namespace sg
