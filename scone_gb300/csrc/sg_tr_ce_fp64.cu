// sg_tr_ce_fp64.cu -- all-FP64 verification form of the history loop and event kernels with
// continuous-energy data (neutronCEstd).  Built with -fmad=false, like sg_tr_fp64.cu, so the
// arithmetic rounds exactly as SCONE's.
#include <algorithm>
#include "sg_dispatch.cuh"

namespace sg {

template <>
cudaError_t launch_kind_ce<double>(int kind, const TransportArgs<double>& a, int maxl, bool dt, size_t smem,
                                   cudaStream_t s, int* grid_out) {
  return launch_kind_impl<double, true>(kind, a, maxl, dt, smem, s, grid_out);
}

}  // namespace sg
