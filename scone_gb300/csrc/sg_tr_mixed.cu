// sg_tr_mixed.cu -- mixed form of the history loop: FP32 cross sections, distances and sampling,
// FP64 positions, coincidence tests and tally sums.
#include <algorithm>
#include "sg_dispatch.cuh"

namespace sg {

template <>
cudaError_t launch_kind<float>(int kind, const TransportArgs<float>& a, int maxl, bool dt, size_t smem,
                             cudaStream_t s, int* grid_out) {
  return launch_kind_impl<float, false>(kind, a, maxl, dt, smem, s, grid_out);
}

template <>
cudaError_t launch_transport<float>(const TransportArgs<float>& a, int maxl, bool dt, size_t smem,
                                  cudaStream_t s, int* grid_out) {
  return launch_kind_impl<float, false>(K_HISTORY, a, maxl, dt, smem, s, grid_out);
}

}  // namespace sg
