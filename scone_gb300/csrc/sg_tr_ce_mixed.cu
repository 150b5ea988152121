// sg_tr_ce_mixed.cu -- mixed form with continuous-energy data: FP32 cross sections, densities,
// distances and direction kinematics; FP64 energies, energy grids, positions and tally sums.
#include <algorithm>
#include "sg_dispatch.cuh"

namespace sg {

template <>
cudaError_t launch_kind_ce<float>(int kind, const TransportArgs<float>& a, int maxl, bool dt, size_t smem,
                                  cudaStream_t s, int* grid_out) {
  return launch_kind_impl<float, true>(kind, a, maxl, dt, smem, s, grid_out);
}

}  // namespace sg
