// sg_tr_fp64.cu -- all-FP64 verification form of the history loop.  Built with -fmad=false so the
// arithmetic rounds exactly as SCONE's (no fused multiply-add anywhere in this translation unit).
#include <algorithm>
#include "sg_dispatch.cuh"
#include "sg_source.cuh"

namespace sg {

template <>
cudaError_t launch_kind<double>(int kind, const TransportArgs<double>& a, int maxl, bool dt, size_t smem,
                             cudaStream_t s, int* grid_out) {
  return launch_kind_impl<double, false>(kind, a, maxl, dt, smem, s, grid_out);
}

template <>
cudaError_t launch_transport<double>(const TransportArgs<double>& a, int maxl, bool dt, size_t smem,
                                  cudaStream_t s, int* grid_out) {
  return launch_kind_impl<double, false>(K_HISTORY, a, maxl, dt, smem, s, grid_out);
}

cudaError_t launch_fission_source(const DGeom& g, const DMG<double>& mg, DBank out, int n,
                                  unsigned long long master, const double* bounds6, int maxl,
                                  int* err, cudaStream_t s) {
  FissionSourceArgs a;
  a.geom = g; a.mg = mg; a.out = out; a.n = n; a.master = master; a.err = err;
  for (int i = 0; i < 6; ++i) a.bounds[i] = bounds6[i];
  int grid = (n + 127) / 128;
  if (maxl <= 2) k_fission_source<2><<<grid, 128, 0, s>>>(a);
  else k_fission_source<4><<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sg
