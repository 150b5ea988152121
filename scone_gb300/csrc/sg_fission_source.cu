// sg_fission_source.cu -- fissionSource sampling on the device.  Built with -fmad=false: the
// initial eigenvalue bank is FP64 in both precision forms and matches the reference's rounding.
#include "sg_source.cuh"
#include "sg_launch.h"

namespace sg {

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

cudaError_t launch_file_source(const FileSourceArgs& a, int maxl, cudaStream_t s) {
  const int grid = (a.n + 127) / 128;
  if (maxl <= 2) k_file_source<2><<<grid, 128, 0, s>>>(a);
  else k_file_source<4><<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sg
