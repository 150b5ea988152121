// sg_tr_fp64.cu -- all-FP64 verification form of the history loop.  Built with -fmad=false so the
// arithmetic rounds exactly as SCONE's (no fused multiply-add anywhere in this translation unit).
#include "sg_transport.cuh"
#include "sg_launch.h"
#include "sg_source.cuh"

namespace sg {

template <>
int transport_grid<double>(int maxl, bool dt, size_t smem) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* f = maxl <= 2 ? (dt ? (const void*)k_transport<double, 2, true> : (const void*)k_transport<double, 2, false>)
                            : (dt ? (const void*)k_transport<double, 4, true> : (const void*)k_transport<double, 4, false>);
  if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, 128, smem);
  if (per < 1) per = 1;
  return sms * per;
}

template <>
cudaError_t launch_transport<double>(const TransportArgs<double>& a, int maxl, bool dt, size_t smem,
                                     cudaStream_t s, int* grid_out) {
  int grid = transport_grid<double>(maxl, dt, smem);
  if (grid_out) *grid_out = grid;
  if (maxl <= 2) {
    if (dt) k_transport<double, 2, true><<<grid, 128, smem, s>>>(a);
    else k_transport<double, 2, false><<<grid, 128, smem, s>>>(a);
  } else {
    if (dt) k_transport<double, 4, true><<<grid, 128, smem, s>>>(a);
    else k_transport<double, 4, false><<<grid, 128, smem, s>>>(a);
  }
  return cudaGetLastError();
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
