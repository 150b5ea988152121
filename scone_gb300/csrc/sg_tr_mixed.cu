// sg_tr_mixed.cu -- mixed form of the history loop: FP32 cross sections, distances and sampling,
// FP64 positions, coincidence tests and tally sums.
#include "sg_transport.cuh"
#include "sg_launch.h"

namespace sg {

template <>
int transport_grid<float>(int maxl, bool dt, size_t smem) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* f = maxl <= 2 ? (dt ? (const void*)k_transport<float, 2, true> : (const void*)k_transport<float, 2, false>)
                            : (dt ? (const void*)k_transport<float, 4, true> : (const void*)k_transport<float, 4, false>);
  if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, 128, smem);
  if (per < 1) per = 1;
  return sms * per;
}

template <>
cudaError_t launch_transport<float>(const TransportArgs<float>& a, int maxl, bool dt, size_t smem,
                                    cudaStream_t s, int* grid_out) {
  int grid = transport_grid<float>(maxl, dt, smem);
  if (grid_out) *grid_out = grid;
  if (maxl <= 2) {
    if (dt) k_transport<float, 2, true><<<grid, 128, smem, s>>>(a);
    else k_transport<float, 2, false><<<grid, 128, smem, s>>>(a);
  } else {
    if (dt) k_transport<float, 4, true><<<grid, 128, smem, s>>>(a);
    else k_transport<float, 4, false><<<grid, 128, smem, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace sg
