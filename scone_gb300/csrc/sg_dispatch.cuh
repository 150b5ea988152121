// sg_dispatch.cuh -- launch of the history-loop and event kernels for one precision, one kind of
// nuclear data and one transport operator (included by the translation unit of that combination).
#pragma once
#include "sg_transport.cuh"
#include "sg_launch.h"

namespace sg {

template <class R, int MAXL, int OP, bool CE>
const void* kernel_ptr(int kind) {
  switch (kind) {
    case K_HISTORY: return (const void*)k_transport<R, MAXL, OP, CE>;
    case K_EV_START: return (const void*)k_ev_start<R, MAXL, OP, CE>;
    case K_EV_TRANSIT: return (const void*)k_ev_transit<R, MAXL, OP, CE, false>;
    case K_EV_COLLIDE: return (const void*)k_ev_collide<R, MAXL, OP, CE>;
    default: return (const void*)k_ev_transit<R, MAXL, OP, CE, true>;
  }
}

// persistent grid: SM count x resident blocks of 128 threads (occupancy calculator)
template <class R, int MAXL, int OP, bool CE>
int persistent_grid(int kind, size_t smem) {
  static int cached[K_KINDS] = {0};
  static size_t cached_smem = 0;
  if (kind == K_HISTORY && smem != cached_smem) { cached[K_HISTORY] = 0; cached_smem = smem; }
  if (!cached[kind]) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const void* f = kernel_ptr<R, MAXL, OP, CE>(kind);
    if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, 128, kind == K_HISTORY ? smem : 0);
    cached[kind] = sms * (per < 1 ? 1 : per);
  }
  return cached[kind];
}

template <class R, int MAXL, int OP, bool CE>
cudaError_t launch_one(int kind, const TransportArgs<R>& a, size_t smem, cudaStream_t s, int* grid_out) {
  int grid = persistent_grid<R, MAXL, OP, CE>(kind, smem);
  if (kind == K_EV_START) grid = std::max(1, std::min(grid * 4, (a.n + 127) / 128));
  if (grid_out) *grid_out = grid;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(kernel_ptr<R, MAXL, OP, CE>(kind), dim3(grid), dim3(128), args,
                          kind == K_HISTORY ? smem : 0, s);
}

// the body of one translation unit's launch_kind_op specialisation
template <class R, bool CE, int OP>
cudaError_t launch_unit(int kind, const TransportArgs<R>& a, int maxl, size_t smem, cudaStream_t s, int* grid_out) {
  if (maxl <= 2) return launch_one<R, 2, OP, CE>(kind, a, smem, s, grid_out);
  return launch_one<R, 4, OP, CE>(kind, a, smem, s, grid_out);
}

}  // namespace sg
