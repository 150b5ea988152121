// sg_dispatch.cuh -- launch of the history-loop or the event kernels for one precision, one kind of
// nuclear data, one transport operator and one nesting bound (included by sg_tr_unit.cu, which is
// compiled once per such part).
#pragma once
#include <mutex>
#include "sg_transport.cuh"
#include "sg_launch.h"

namespace sg {

// EV = false: the history-loop kernel (LEAN: its lean instantiation); EV = true: the event kernels
// (one part each)
template <class R, int MAXL, int OP, bool CE, bool EV, bool LEAN = false>
const void* kernel_ptr(int kind) {
  if constexpr (!EV) {
    (void)kind;
    return (const void*)k_transport<R, MAXL, OP, CE, LEAN>;
  } else {
    switch (kind) {
      case K_EV_START: return (const void*)k_ev_start<R, MAXL, OP, CE>;
      case K_EV_TRANSIT: return (const void*)k_ev_transit<R, MAXL, OP, CE, false>;
      case K_EV_COLLIDE: return (const void*)k_ev_collide<R, MAXL, OP, CE>;
      default: return (const void*)k_ev_transit<R, MAXL, OP, CE, true>;
    }
  }
}

// persistent grid: SM count x resident blocks of 128 threads (occupancy calculator); the cache is
// shared by every handle, so it is locked for callers that drive handles from several threads
template <class R, int MAXL, int OP, bool CE, bool EV, bool LEAN>
int persistent_grid(int kind, size_t smem) {
  static std::mutex mu;
  static int cached[K_KINDS] = {0};
  static size_t cached_smem = 0;
  std::lock_guard<std::mutex> lock(mu);
  if (kind == K_HISTORY && smem != cached_smem) { cached[K_HISTORY] = 0; cached_smem = smem; }
  if (!cached[kind]) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const void* f = kernel_ptr<R, MAXL, OP, CE, EV, LEAN>(kind);
    if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, 128, kind == K_HISTORY ? smem : 0);
    cached[kind] = sms * (per < 1 ? 1 : per);
  }
  return cached[kind];
}

template <class R, int MAXL, int OP, bool CE, bool EV, bool LEAN = false>
cudaError_t launch_one(int kind, const TransportArgs<R>& a, size_t smem, cudaStream_t s, int* grid_out) {
  if ((kind == K_HISTORY) == EV) return cudaErrorInvalidValue;     // the kind belongs to the other part
  int grid = persistent_grid<R, MAXL, OP, CE, EV, LEAN>(kind, smem);
  if (kind == K_EV_START) grid = std::max(1, std::min(grid * 4, (a.n + 127) / 128));
  if (grid_out) *grid_out = grid;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(kernel_ptr<R, MAXL, OP, CE, EV, LEAN>(kind), dim3(grid), dim3(128), args,
                          kind == K_HISTORY ? smem : 0, s);
}

}  // namespace sg
