// sg_launch.h -- host-callable launch wrappers of the kernels (one definition per translation unit).
#pragma once
#include "sg_internal.h"

namespace sg {

// kernel kinds of the history loop and of the event form
enum { K_HISTORY = 0, K_EV_START = 1, K_EV_TRANSIT = 2, K_EV_COLLIDE = 3, K_EV_TAIL = 4, K_KINDS = 5 };

template <class R>
cudaError_t launch_kind(int kind, const TransportArgs<R>& a, int maxl, bool dt, size_t smem,
                        cudaStream_t s, int* grid_out);

// persistent history-loop kernel; maxl is the compile-time nesting bound (2 or 4)
template <class R>
cudaError_t launch_transport(const TransportArgs<R>& a, int maxl, bool dt, size_t smem,
                             cudaStream_t s, int* grid_out);

// the same kernels for continuous-energy data (neutronCEstd physics); defined in sg_tr_ce_*.cu
template <class R>
cudaError_t launch_kind_ce(int kind, const TransportArgs<R>& a, int maxl, bool dt, size_t smem,
                           cudaStream_t s, int* grid_out);

// fissionSource sampling on the device (fissionSource_class.f90:149-271), FP64 arithmetic
cudaError_t launch_fission_source(const DGeom& g, const DMG<double>& mg, DBank out, int n,
                                  unsigned long long master, const double* bounds6, int maxl,
                                  int* err, cudaStream_t s);

}  // namespace sg
