// sg_launch.h -- host-callable launch wrappers of the kernels.  The transport kernels of one
// (precision, data, operator) combination are compiled in six parts, each its own translation unit
// (sg_tr_unit.cu built with the SG_* macros): part 0 the history loop for nesting bound 2, part 1
// the event kernels for bound 2, parts 2 and 3 the same for bound 3, parts 4 and 5 for bound 4;
// multigroup data add parts 6, 7 and 8, the lean history loop for bounds 2, 3 and 4 (launches
// without rotated universes, cell maps, current clerks, neutronMGimp or P1 scattering: +21 % with
// delta tracking and +37 % with surface tracking on the 17x17 lattice, same GB300).
// A kernel compiled for the geometry's own nesting depth keeps fewer level arrays in registers and
// less unrolled code than one compiled for a deeper bound (3 instead of 4 levels measured 7 % faster
// on the lattice with delta tracking, 11 % with surface tracking).
#pragma once
#include "sg_internal.h"

namespace sg {

// kernel kinds of the history loop and of the event form
enum { K_HISTORY = 0, K_EV_START = 1, K_EV_TRANSIT = 2, K_EV_COLLIDE = 3, K_EV_TAIL = 4, K_KINDS = 5 };

// one part's launch (defined by that part's translation unit)
template <class R, bool CE, int OP, int PART>
cudaError_t launch_part(int kind, const TransportArgs<R>& a, size_t smem, cudaStream_t s, int* grid_out);

// launch of kernel `kind` for working precision R, data kind CE (continuous energy) and transport
// operator OP; maxl is the geometry's nesting bound (2, 3 or 4 compiled).  A multigroup history loop
// whose launch uses none of the optional features (a.lean) runs the lean instantiation, parts 6-8.
template <class R, bool CE, int OP>
inline cudaError_t launch_kind_op(int kind, const TransportArgs<R>& a, int maxl, size_t smem, cudaStream_t s,
                                  int* grid_out) {
  const bool ev = kind != K_HISTORY;
  if constexpr (!CE) {
    if (!ev && a.lean) {
      if (maxl <= 2) return launch_part<R, CE, OP, 6>(kind, a, smem, s, grid_out);
      if (maxl == 3) return launch_part<R, CE, OP, 7>(kind, a, smem, s, grid_out);
      return launch_part<R, CE, OP, 8>(kind, a, smem, s, grid_out);
    }
  }
  if (maxl <= 2)
    return ev ? launch_part<R, CE, OP, 1>(kind, a, smem, s, grid_out) : launch_part<R, CE, OP, 0>(kind, a, smem, s, grid_out);
  if (maxl == 3)
    return ev ? launch_part<R, CE, OP, 3>(kind, a, smem, s, grid_out) : launch_part<R, CE, OP, 2>(kind, a, smem, s, grid_out);
  return ev ? launch_part<R, CE, OP, 5>(kind, a, smem, s, grid_out) : launch_part<R, CE, OP, 4>(kind, a, smem, s, grid_out);
}

template <class R, bool CE>
inline cudaError_t launch_kind_data(int kind, const TransportArgs<R>& a, int maxl, int op, size_t smem,
                                    cudaStream_t s, int* grid_out) {
  if (op == OP_DT) return launch_kind_op<R, CE, OP_DT>(kind, a, maxl, smem, s, grid_out);
  if (op == OP_HT) return launch_kind_op<R, CE, OP_HT>(kind, a, maxl, smem, s, grid_out);
  return launch_kind_op<R, CE, OP_ST>(kind, a, maxl, smem, s, grid_out);
}

// multigroup data (neutronMGstd physics)
template <class R>
inline cudaError_t launch_kind(int kind, const TransportArgs<R>& a, int maxl, int op, size_t smem,
                               cudaStream_t s, int* grid_out) {
  return launch_kind_data<R, false>(kind, a, maxl, op, smem, s, grid_out);
}

// persistent history-loop kernel, multigroup data
template <class R>
inline cudaError_t launch_transport(const TransportArgs<R>& a, int maxl, int op, size_t smem,
                                    cudaStream_t s, int* grid_out) {
  return launch_kind_data<R, false>(K_HISTORY, a, maxl, op, smem, s, grid_out);
}

// continuous-energy data (neutronCEstd physics)
template <class R>
inline cudaError_t launch_kind_ce(int kind, const TransportArgs<R>& a, int maxl, int op, size_t smem,
                                  cudaStream_t s, int* grid_out) {
  return launch_kind_data<R, true>(kind, a, maxl, op, smem, s, grid_out);
}

// fissionSource sampling on the device (fissionSource_class.f90:149-271), FP64 arithmetic
cudaError_t launch_fission_source(const DGeom& g, const DMG<double>& mg, DBank out, int n,
                                  unsigned long long master, const double* bounds6, int maxl,
                                  int* err, cudaStream_t s);

struct FileSourceArgs;
// fileSource sampling on the device (fileSource_class.f90:146-190), FP64
cudaError_t launch_file_source(const FileSourceArgs& a, int maxl, cudaStream_t s);

}  // namespace sg
