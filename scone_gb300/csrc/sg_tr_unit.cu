// sg_tr_unit.cu -- one part of the transport kernels, chosen by the macros the build passes:
//   SG_R     float (mixed form: FP32 cross sections, distances and sampling; FP64 positions,
//            coincidence tests and tally sums) or double (FP64 verification form)
//   SG_CE    0 multigroup data (neutronMGstd / neutronMGimp), 1 continuous energy (neutronCEstd / CEimp)
//   SG_OP    OP_ST, OP_DT or OP_HT (transportOperatorST / DT / HT)
//   SG_PART  0 history loop, nesting bound 2; 1 event kernels, bound 2; 2 and 3 the same, bound 3;
//            4 and 5 the same, bound 4; 6, 7, 8 the lean history loop (multigroup only) for bounds
//            2, 3, 4
// Splitting each combination six ways keeps every translation unit small enough to compile in
// parallel in a minute or two.
#include <algorithm>
#include "sg_dispatch.cuh"

#if !defined(SG_R) || !defined(SG_CE) || !defined(SG_OP) || !defined(SG_PART)
#error "sg_tr_unit.cu needs SG_R, SG_CE, SG_OP and SG_PART"
#endif


#if SG_PART >= 6 && SG_CE
#error "the lean history loop (parts 6-8) is compiled for multigroup data only"
#endif

namespace sg {
template <>
cudaError_t launch_part<SG_R, (SG_CE != 0), SG_OP, SG_PART>(int kind, const TransportArgs<SG_R>& a, size_t smem,
                                                           cudaStream_t s, int* grid_out) {
#if SG_PART >= 6
  return launch_one<SG_R, SG_PART - 4, SG_OP, false, false, true>(kind, a, smem, s, grid_out);
#else
  return launch_one<SG_R, (SG_PART < 2 ? 2 : (SG_PART < 4 ? 3 : 4)), SG_OP, (SG_CE != 0), ((SG_PART & 1) != 0)>(kind, a, smem, s,
                                                                                        grid_out);
#endif
}
}  // namespace sg
