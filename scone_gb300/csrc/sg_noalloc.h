// sg_noalloc.h -- what sg_transport_bank_noalloc (sg_noalloc.cu) reads from a handle.
#pragma once
#include <string>
#include "sg_internal.h"

namespace sg {
struct NoAllocView {
  cudaStream_t stream;
  int precision, transport, maxl;
  std::string* err;
};
// Fills the view and the launch arguments shared by every call (geometry, data, clerks of `admin`
// and its attachment, score memory).  Allocates nothing.
int noalloc_view(sg_handle h, int admin, NoAllocView* v, TransportArgs<double>* t64, TransportArgs<float>* t32,
                 long long* lo);
}  // namespace sg
