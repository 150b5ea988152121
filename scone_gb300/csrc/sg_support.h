// sg_support.h -- launch wrappers of the per-cycle support kernels (sg_support.cu).
#pragma once
#include "sg_internal.h"

namespace sg {

struct PointSourceArgs {
  double r[3];
  double dir[3];
  int isotropic;
  int G;
  int n_prob_g;
  const double* prob_g;   // device
  double E;               // CE source energy (written when out.E is set)
  DBank out;
  int n;
  unsigned long long master;
};
cudaError_t launch_point_source(const PointSourceArgs& a, cudaStream_t s);

// exclusive scan of n int32 values; tmp needs scan_tmp_size(n) ints; *total gets the sum
cudaError_t exclusive_scan(const int* in, int n, int* out, int* tmp, int* total, cudaStream_t s);
int scan_tmp_size(int n);

cudaError_t launch_site_scatter(const DSites& src, const int* start, DBank out, int cap, int* err,
                                cudaStream_t s);

static constexpr int SUM_BLOCKS = 256;
// deterministic sum of n doubles; part needs SUM_BLOCKS doubles
cudaError_t deterministic_sum(const double* v, int n, double* part, double* out, cudaStream_t s);

// population control
__global__ void k_rn_keys(unsigned long long master, int S, unsigned long long* keys);
static constexpr int WIN_CAP = 16384;   // keys the window select of the heap threshold can gather
cudaError_t quantile_select(const unsigned long long* keys, int S, int kth, unsigned long long* sel, int* kbuf,
                            unsigned int* hist, unsigned long long* cnt, unsigned long long* cand, cudaStream_t s);
cudaError_t launch_flags(const unsigned long long* keys, int S, const unsigned long long* sel, int keep,
                         int* flags, cudaStream_t s);
cudaError_t launch_compact(const DBank& in, int S, const int* flags, const int* pos, const DBank& out,
                           cudaStream_t s);
cudaError_t launch_replicate(const DBank& in, int S, const int* flags, const int* dpos, const int* start,
                             int n_copies, const DBank& out, cudaStream_t s);
cudaError_t launch_brood_starts(const int* brood, int S, int nb, int* start, cudaStream_t s);

struct TallyCloseArgs {
  double* acc;
  double* bin;
  double* csum;
  double* csum2;
  long long N;
  int last_cycle;
  int close_batch;
  long long keff_analog;      // address (0-based, admin-relative) or -1
  long long keff_implicit;
  long long norm_addr;
  double norm_val;
  const double* end_weight;   // device scalar (popWeight of the end dungeon)
  const double* k_end;        // device scalar (end%k_eff)
  double* k_out;              // device scalar: keffResult mean, or null
  long long k_addr;           // address of the k estimate bin or -1
  int batchN;                 // batch count after this close
};
cudaError_t launch_tally_close(const TallyCloseArgs& a, cudaStream_t s);
cudaError_t add_scalar(double* p, const double* v, double c, cudaStream_t s);

}  // namespace sg
