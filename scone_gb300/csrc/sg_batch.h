// sg_batch.h -- records of the batched form: many independent fixed-source problems, each with its
// own geometry, MG data, point source, tallies and RNG seed, transported by one persistent launch.
#pragma once
#include <string>
#include <vector>
#include "sg_internal.h"

namespace sg {

// One resident problem as the batched kernel reads it.  A warp copies the record of the problem it
// works on into shared memory, so every lane of the warp sees the same geometry, data and clerks.
// `t.acc` is the score memory of cycle 1; cycle c (0-based) scores at t.acc + c * n_bins.
template <class R>
struct __align__(16) BatchProblem {
  TransportArgs<R> t;
  double src_r[3];
  double src_dir[3];
  const double* src_prob_g;     // pointSource group CDF (device), or null
  int src_isotropic;
  int src_G;
  int src_n_prob_g;
  int pop;                      // histories per cycle (fixedSource `pop`)
  int cycles;
  int maxl;
  unsigned long long master;    // RNG state at the start of cycle 1
  long long n_bins;             // score memory of one cycle
};

// A contiguous run of one problem's histories in flat order: flat index f = c * pop + (n - 1) for
// history n of cycle c.
struct WorkItem {
  int slot;
  int first;
  int count;
  int pad;
};

// Score memory of one problem: acc[cycles][n] (one accumulator per cycle), then SCONE's
// bins(n, {BIN, CSUM, CSUM2}) (scoreMemory_class.f90:16-18,87-97).
struct BatchTally {
  double* acc;
  double* bin;
  double* csum;
  double* csum2;
  long long n;
  long long norm_addr;          // 0-based, or -1
  double norm_val;
  int cycles;
  int pad;
};

struct BatchLaunch {
  const void* problems;         // BatchProblem<R>[slots]
  const WorkItem* items;
  const int* n_items;           // device count, read at launch (graph replays see the new value)
  int* head;                    // next work item
  DCounters* ctr;
  const double* k_one;          // 1.0: the k of fixed-source collisions
  int maxl;
  int lean;                     // 1: every problem of the launch can run the lean history loop
};

// the batched kernel for precision R and transport operator OP (one translation unit each)
template <class R, int OP>
cudaError_t launch_batch_op(const BatchLaunch& L, int grid, int block, cudaStream_t s);
template <class R, int OP>
int batch_occupancy_op(int maxl, int lean, int block);

template <class R>
inline cudaError_t launch_batch(const BatchLaunch& L, int op, int grid, int block, cudaStream_t s) {
  if (op == OP_DT) return launch_batch_op<R, OP_DT>(L, grid, block, s);
  if (op == OP_HT) return launch_batch_op<R, OP_HT>(L, grid, block, s);
  return launch_batch_op<R, OP_ST>(L, grid, block, s);
}
template <class R>
inline int batch_occupancy(int maxl, int lean, int op, int block) {
  if (op == OP_DT) return batch_occupancy_op<R, OP_DT>(maxl, lean, block);
  if (op == OP_HT) return batch_occupancy_op<R, OP_HT>(maxl, lean, block);
  return batch_occupancy_op<R, OP_ST>(maxl, lean, block);
}

// scoreMemory%closeCycle for every cycle of the listed problems, in cycle order (sg_batch_host.cu)
cudaError_t launch_batch_close(const BatchTally* tallies, const int* slots, const int* n, int grid, cudaStream_t s);

// ---- bridges into the single-problem host code (sg_host.cu)

// Host image of one problem's resident data as the batched form lays it out: geometry, MG data
// (both precisions), the group CDF of the source and the clerk table, with device pointers into
// the block that starts at `dev` (null: only count the bytes into *bytes).
struct StagedProblem {
  TransportArgs<double> t64;
  TransportArgs<float> t32;
  int maxl;
  long long n_bins;
  long long norm_addr;
  double norm_val;
  const double* prob_g;
  bool any_fissile;
  std::vector<sg_clerk_desc> clerks;   // the admin's clerks and their 1-based addresses
  std::vector<long long> addr;
  std::vector<const void*> tab64, tab32;   // map tables in the problem's block, [3 * clerk + axis]
};
int stage_problem(const sg_geometry_desc* g, const sg_mg_desc* mg, const sg_point_source_desc* src,
                  const sg_tally_desc* tally, char* dev, std::vector<char>* host, size_t cap, size_t* bytes,
                  StagedProblem* out, std::string* err);

// The plain form: `cycles` calls of sg_fixed_source_cycle on the work handle `h` (its own form,
// event or history loop) with the staged problem bound in place of the handle's own geometry, data,
// source and tally admin; the score memory is the problem's (acc of cycle 1, bin, csum, csum2).
// The handle's own state is restored afterwards.  `st` receives the summed statistics.
int plain_fixed_source(sg_handle h, const StagedProblem& p, const sg_point_source_desc* src, double* acc,
                       double* bin, double* csum, double* csum2, int pop, int cycles,
                       unsigned long long master, sg_cycle_stats* st);

}  // namespace sg
