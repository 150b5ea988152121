// sg_batch.cuh -- the batched form of the gen loop: every cycle of many independent fixed-source
// problems transported by one persistent launch, fed from a device work queue.
//
// SCONE runs one problem per process: fixedSourcePhysicsPackage%cycles generates the source, runs
// the `gen:` loop and closes the tallies, cycle after cycle (fixedSourcePhysicsPackage_class.f90:
// 183-289).  Here the cycles of all problems are flattened into one history space per problem
// (f = c * pop + n - 1) and cut into work items; warps take items from a global queue.  A warp works
// on one problem at a time: the problem's record (geometry, MG data, clerks) sits in the warp's slot
// of shared memory, and lanes that end a history take the next history of the same item at once.
// The warp moves to an item of another problem only when all of its lanes are idle.
//
// Each history follows the single-problem path: pointSource sampling with master_c + stride(n)
// (source_inter.f90:98-119, pointSource_class.f90:189-270), then transport with master_c +
// stride(pop + n), where master_c is the problem's master strided by 2 * pop per cycle
// (fixedSourcePhysicsPackage_class.f90:186-189,264).  In the FP64 form every draw and result is
// the single-problem path's; the mixed form samples the source direction in FP32.  Scores of cycle
// c go to that cycle's own accumulator; the cycles are closed in order after the launch.
#pragma once
#include "sg_transport.cuh"
#include "sg_batch.h"

namespace sg {

static constexpr int BATCH_MAX_WARPS = 4;   // __launch_bounds__(128)

// The record of a problem into the warp's shared slot by one bulk asynchronous copy (the copy
// engine moves the ~3 KB record while the warp waits on its mbarrier); counters and errors then go
// to this launch's.  Returns false if the copy did not complete within the bounded wait (after a
// second bounded wait for the copy in flight): the warp must stop.
template <class R>
__device__ __forceinline__ bool stage_problem_warp(BatchProblem<R>* dst, const BatchProblem<R>* src, int lane,
                                                   DCounters* ctr, unsigned long long* bar, unsigned& phase) {
  static_assert(sizeof(BatchProblem<R>) % 16 == 0, "record size");
  __syncwarp();                                        // the previous record is no longer read
  if (lane == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect(bar, (unsigned)sizeof(BatchProblem<R>));
    bulk_to_smem(dst, src, (unsigned)sizeof(BatchProblem<R>), bar);
  }
  const bool ok = __all_sync(FULL, mbar_wait(bar, phase));
  if (!ok) {
    (void)mbar_wait(bar, phase);
    return false;
  }
  phase ^= 1u;
  if (lane == 0) dst->t.ctr = ctr;
  __syncwarp();
  return true;
}

// pointSource%sampleParticle (pointSource_class.f90:189-270), then the particle enters the gen loop
// as thisCycle%copy + placeCoord would leave it.
// s_src / s_tr: the source and transport RNG states of this history, master_c + stride(n) and
// master_c + stride(pop + n)
template <class R, int MAXL, int OP, bool LEAN>
__device__ __forceinline__ void start_batched(Tracker<R, MAXL, OP, false, LEAN>& T, const BatchProblem<R>& P, int f,
                                              unsigned long long s_src, unsigned long long s_tr) {
  const int c = f / P.pop;
  const int n = f - c * P.pop + 1;
  // the source direction in the working precision: FP64 as SCONE in the verification form; FP32
  // in the mixed form (the direction is kept in FP32 there, and FP64 is scarce on this GPU)
  Rng<R> rs;
  rs.s = s_src;
  R d0 = (R)P.src_dir[0], d1 = (R)P.src_dir[1], d2 = (R)P.src_dir[2];
  if (P.src_isotropic) {
    const R mu = R(2) * rs.get() - R(1);
    R sp, cp;
    sincos_phi<R>(rs.get(), sp, cp);
    d0 = R(1); d1 = R(0); d2 = R(0);
    rotate_vector<R>(d0, d1, d2, mu, sp, cp);
  }
  int g = P.src_G;
  if (P.src_n_prob_g > 0) {
    R r = rs.get();
    for (g = 1; g <= P.src_n_prob_g; ++g) {
      r = r - (R)P.src_prob_g[g - 1];
      if (r < R(0)) break;
    }
  }
  T.hist = n;
  T.c.r0[0] = P.src_r[0];
  T.c.r0[1] = P.src_r[1];
  T.c.r0[2] = P.src_r[2];
  T.c.u[0] = d0;
  T.c.u[1] = d1;
  T.c.u[2] = d2;
  T.w = R(1);
  T.w0 = R(1);
  T.G = g;
  T.time = R(0);
  T.rng.s = s_tr;
  T.collN = 0;
  T.nsites = 0;
  T.segs = 0;
  T.cache.lvl = 0;
  T.onSurf = false;
  T.acc = P.t.acc + (long long)c * P.n_bins;
  if (!T.geom.place(T.c, false)) raise_error(P.t.ctr, SG_ERR_UNDEF_MAT, n);
  T.select_ht();
}

// LEAN: every problem of the launch runs without rotated universes, cell maps, current clerks or P1
// scattering (BatchLaunch::lean), so the lean Tracker is compiled
template <class R, int MAXL, int OP, bool LEAN = false>
__global__ void __launch_bounds__(128, (batch_min_blocks<R, OP>())) k_batch(const __grid_constant__ BatchLaunch L) {
  __shared__ __align__(16) unsigned char s_rec[BATCH_MAX_WARPS][sizeof(BatchProblem<R>)];
  __shared__ __align__(8) unsigned long long s_bar[BATCH_MAX_WARPS];
  __shared__ RngJump s_jump;
  rng_jump_table(s_jump);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  BatchProblem<R>& P = *reinterpret_cast<BatchProblem<R>*>(s_rec[threadIdx.x >> 5]);
  unsigned long long* bar = &s_bar[threadIdx.x >> 5];
  unsigned phase = 0;
  if (lane == 0) mbar_init(bar);
  const BatchProblem<R>* probs = static_cast<const BatchProblem<R>*>(L.problems);
  if (lane == 0) {                  // a neutral record until the first item is staged
    P.t.k_eff = L.k_one;
    P.t.ctr = L.ctr;
    P.t.keff_clerk = -1;
    P.t.n_clerks = 0;
    P.t.acc = nullptr;
  }
  __syncwarp();
  Tracker<R, MAXL, OP, false, LEAN> T(P.t, nullptr);
  const int nItems = *L.n_items;
  int cur = -1;                     // slot of the staged problem (warp-uniform)
  int pend = -1;                    // claimed item of another problem, waiting for the warp to drain
  int q_next = 0, q_end = 0;        // warp-uniform range of flat histories of the current item
  // the chunk being started: at most 32 histories of one cycle of the item, from flat history
  // ch_base, whose source and transport RNG states are s_src / s_tr (warp-uniform)
  int ch_base = 0, ch_end = 0;
  unsigned long long s_src = 0, s_tr = 0;
  bool alive = false, done = false;
  bool stopped = false;             // warp-uniform: a record copy timed out

  while (true) {
    unsigned need = __ballot_sync(FULL, !alive && !done);
    while (need) {
      if (q_next >= q_end) {
        int it = pend;
        if (it < 0) {
          int b = 0;
          if (lane == 0) b = atomicAdd(L.head, 1);
          it = __shfl_sync(FULL, b, 0);
          if (it >= nItems) {
            if (!alive) done = true;
            break;
          }
        }
        const WorkItem wi = L.items[it];
        if (wi.slot != cur) {
          if (__any_sync(FULL, alive)) { pend = it; break; }
          if (!stage_problem_warp<R>(&P, probs + wi.slot, lane, L.ctr, bar, phase)) {
            if (lane == 0) raise_error(L.ctr, SG_ERR_TIMEOUT, wi.first + 1);
            done = true;                               // no lane is alive here: the warp stops
            stopped = true;
            break;
          }
          cur = wi.slot;
        }
        pend = -1;
        q_next = wi.first;
        q_end = wi.first + wi.count;
        ch_end = q_next;
      }
      if (q_next >= ch_end) {                         // a new chunk: one skip for the warp
        const int c = q_next / P.pop;
        const int n = q_next - c * P.pop + 1;
        ch_base = q_next;
        ch_end = min(min(q_next + 32, q_end), (c + 1) * P.pop);
        s_src = lcg_skip(P.master, RNG_STRIDE * (2LL * P.pop * c + n));
        s_tr = lcg_skip(s_src, RNG_STRIDE * (long long)P.pop);
      }
      const int avail = ch_end - q_next;
      const int rank = __popc(need & ((1u << lane) - 1u));
      const bool mine = ((need >> lane) & 1u) && rank < avail;
      if (mine) {
        const int off = q_next + rank - ch_base;
        start_batched<R, MAXL, OP>(T, P, q_next + rank, rng_jump(s_jump, off, s_src), rng_jump(s_jump, off, s_tr));
        alive = true;
      }
      q_next += min(__popc(need), avail);
      need &= ~__ballot_sync(FULL, mine);
    }
    if (stopped) break;
    if (__all_sync(FULL, !alive)) {
      if (__all_sync(FULL, done)) break;
      continue;
    }
    // flight and collision in one branch: deferring collisions measured 2 % slower on the uneven
    // batch, and a warp vote between flight and collision (as k_transport has) no faster
    if (alive) {
      if (T.step()) { T.finish(); alive = false; }
    }
  }
  if (stopped) {                    // the record slot may hold a partial copy: count into this launch
    if (lane == 0) { P.t.ctr = L.ctr; P.t.keff_clerk = -1; }
    __syncwarp();
  }
  flush_counters(T, P.t, lane);
}

}  // namespace sg

namespace sg {

template <class R, int OP>
const void* batch_kernel_ptr(int maxl, bool lean) {
  if (lean) return maxl <= 2 ? (const void*)k_batch<R, 2, OP, true> : (const void*)k_batch<R, 4, OP, true>;
  return maxl <= 2 ? (const void*)k_batch<R, 2, OP> : (const void*)k_batch<R, 4, OP>;
}

// the bodies of one translation unit's launch_batch_op / batch_occupancy_op specialisations
template <class R, int OP>
cudaError_t launch_batch_unit(const BatchLaunch& L, int grid, int block, cudaStream_t s) {
  if (block < 32 || block > 32 * BATCH_MAX_WARPS || block % 32) return cudaErrorInvalidValue;
  void* args[] = {(void*)&L};
  return cudaLaunchKernel(batch_kernel_ptr<R, OP>(L.maxl, L.lean != 0), dim3(grid), dim3(block), args, 0, s);
}

template <class R, int OP>
int batch_occupancy_unit(int maxl, bool lean, int block) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_kernel_ptr<R, OP>(maxl, lean), block, 0) != cudaSuccess)
    return 1;
  return per < 1 ? 1 : per;
}

}  // namespace sg
