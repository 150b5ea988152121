// sg_support.cu -- the per-cycle kernels around the history loop: point-source sampling, ordering of
// fission sites by brood ID, population control (normSize_Repr), deterministic reductions and the
// scoreMemory/tallyAdmin cycle-end update.  All are bandwidth- or latency-trivial next to the
// history loop; they exist so that a whole eigenvalue cycle stays on the device.
#include <atomic>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include "sg_device.cuh"
#include "sg_support.h"

namespace sg {

// ------------------------------------------------------------------ pointSource (pointSource_class.f90:189-270)
__global__ void k_point_source(PointSourceArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  Rng<double> rng;
  rng.s = lcg_skip(a.master, RNG_STRIDE * (long long)(i + 1));   // source_inter.f90:113-114
  double d0 = a.dir[0], d1 = a.dir[1], d2 = a.dir[2];
  if (a.isotropic) {
    double mu = 2.0 * rng.get() - 1.0;
    double sp, cp;
    sincos_phi<double>(rng.get(), sp, cp);
    d0 = 1.0; d1 = 0.0; d2 = 0.0;
    rotate_vector<double>(d0, d1, d2, mu, sp, cp);
  }
  int g = a.G;
  if (a.n_prob_g > 0) {
    double r = rng.get();
    for (g = 1; g <= a.n_prob_g; ++g) {
      r = r - a.prob_g[g - 1];
      if (r < 0.0) break;
    }
  }
  a.out.r[3 * i + 0] = a.r[0]; a.out.r[3 * i + 1] = a.r[1]; a.out.r[3 * i + 2] = a.r[2];
  a.out.dir[3 * i + 0] = d0; a.out.dir[3 * i + 1] = d1; a.out.dir[3 * i + 2] = d2;
  a.out.wgt[i] = 1.0;
  a.out.G[i] = g;
  a.out.brood[i] = 0;
  a.out.time[i] = 0.0;
  if (a.out.E) a.out.E[i] = a.E;                                  // pointSource `E` (CE)
}

cudaError_t launch_point_source(const PointSourceArgs& a, cudaStream_t s) {
  k_point_source<<<(a.n + 255) / 256, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ exclusive scan of int32 (3 passes)
static constexpr int SCAN_CHUNK = 2048;   // elements per block (256 threads x 8)

__global__ void k_scan_reduce(const int* in, int n, int* block_sums) {
  __shared__ int s[256];
  const int base = blockIdx.x * SCAN_CHUNK;
  int v = 0;
  for (int k = threadIdx.x; k < SCAN_CHUNK; k += 256) {
    int i = base + k;
    if (i < n) v += in[i];
  }
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = s[0];
}

__global__ void k_scan_blocks(int* block_sums, int nb, int* total) {
  // single block, sequential chunks of 1024 with a running carry
  __shared__ int s[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    int i = base + threadIdx.x;
    int v = (i < nb) ? block_sums[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      int t = (threadIdx.x >= o) ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) block_sums[i] = carry + s[threadIdx.x] - v;   // exclusive
    __syncthreads();
    if (threadIdx.x == 1023) carry += s[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_apply(const int* in, int n, const int* block_off, int* out) {
  __shared__ int s[256];
  const int base = blockIdx.x * SCAN_CHUNK;
  // each thread owns 8 consecutive elements
  int v[8];
  int sum = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    int i = base + threadIdx.x * 8 + k;
    v[k] = (i < n) ? in[i] : 0;
    sum += v[k];
  }
  s[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    int t = (threadIdx.x >= o) ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  int run = block_off[blockIdx.x] + s[threadIdx.x] - sum;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    int i = base + threadIdx.x * 8 + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

cudaError_t exclusive_scan(const int* in, int n, int* out, int* tmp, int* total, cudaStream_t s) {
  int nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if (nb < 1) nb = 1;
  k_scan_reduce<<<nb, 256, 0, s>>>(in, n, tmp);
  k_scan_blocks<<<1, 1024, 0, s>>>(tmp, nb, total);
  k_scan_apply<<<nb, 256, 0, s>>>(in, n, tmp, out);
  return cudaGetLastError();
}
int scan_tmp_size(int n) { return (n + SCAN_CHUNK - 1) / SCAN_CHUNK + 1; }

// ------------------------------------------------------------------ fission sites -> ordered bank
// Site (brood b, seq q) goes to start[b-1] + q: the order particleDungeon%sortByBroodID produces
// (particleDungeon_class.f90:923-981), independent of the order the sites were appended.
__global__ void k_site_scatter(DSites src, const int* start, DBank out, int cap, int* err) {
  const int region = blockIdx.y;
  const int cnt = min(src.cursor[region], src.region_cap);
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < cnt; slot += gridDim.x * blockDim.x) {
    long long i = (long long)region * src.region_cap + slot;
    int b = src.brood[i];
    int dst = start[b - 1] + src.seq[i];
    if (dst >= cap) { atomicCAS(err, 0, SG_ERR_BANK_OVERFLOW); continue; }
    out.r[3 * dst + 0] = src.r[3 * i + 0];
    out.r[3 * dst + 1] = src.r[3 * i + 1];
    out.r[3 * dst + 2] = src.r[3 * i + 2];
    out.dir[3 * dst + 0] = src.dir[3 * i + 0];
    out.dir[3 * dst + 1] = src.dir[3 * i + 1];
    out.dir[3 * dst + 2] = src.dir[3 * i + 2];
    out.wgt[dst] = src.wgt[i];
    out.G[dst] = src.G[i];
    out.brood[dst] = b;
    out.time[dst] = src.time[i];
  }
}

cudaError_t launch_site_scatter(const DSites& src, const int* start, DBank out, int cap, int* err,
                                cudaStream_t s) {
  dim3 grid(64, SITE_REGIONS);
  k_site_scatter<<<grid, 256, 0, s>>>(src, start, out, cap, err);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ deterministic sum of doubles
// Fixed block decomposition and fixed tree order, so the result does not depend on scheduling.
__global__ void k_sum_partial(const double* v, int n, double* part) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) acc += v[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
__global__ void k_sum_final(const double* part, int nb, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.0;
    for (int i = 0; i < nb; ++i) a += part[i];
    *out = a;
  }
}
cudaError_t deterministic_sum(const double* v, int n, double* part, double* out, cudaStream_t s) {
  k_sum_partial<<<SUM_BLOCKS, 256, 0, s>>>(v, n, part);
  k_sum_final<<<1, 32, 0, s>>>(part, SUM_BLOCKS, out);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ normSize_Repr (particleDungeon_class.f90:431-605)
// Keys: the bit pattern of xi_j, j = 1..S, drawn in sequence from the master stream.  Positive
// doubles order like their bit patterns, so the heap threshold (the heapSize-th smallest xi) is a
// 64-bit radix select.
__global__ void k_rn_keys(unsigned long long master, int S, unsigned long long* keys) {
  const int CH = 32;
  const int first = (blockIdx.x * blockDim.x + threadIdx.x) * CH;
  if (first >= S) return;
  uint64_t s = lcg_skip(master, first);
  for (int j = first; j < min(first + CH, S); ++j) {
    s = lcg_next(s);
    double xi = __ll2double_rn((long long)s) * 0x1p-63;
    keys[j] = (unsigned long long)__double_as_longlong(xi);
  }
}

// The heap threshold is first looked for in a window around its expected place: the xi are
// uniform on (0,1), so the kth smallest of S lies within a few standard deviations
// (sqrt(p (1 - p) / S), p = k / S) of k / S.  One pass counts the keys below the window and gathers
// the keys inside it; one block sorts the gathered keys and picks the kth.  The result is the kth
// smallest key itself, whichever way it is found.  When the window misses (the kth key outside it,
// or more keys in it than the buffer holds) the radix select below runs; its kernels return at
// once when the window found the key (ok flag).
__global__ void k_win_gather(const unsigned long long* keys, int S, unsigned long long lo, unsigned long long hi,
                             unsigned long long* cnt, unsigned long long* cand, int cap) {
  __shared__ unsigned long long below_s;
  if (threadIdx.x == 0) below_s = 0;
  __syncthreads();
  unsigned long long below = 0;
  const int lane = threadIdx.x & 31;
  for (int base = blockIdx.x * blockDim.x; base < S; base += gridDim.x * blockDim.x) {
    const int i = base + threadIdx.x;
    unsigned long long k = 0;
    bool in = false;
    if (i < S) {
      k = keys[i];
      below += (k < lo) ? 1 : 0;
      in = (k >= lo && k <= hi);
    }
    const unsigned m = __ballot_sync(0xffffffffu, in);
    if (m) {
      unsigned long long pos = 0;
      if (lane == 0) pos = atomicAdd(cnt + 1, (unsigned long long)__popc(m));
      pos = __shfl_sync(0xffffffffu, pos, 0);
      if (in) {
        const unsigned long long at = pos + __popc(m & ((1u << lane) - 1u));
        if (at < (unsigned long long)cap) cand[at] = k;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) below += __shfl_down_sync(0xffffffffu, below, o);
  if (lane == 0 && below) atomicAdd(&below_s, below);
  __syncthreads();
  if (threadIdx.x == 0 && below_s) atomicAdd(cnt, below_s);
}

// one block: bitonic sort of the gathered keys in shared memory, then the pick.  ok[0] = 1 on
// success; otherwise the radix select's state (sel = 0, kth) is set up.
__global__ void k_win_pick(const unsigned long long* cand, const unsigned long long* cnt, int cap, int kth,
                           unsigned long long* sel, int* kbuf) {
  extern __shared__ unsigned long long sk[];
  const unsigned long long nb = cnt[0], nin = cnt[1];
  const long long r = (long long)kth - (long long)nb;     // 1-based rank inside the window
  const bool hit = r >= 1 && (unsigned long long)r <= nin && nin <= (unsigned long long)cap;
  if (!hit) {
    if (threadIdx.x == 0) { sel[0] = 0; sel[1] = 0; kbuf[0] = kth; kbuf[1] = 0; }
    return;
  }
  int P = 1;
  while (P < (int)nin) P <<= 1;
  for (int i = threadIdx.x; i < P; i += blockDim.x) sk[i] = (i < (int)nin) ? cand[i] : ~0ull;
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = sk[i], b = sk[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) { sk[i] = b; sk[l] = a; }
        }
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) { sel[0] = sk[r - 1]; sel[1] = ~0ull; kbuf[0] = 1; kbuf[1] = 1; }
}

__global__ void k_radix_hist(const unsigned long long* keys, int S, const unsigned long long* sel,
                             int shift, unsigned int* hist, const int* ok) {
  if (*ok) return;
  // sel[0] = prefix, sel[1] = mask of the bits already fixed
  const unsigned long long prefix = sel[0], mask = sel[1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x) {
    unsigned long long k = keys[i];
    if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 0xFFFFu], 1u);
  }
}

__global__ void k_radix_pick(unsigned int* hist, unsigned long long* sel, int* kth, int shift) {
  // single block of 1024: find the digit containing the kth (1-based) key, then clear hist
  if (kth[1]) return;                                    // the window select found it
  __shared__ unsigned int part[1024];
  __shared__ int chosen;
  __shared__ unsigned int below;
  const int t = threadIdx.x;
  unsigned int sum = 0;
  for (int d = t * 64; d < t * 64 + 64; ++d) sum += hist[d];
  part[t] = sum;
  __syncthreads();
  if (t == 0) {
    unsigned int run = 0;
    int k = *kth;
    int c = 0;
    for (c = 0; c < 1024; ++c) {
      if (run + part[c] >= (unsigned int)k) break;
      run += part[c];
    }
    unsigned int r2 = run;
    int d;
    for (d = c * 64; d < c * 64 + 64; ++d) {
      if (r2 + hist[d] >= (unsigned int)k) break;
      r2 += hist[d];
    }
    chosen = d;
    below = r2;
  }
  __syncthreads();
  for (int d = t; d < 65536; d += 1024) hist[d] = 0;
  if (t == 0) {
    sel[0] |= ((unsigned long long)chosen) << shift;
    sel[1] |= 0xFFFFull << shift;
    *kth = *kth - (int)below;
  }
}

// kth smallest (1-based) of the S keys into sel[0].  hist (65536 counters) is zero on entry and on
// exit; kbuf holds [kth remaining, window found]; cnt two counters; cand WIN_CAP keys.
cudaError_t quantile_select(const unsigned long long* keys, int S, int kth, unsigned long long* sel, int* kbuf,
                            unsigned int* hist, unsigned long long* cnt, unsigned long long* cand, cudaStream_t s) {
  static std::atomic<int> attrDevice{-1};         // the attribute is set once per device
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev != attrDevice.load()) {
    e = cudaFuncSetAttribute(k_win_pick, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(WIN_CAP * sizeof(unsigned long long)));
    if (e != cudaSuccess) return e;
    attrDevice.store(dev);
  }
  const double p = (double)kth / S;
  const double d = 8.0 * sqrt(p * (1.0 - p) / S) + 4.0 / S;
  const double lo = p - d, hi = p + d;
  unsigned long long klo = 0, khi = ~0ull >> 1;
  if (lo > 0.0) std::memcpy(&klo, &lo, sizeof(double));
  if (hi < 1.0) std::memcpy(&khi, &hi, sizeof(double));
  const char* off = std::getenv("SCONE_GB300_NO_WINDOW_SELECT");   // empty window: radix select only
  if (off && off[0] == '1') { klo = 1; khi = 0; }
  cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), s);
  const int blocks = std::min(1216, (S + 255) / 256);
  k_win_gather<<<blocks, 256, 0, s>>>(keys, S, klo, khi, cnt, cand, WIN_CAP);
  k_win_pick<<<1, 1024, WIN_CAP * sizeof(unsigned long long), s>>>(cand, cnt, WIN_CAP, kth, sel, kbuf);
  for (int shift = 48; shift >= 0; shift -= 16) {
    k_radix_hist<<<256, 256, 0, s>>>(keys, S, sel, shift, hist, kbuf + 1);
    k_radix_pick<<<1, 1024, 0, s>>>(hist, sel, kbuf, shift);
  }
  return cudaGetLastError();
}

// keep flags (excess > 0: xi > threshold) or duplicate flags (excess < 0: xi <= threshold)
__global__ void k_flags(const unsigned long long* keys, int S, const unsigned long long* sel, int keep_mode,
                        int* flags) {
  const unsigned long long thr = sel[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x) {
    double xi = __longlong_as_double((long long)keys[i]);
    double th = __longlong_as_double((long long)thr);
    flags[i] = keep_mode ? (xi > th) : (xi <= th);
  }
}

__device__ __forceinline__ void copy_particle(const DBank& a, int i, DBank& b, int j) {
  b.r[3 * j + 0] = a.r[3 * i + 0]; b.r[3 * j + 1] = a.r[3 * i + 1]; b.r[3 * j + 2] = a.r[3 * i + 2];
  b.dir[3 * j + 0] = a.dir[3 * i + 0]; b.dir[3 * j + 1] = a.dir[3 * i + 1]; b.dir[3 * j + 2] = a.dir[3 * i + 2];
  b.wgt[j] = a.wgt[i];
  b.G[j] = a.G[i];
  b.brood[j] = a.brood[i];
  b.time[j] = a.time[i];
}

// excess > 0: stable compaction of the kept sites
__global__ void k_compact(DBank in, int S, const int* flags, const int* pos, DBank out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x)
    if (flags[i]) copy_particle(in, i, out, pos[i]);
}

// excess < 0: n_copies full copies plus duplicates, written straight into brood-sorted order
__global__ void k_replicate(DBank in, int S, const int* flags, const int* dpos, const int* start,
                            int n_copies, DBank out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x) {
    int b = in.brood[i];
    int bs = start[b - 1];
    int cnt = start[b] - bs;
    int base = (n_copies + 1) * bs + dpos[bs];
    for (int t = 0; t <= n_copies; ++t) copy_particle(in, i, out, base + t * cnt + (i - bs));
    if (flags[i]) copy_particle(in, i, out, base + (n_copies + 1) * cnt + (dpos[i] - dpos[bs]));
  }
}

cudaError_t launch_flags(const unsigned long long* keys, int S, const unsigned long long* sel, int keep,
                         int* flags, cudaStream_t s) {
  k_flags<<<(S + 255) / 256, 256, 0, s>>>(keys, S, sel, keep, flags);
  return cudaGetLastError();
}
cudaError_t launch_compact(const DBank& in, int S, const int* flags, const int* pos, const DBank& out,
                           cudaStream_t s) {
  k_compact<<<(S + 255) / 256, 256, 0, s>>>(in, S, flags, pos, out);
  return cudaGetLastError();
}
cudaError_t launch_replicate(const DBank& in, int S, const int* flags, const int* dpos, const int* start,
                             int n_copies, const DBank& out, cudaStream_t s) {
  k_replicate<<<(S + 255) / 256, 256, 0, s>>>(in, S, flags, dpos, start, n_copies, out);
  return cudaGetLastError();
}

// The brood offsets k_replicate reads, for a bank sorted by brood that did not come from this
// handle's gen loop: start[b] = the first index whose brood exceeds b, b = 0..nb (a lower-bound
// search per entry).
__global__ void k_brood_starts(const int* brood, int S, int nb, int* start) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b <= nb; b += gridDim.x * blockDim.x) {
    int lo = 0, hi = S;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (brood[mid] <= b) lo = mid + 1;
      else hi = mid;
    }
    start[b] = lo;
  }
}
cudaError_t launch_brood_starts(const int* brood, int S, int nb, int* start, cudaStream_t s) {
  k_brood_starts<<<(nb + 1 + 255) / 256, 256, 0, s>>>(brood, S, nb, start);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ scoreMemory / tallyAdmin cycle end
// Order of tallyAdmin%reportCycleEnd (tallyAdmin_class.f90:721-788) for one admin: clerk
// reportCycleEnd (keffAnalog END_POP), mem%reduceBins, clerk closeCycle (k estimators),
// normalisation, mem%closeCycle.
__global__ void k_tally_close(TallyCloseArgs a) {
  __shared__ double normFactor;
  if (threadIdx.x == 0) {
    if (a.keff_analog >= 0) a.acc[a.keff_analog + 1] += *a.end_weight;
    normFactor = 1.0;
  }
  __syncthreads();
  if (a.last_cycle) {
    for (long long i = threadIdx.x; i < a.N; i += blockDim.x) { a.bin[i] = a.acc[i]; a.acc[i] = 0.0; }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (a.last_cycle && a.keff_analog >= 0) {          // keffAnalogClerk%closeCycle (:162-181)
      long long o = a.keff_analog;
      double k = a.bin[o + 1] / a.bin[o + 0] * (*a.k_end);
      a.csum[o + 2] = a.csum[o + 2] + k;
      a.csum2[o + 2] = a.csum2[o + 2] + k * k;
    }
    if (a.last_cycle && a.keff_implicit >= 0) {        // keffImplicitClerk%closeCycle (:306-326)
      long long o = a.keff_implicit;
      double k = a.bin[o + 0] / (a.bin[o + 2] + a.bin[o + 3] - a.bin[o + 1]);
      a.csum[o + 4] = a.csum[o + 4] + k;
      a.csum2[o + 4] = a.csum2[o + 4] + k * k;
    }
    if (a.norm_addr >= 0) normFactor = a.norm_val / a.bin[a.norm_addr];
  }
  __syncthreads();
  if (a.close_batch) {                                  // scoreMemory%closeCycle (:319-345)
    const double f = normFactor;
    for (long long i = threadIdx.x; i < a.N; i += blockDim.x) {
      double res = a.bin[i] * f;
      a.bin[i] = 0.0;
      a.csum[i] = a.csum[i] + res;
      a.csum2[i] = a.csum2[i] + res * res;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && a.k_out && a.k_addr >= 0 && a.batchN > 0)   // keffResult mean (:537-573)
    *a.k_out = a.csum[a.k_addr] / a.batchN;
}

cudaError_t launch_tally_close(const TallyCloseArgs& a, cudaStream_t s) {
  k_tally_close<<<1, 1024, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void k_add_scalar(double* p, const double* v, double c) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p += (v ? *v : c);
}
cudaError_t add_scalar(double* p, const double* v, double c, cudaStream_t s) {
  k_add_scalar<<<1, 32, 0, s>>>(p, v, c);
  return cudaGetLastError();
}

}  // namespace sg
