// sg_noalloc.cu -- sg_transport_bank_noalloc: the gen loop for callers that cannot allocate device
// memory.
//
// Some callers cannot call cudaMalloc at the point where they run a cycle: host programs whose
// device memory is owned by another allocator or by a pool reserved up front (a cudaMalloc would
// bypass it, or fail once the pool holds the GPU's memory), and real-time sections that must not
// enter the driver's allocator, whose calls can block.  For them this entry point runs the
// history-loop kernel on banks the caller already holds in device memory and keeps all of its
// per-call scratch (fission-site staging, per-history site counts, scan partial sums, counters, k)
// in one file-scope static __device__ array.  The handle (geometry, multigroup data, tallies) must
// have been set up beforehand; continuous-energy handles are refused.
//
// Limits: at most SG_NOALLOC_MAX_HISTORIES histories and SG_NOALLOC_MAX_SITES fission sites per
// call (3 MiB of device memory, held on every GPU that loads this library until the process exits).
// Every site goes to one region of the staging buffer, so the site limit is the call's total, however
// the sites fall over the warps.  All calls share the array: calls that overlap on the GPU
// (different streams or threads) race.
#include <cstdio>
#include <cstring>
#include <string>

#include "sg_internal.h"
#include "sg_launch.h"
#include "sg_support.h"
#include "sg_noalloc.h"

namespace {

constexpr int NA_MAX_HIST = SG_NOALLOC_MAX_HISTORIES;
constexpr int NA_MAX_SITES = SG_NOALLOC_MAX_SITES;
constexpr size_t NA_SCRATCH_BYTES = 3u << 20;

// byte layout of the scratch array (offsets 256-byte aligned)
constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t OFF_R = 0;
constexpr size_t OFF_DIR = al(OFF_R + 3 * sizeof(double) * NA_MAX_SITES);
constexpr size_t OFF_WGT = al(OFF_DIR + 3 * sizeof(double) * NA_MAX_SITES);
constexpr size_t OFF_TIME = al(OFF_WGT + sizeof(double) * NA_MAX_SITES);
constexpr size_t OFF_G = al(OFF_TIME + sizeof(double) * NA_MAX_SITES);
constexpr size_t OFF_BROOD = al(OFF_G + sizeof(int) * NA_MAX_SITES);
constexpr size_t OFF_SEQ = al(OFF_BROOD + sizeof(int) * NA_MAX_SITES);
constexpr size_t OFF_CURSOR = al(OFF_SEQ + sizeof(int) * NA_MAX_SITES);
constexpr size_t OFF_HISTN = al(OFF_CURSOR + sizeof(int) * sg::SITE_REGIONS);
constexpr size_t OFF_START = al(OFF_HISTN + sizeof(int) * (NA_MAX_HIST + 1));
constexpr size_t OFF_SCAN = al(OFF_START + sizeof(int) * (NA_MAX_HIST + 1));
constexpr size_t OFF_TOTALS = al(OFF_SCAN + sizeof(int) * 64);
constexpr size_t OFF_CTR = al(OFF_TOTALS + sizeof(int) * 8);
constexpr size_t OFF_K = al(OFF_CTR + sizeof(sg::DCounters));
constexpr size_t OFF_END = al(OFF_K + sizeof(double));
static_assert(OFF_END <= NA_SCRATCH_BYTES, "scratch layout exceeds the static array");

}  // namespace

// The scratch itself.  In host code this name is only a host-side stand-in: its device address
// comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_sg_noalloc_scratch[NA_SCRATCH_BYTES];

namespace {

constexpr int NA_MAX_DEVICES = 64;
void* g_scratch_ptr[NA_MAX_DEVICES] = {nullptr};

// Once per device, with that device current: the device address of the scratch array.
cudaError_t scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= NA_MAX_DEVICES) return cudaErrorInvalidDevice;
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sg_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[dev]);
  return cudaSuccess;
}

}  // namespace


namespace {

template <class R>
int run_noalloc(const sg::NoAllocView& v, sg::TransportArgs<R> t, unsigned char* S, const sg_bank* in, int n,
                uint64_t master, double k_eff, sg_bank* next, int next_cap, int32_t* n_next) {
  using namespace sg;
  cudaStream_t s = v.stream;
  auto fail = [&](int code, const char* m) {
    *v.err = m;
    return code;
  };
  double* dk = reinterpret_cast<double*>(S + OFF_K);
  t.in = DBank{in->r, in->dir, in->wgt, in->G, in->brood_id, in->time};
  t.n = n;
  t.master = master;
  t.k_eff = dk;
  t.sites = DSites{reinterpret_cast<double*>(S + OFF_R), reinterpret_cast<double*>(S + OFF_DIR),
                   reinterpret_cast<double*>(S + OFF_WGT), reinterpret_cast<int*>(S + OFF_G),
                   reinterpret_cast<int*>(S + OFF_BROOD), reinterpret_cast<int*>(S + OFF_SEQ),
                   reinterpret_cast<double*>(S + OFF_TIME), reinterpret_cast<int*>(S + OFF_CURSOR), NA_MAX_SITES,
                   0 /* one region: the site limit is the total */};
  int* histN = reinterpret_cast<int*>(S + OFF_HISTN);
  int* start = reinterpret_cast<int*>(S + OFF_START);
  int* scanTmp = reinterpret_cast<int*>(S + OFF_SCAN);
  int* totals = reinterpret_cast<int*>(S + OFF_TOTALS);
  t.hist_nsites = histN;
  t.rec_coll = nullptr;
  t.rec_rng = nullptr;
  t.ctr = reinterpret_cast<DCounters*>(S + OFF_CTR);
  size_t smem = (size_t)t.acc_n * sizeof(double);
  t.use_smem = scores_in_shared_memory(t.acc_n) ? 1 : 0;
  if (!t.use_smem) smem = 0;
  // the scratch keeps the previous call's contents: clear what must start at zero
  cudaError_t e;
  if ((e = cudaMemcpyAsync(dk, &k_eff, sizeof(double), cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemsetAsync(S + OFF_CTR, 0, sizeof(DCounters), s)) ||
      (e = cudaMemsetAsync(S + OFF_CURSOR, 0, sizeof(int) * SITE_REGIONS, s)) ||
      (e = cudaMemsetAsync(histN, 0, sizeof(int) * (n + 1), s)) ||
      (e = cudaMemsetAsync(totals, 0, sizeof(int) * 8, s)))
    return fail(SG_ERR_CUDA, cudaGetErrorString(e));
  if ((e = launch_transport<R>(t, v.maxl, transport_op(v.transport), smem, s, nullptr)) ||
      (e = exclusive_scan(histN, n + 1, start, scanTmp, totals + 0, s)))
    return fail(SG_ERR_CUDA, cudaGetErrorString(e));
  DBank out{next->r, next->dir, next->wgt, next->G, next->brood_id, next->time};
  if ((e = launch_site_scatter(t.sites, start, out, next_cap, totals + 3, s)))
    return fail(SG_ERR_CUDA, cudaGetErrorString(e));
  DCounters c;
  int tot[8];
  if ((e = cudaMemcpyAsync(&c, t.ctr, sizeof(c), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaMemcpyAsync(tot, totals, sizeof(tot), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return fail(SG_ERR_CUDA, cudaGetErrorString(e));
  if (c.err_code) {
    char m[160];
    if (c.err_code == SG_ERR_BANK_OVERFLOW)
      std::snprintf(m, sizeof(m), "sg_transport_bank_noalloc: more than SG_NOALLOC_MAX_SITES (%d) fission sites "
                    "(history %d); this call's partial scores stay in the tallies", NA_MAX_SITES, c.err_hist);
    else
      std::snprintf(m, sizeof(m), "transport: error %d raised in history %d", c.err_code, c.err_hist);
    return fail(c.err_code, m);
  }
  if (tot[3] || tot[0] > next_cap)
    return fail(SG_ERR_BANK_OVERFLOW, "sg_transport_bank_noalloc: next bank capacity too small");
  *n_next = tot[0];
  return SG_OK;
}

}  // namespace

extern "C" int32_t sg_transport_bank_noalloc(sg_handle h, int32_t admin, const sg_bank* dev_in, int32_t n,
                                             uint64_t master_state, double k_eff, sg_bank* dev_next,
                                             int32_t next_cap, int32_t* n_next) {
  using namespace sg;
  if (!h || !dev_in || !dev_next || !n_next) return SG_ERR_BAD_ARG;
  NoAllocView v;
  TransportArgs<double> t64;
  TransportArgs<float> t32;
  long long lo = 0;
  int rc = noalloc_view(h, admin, &v, &t64, &t32, &lo);
  if (rc) return rc;
  auto fail = [&](int code, const char* m) {
    *v.err = m;
    return code;
  };
  if (n < 0 || n > NA_MAX_HIST)
    return fail(SG_ERR_BAD_ARG, "sg_transport_bank_noalloc: n exceeds SG_NOALLOC_MAX_HISTORIES (16384)");
  if (next_cap < 0) return fail(SG_ERR_BAD_ARG, "sg_transport_bank_noalloc: negative next_cap");
  if (!dev_in->r || !dev_in->dir || !dev_in->wgt || !dev_in->G || !dev_in->time)
    return fail(SG_ERR_BAD_ARG, "sg_transport_bank_noalloc: input bank needs r, dir, wgt, G and time");
  if (!dev_next->r || !dev_next->dir || !dev_next->wgt || !dev_next->G || !dev_next->time || !dev_next->brood_id)
    return fail(SG_ERR_BAD_ARG, "sg_transport_bank_noalloc: output bank needs every array");
  unsigned char* S = nullptr;
  cudaError_t e = scratch_address(&S);
  if (e != cudaSuccess) return fail(SG_ERR_CUDA, cudaGetErrorString(e));
  *n_next = 0;
  if (n == 0) return SG_OK;
  if (v.precision == SG_PREC_MIXED)
    return run_noalloc<float>(v, t32, S, dev_in, n, master_state, k_eff, dev_next, next_cap, n_next);
  return run_noalloc<double>(v, t64, S, dev_in, n, master_state, k_eff, dev_next, next_cap, n_next);
}
