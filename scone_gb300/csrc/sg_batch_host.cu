// sg_batch_host.cu -- host side of the batched and served forms (include/scone_gpu.h, sg_batch_* and
// sg_serve_*).
//
// A batch owns one device arena (its HBM budget) holding every resident problem's geometry, MG data,
// source CDF and score memory, a table of problem records (BatchProblem) the kernel stages into
// shared memory, a table of score-memory records (BatchTally) for the cycle closes, and the device
// work queue.  A run is one CUDA graph: work-list upload, counter reset, the persistent batched
// kernel, the cycle closes and the counter read-back.  Serving runs the same graph once per wave.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include "sg_batch.h"

using namespace sg;

namespace {

// First-fit allocator over [0, cap) in 256-byte units, free blocks coalesced.
class ArenaAlloc {
 public:
  void init(size_t cap) {
    free_.clear();
    cap_ = cap & ~size_t(255);
    if (cap_) free_[0] = cap_;
    used_ = 0;
  }
  bool take(size_t bytes, size_t* off) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        size_t rest = it->second - bytes, at = it->first + bytes;
        free_.erase(it);
        if (rest) free_[at] = rest;
        used_ += bytes;
        return true;
      }
    }
    return false;
  }
  void give(size_t off, size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
    }
  }
  size_t used() const { return used_; }
  size_t cap() const { return cap_; }

 private:
  std::map<size_t, size_t> free_;
  size_t cap_ = 0, used_ = 0;
};

struct Slot {
  bool used = false;
  size_t dataOff = 0, dataBytes = 0, tallyOff = 0, tallyBytes = 0;
  StagedProblem sp;
  sg_point_source_desc src{};
  int pop = 0, cycles = 0;
  unsigned long long master = 0;
  BatchTally tl{};
  int parent = -1;             // instance of a resident problem: the slot whose data it shares
  int children = 0;            // instances sharing this slot's data
};

// a request of the serving loop
struct Request {
  int slot;
  long long next, total;       // flat histories launched / to launch
  double submit;               // host clock
};

struct Wave {
  cudaEvent_t done = nullptr;
  int mirror = 0;
  std::vector<Request> closing;   // requests whose last histories ran in this wave
  long long histories = 0;
};

double host_now() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct sg_batch_t {
  sg_batch_config cfg{};
  cudaStream_t stream = nullptr;
  std::string err;
  int sms = 0;

  char* arena = nullptr;
  ArenaAlloc alloc;
  std::vector<char> staging;
  std::vector<Slot> slots;

  void* dProbs = nullptr;          // BatchProblem<R>[max_problems]
  size_t recBytes = 0;
  BatchTally* dTallies = nullptr;
  // device work list, counts, close list and counters of each mirror set (serving keeps two waves
  // in flight, on two streams)
  WorkItem* dItems[2] = {nullptr, nullptr};
  int* dInts[2] = {nullptr, nullptr};      // [0] n_items, [1] head, [2] n_close
  int* dClose[2] = {nullptr, nullptr};     // [max_problems]
  DCounters* dCtr[2] = {nullptr, nullptr};
  cudaStream_t ws[2] = {nullptr, nullptr}; // wave streams
  cudaStream_t cstream = nullptr;          // cycle closes of the waves
  cudaEvent_t kdone[2] = {nullptr, nullptr};
  cudaEvent_t upl = nullptr;
  double* dOne = nullptr;

  cudaStream_t rstream = nullptr;  // read-back of completed score memory while waves run
  char* hRec = nullptr;            // pinned problem records, one per slot (async uploads)
  BatchTally* hTl = nullptr;

  // pinned host mirrors read by the graph's copies (two sets: serving keeps two waves in flight)
  WorkItem* hItems[2] = {nullptr, nullptr};
  int* hInts[2] = {nullptr, nullptr};
  int* hClose[2] = {nullptr, nullptr};
  DCounters* hCtr[2] = {nullptr, nullptr};

  sg_batch_tuning tune{1024, 0, 128, 1};
  int maxlUsed = 2;

  // run graph per (mirror set, nesting class): rebuilt when the tuning changes
  struct Graph {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t itemsCopy = nullptr, closeCopy = nullptr;
    sg_batch_tuning tune{};
  } graph[2][4][2];               // [mirror][kernel class: nesting 2 or 4, + 2 lean][SMs reserved for other streams]
  int reserve = 0;                 // blocks per SM the serving waves leave to other streams' kernels
  int reserving = 0;               // reserve in force (serving with other work on the device)
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

  sg_handle plainWork = nullptr;
  int plainForm = -1;
  int plainCap = 0;
  sg_event_tuning plainTune{4, 4096, 64};

  // serving
  bool serving = false;
  long long waveHist = 0;
  int serveItem = 1024;
  std::deque<Request> active;
  std::deque<Wave> waves;
  std::vector<int> doneSlots;      // completed requests not yet handed out
  std::vector<double> doneLat;
  long long wavesLaunched = 0;
  long long servedEvents = 0, servedHistories = 0;   // of retired waves
  int mirror = 0;
  cudaEvent_t ref = nullptr;
  double refHost = 0.0;

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
};

#define BCK(call)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return b->fail(SG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

namespace sg {

// scoreMemory%closeCycle of every cycle of the listed problems, in cycle order
// (scoreMemory_class.f90:319-345, tallyAdmin_class.f90:744-788 with batchSize 1): BIN = the cycle's
// accumulator, normalised by `norm` when set; CSUM += BIN; CSUM2 += BIN^2; BIN = 0.
__global__ void k_batch_close(const BatchTally* __restrict__ tl, const int* __restrict__ slots, const int* n_close) {
  __shared__ double f;
  const int n = *n_close;
  for (int p = blockIdx.x; p < n; p += gridDim.x) {
    const BatchTally T = tl[slots[p]];
    for (int c = 0; c < T.cycles; ++c) {
      double* a = T.acc + (long long)c * T.n;
      __syncthreads();
      if (threadIdx.x == 0) f = (T.norm_addr >= 0) ? T.norm_val / a[T.norm_addr] : 1.0;
      __syncthreads();
      const double fc = f;
      for (long long i = threadIdx.x; i < T.n; i += blockDim.x) {
        const double res = a[i] * fc;
        a[i] = 0.0;
        T.bin[i] = 0.0;
        T.csum[i] = T.csum[i] + res;
        T.csum2[i] = T.csum2[i] + res * res;
      }
    }
  }
}

cudaError_t launch_batch_close(const BatchTally* tallies, const int* slots, const int* n, int grid, cudaStream_t s) {
  k_batch_close<<<grid, 256, 0, s>>>(tallies, slots, n);
  return cudaGetLastError();
}

}  // namespace sg

namespace {

bool fp64(sg_batch b) { return b->cfg.precision == SG_PREC_FP64; }

int check_slot(sg_batch b, int slot) {
  if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used) return b->fail(SG_ERR_BAD_ARG, "batch: bad slot");
  return SG_OK;
}

// Whether a problem can run the lean history loop: no rotated universe, cell map, surface-current
// clerk or P1 scattering (the batched form runs the standard collision processors).
bool slot_lean(const Slot& S) {
  const auto& t = S.sp.t64;
  return t.geom.rot == nullptr && !t.has_cellmap && !t.has_current && !t.coll_imp && t.mg.P1n == nullptr;
}

int grid_for(sg_batch b, int maxl, int lean) {
  const int dt = transport_op(b->cfg.transport);
  const int occ = fp64(b) ? batch_occupancy<double>(maxl, lean, dt, b->tune.block_threads)
                          : batch_occupancy<float>(maxl, lean, dt, b->tune.block_threads);
  int per = b->tune.blocks_per_sm > 0 ? std::min(b->tune.blocks_per_sm, occ) : occ;
  if (b->reserving) per -= b->reserve;
  return b->sms * std::max(per, 1);
}

void drop_graph(sg_batch_t::Graph& G) {
  if (G.exec) cudaGraphExecDestroy(G.exec);
  if (G.g) cudaGraphDestroy(G.g);
  G = sg_batch_t::Graph();
}

// The transport graph of mirror set m and kernel class x (bit 0: maxl 4 instead of 2; bit 1: the
// lean history loop, for launches whose problems all allow it): copies of the
// work list, the count block and the close list from pinned memory, counter reset and the batched
// kernel.  The two list copies are resized to the current counts before each launch; the kernels
// read the counts from device memory.  The cycle closes run after it (run_closes).
int build_graph(sg_batch b, int m, int x) {
  sg_batch_t::Graph& G = b->graph[m][x][b->reserving];
  if (G.exec) {
    if (std::memcmp(&G.tune, &b->tune, sizeof(G.tune)) == 0) return SG_OK;
    drop_graph(G);
  }
  const int maxl = (x & 1) ? 4 : 2;
  const int lean = x >> 1;
  cudaStream_t s = b->stream;
  const int dt = transport_op(b->cfg.transport);
  BatchLaunch L;
  L.problems = b->dProbs;
  L.items = b->dItems[m];
  L.n_items = b->dInts[m] + 0;
  L.head = b->dInts[m] + 1;
  L.ctr = b->dCtr[m];
  L.k_one = b->dOne;
  L.maxl = maxl;
  L.lean = lean;
  const int grid = grid_for(b, maxl, lean);
  BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  auto step = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  step(cudaMemcpyAsync(b->dItems[m], b->hItems[m], sizeof(WorkItem), cudaMemcpyHostToDevice, s));
  step(cudaMemcpyAsync(b->dInts[m], b->hInts[m], 4 * sizeof(int), cudaMemcpyHostToDevice, s));
  step(cudaMemcpyAsync(b->dClose[m], b->hClose[m], sizeof(int), cudaMemcpyHostToDevice, s));
  step(cudaMemsetAsync(b->dCtr[m], 0, sizeof(DCounters), s));
  step(fp64(b) ? launch_batch<double>(L, dt, grid, b->tune.block_threads, s)
               : launch_batch<float>(L, dt, grid, b->tune.block_threads, s));
  cudaError_t ee = cudaStreamEndCapture(s, &G.g);
  if (e == cudaSuccess) e = ee;
  if (e == cudaSuccess) {
    size_t nn = 0;
    e = cudaGraphGetNodes(G.g, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (e == cudaSuccess && nn) e = cudaGraphGetNodes(G.g, nodes.data(), &nn);
    for (size_t i = 0; e == cudaSuccess && i < nn; ++i) {
      cudaGraphNodeType t;
      e = cudaGraphNodeGetType(nodes[i], &t);
      if (e != cudaSuccess || t != cudaGraphNodeTypeMemcpy) continue;
      cudaMemcpy3DParms pr{};
      e = cudaGraphMemcpyNodeGetParams(nodes[i], &pr);
      if (pr.dstPtr.ptr == (void*)b->dItems[m]) G.itemsCopy = nodes[i];
      if (pr.dstPtr.ptr == (void*)b->dClose[m]) G.closeCopy = nodes[i];
    }
    if (e == cudaSuccess && (!G.itemsCopy || !G.closeCopy)) e = cudaErrorUnknown;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&G.exec, G.g, 0);
  if (e != cudaSuccess) {
    drop_graph(G);
    return b->fail(SG_ERR_CUDA, std::string("batch: run graph: ") + cudaGetErrorString(e));
  }
  G.tune = b->tune;
  return SG_OK;
}

// cut the flat histories [first, end) of a slot into items of at most `size`
void cut_items(std::vector<WorkItem>& out, int slot, long long first, long long end, int size) {
  for (long long f = first; f < end; f += size) {
    WorkItem w;
    w.slot = slot;
    w.first = (int)f;
    w.count = (int)std::min<long long>(size, end - f);
    w.pad = 0;
    out.push_back(w);
  }
}

int write_record(sg_batch b, int slot) {
  Slot& S = b->slots[slot];
  double* acc = reinterpret_cast<double*>(b->arena + S.tallyOff);
  const long long N = S.sp.n_bins;
  S.tl.acc = acc;
  S.tl.bin = acc + (long long)S.cycles * N;
  S.tl.csum = S.tl.bin + N;
  S.tl.csum2 = S.tl.csum + N;
  S.tl.n = N;
  S.tl.norm_addr = S.sp.norm_addr;
  S.tl.norm_val = S.sp.norm_val;
  S.tl.cycles = S.cycles;
  auto fill = [&](auto& rec, const auto& t) {
    std::memset(&rec, 0, sizeof(rec));
    rec.t = t;
    rec.t.n = S.pop;
    rec.t.master = S.master;
    rec.t.k_eff = b->dOne;
    rec.t.acc = acc;
    rec.t.acc_n = (int)N;
    rec.t.use_smem = 0;
    rec.t.ctr = b->dCtr[0];           // replaced by the launch's counters when staged
    rec.t.use_cache = transport_cache(b->cfg.transport);
    rec.t.max_segments = 1000000;
    rec.t.ht_cutoff = (decltype(rec.t.ht_cutoff))(b->cfg.ht_cutoff > 0.0 ? b->cfg.ht_cutoff : 0.9);
    for (int i = 0; i < 3; ++i) { rec.src_r[i] = S.src.r[i]; rec.src_dir[i] = S.src.dir[i]; }
    rec.src_prob_g = S.src.n_prob_g > 0 ? S.sp.prob_g : nullptr;
    rec.src_isotropic = S.src.isotropic;
    rec.src_G = S.src.G;
    rec.src_n_prob_g = S.src.n_prob_g;
    rec.pop = S.pop;
    rec.cycles = S.cycles;
    rec.maxl = S.sp.maxl;
    rec.master = S.master;
    rec.n_bins = N;
  };
  cudaStream_t s = b->stream;
  char* h = b->hRec + b->recBytes * slot;
  if (fp64(b)) fill(*reinterpret_cast<BatchProblem<double>*>(h), S.sp.t64);
  else fill(*reinterpret_cast<BatchProblem<float>*>(h), S.sp.t32);
  b->hTl[slot] = S.tl;
  BCK(cudaMemcpyAsync(static_cast<char*>(b->dProbs) + b->recBytes * slot, h, b->recBytes, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->dTallies + slot, b->hTl + slot, sizeof(BatchTally), cudaMemcpyHostToDevice, s));
  return SG_OK;
}

int clear_tally(sg_batch b, int slot) {
  const Slot& S = b->slots[slot];
  BCK(cudaMemsetAsync(b->arena + S.tallyOff, 0, S.tallyBytes, b->stream));
  return SG_OK;
}

// launches the transport graph of mirror set m, for the items and closes written to that set, on
// stream `s`
int launch_graph(sg_batch b, int m, int maxl, bool lean, cudaStream_t s) {
  const int x = (maxl > 2 ? 1 : 0) + (lean ? 2 : 0);
  int rc = build_graph(b, m, x);
  if (rc) return rc;
  sg_batch_t::Graph& G = b->graph[m][x][b->reserving];
  const size_t ni = (size_t)std::max(1, b->hInts[m][0]), nc = (size_t)std::max(1, b->hInts[m][2]);
  BCK(cudaGraphExecMemcpyNodeSetParams1D(G.exec, G.itemsCopy, b->dItems[m], b->hItems[m], sizeof(WorkItem) * ni,
                                         cudaMemcpyHostToDevice));
  BCK(cudaGraphExecMemcpyNodeSetParams1D(G.exec, G.closeCopy, b->dClose[m], b->hClose[m], sizeof(int) * nc,
                                         cudaMemcpyHostToDevice));
  BCK(cudaGraphLaunch(G.exec, s));
  return SG_OK;
}

// the cycle closes of the problems in mirror set m's close list, then its counters to the host
int run_closes(sg_batch b, int m, cudaStream_t s) {
  BCK(launch_batch_close(b->dTallies, b->dClose[m], b->dInts[m] + 2, b->sms * 4, s));
  BCK(cudaMemcpyAsync(b->hCtr[m], b->dCtr[m], sizeof(DCounters), cudaMemcpyDeviceToHost, s));
  return SG_OK;
}

int read_counters(sg_batch b, int m) {
  const DCounters& c = *b->hCtr[m];
  if (c.err_code) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "batch: transport error %d raised in history %d", c.err_code, c.err_hist);
    return b->fail(c.err_code, msg);
  }
  return SG_OK;
}

int release_slot_memory(sg_batch b, Slot& S) {
  if (S.parent >= 0) b->slots[S.parent].children -= 1;
  if (S.dataBytes && S.parent < 0) b->alloc.give(S.dataOff, S.dataBytes);
  if (S.tallyBytes) b->alloc.give(S.tallyOff, S.tallyBytes);
  S = Slot();
  return SG_OK;
}

}  // namespace

extern "C" {

int32_t sg_batch_create(const sg_batch_config* cfg, sg_batch* out) {
  if (!cfg || !out) return SG_ERR_BAD_ARG;
  *out = nullptr;
  if (cfg->precision != SG_PREC_FP64 && cfg->precision != SG_PREC_MIXED) return SG_ERR_BAD_ARG;
  if (cfg->transport < SG_TRANSPORT_ST || cfg->transport > SG_TRANSPORT_HT_NOCACHE) return SG_ERR_BAD_ARG;
  if (!(cfg->ht_cutoff >= 0.0 && cfg->ht_cutoff < 1.0)) return SG_ERR_BAD_ARG;
  if (cfg->max_problems <= 0 || cfg->arena_bytes <= 0 || cfg->max_work_items <= 0) return SG_ERR_BAD_ARG;
  sg_batch b = new sg_batch_t();
  b->cfg = *cfg;
  auto bad = [&](int code) { sg_batch_destroy(b); return code; };
  if (cudaSetDevice(cfg->device) != cudaSuccess) return bad(SG_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->rstream, cudaStreamNonBlocking) != cudaSuccess)
    return bad(SG_ERR_CUDA);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, cfg->device);
  b->recBytes = fp64(b) ? sizeof(BatchProblem<double>) : sizeof(BatchProblem<float>);
  const size_t P = (size_t)cfg->max_problems, W = (size_t)cfg->max_work_items;
  if (cudaMalloc((void**)&b->arena, (size_t)cfg->arena_bytes) != cudaSuccess) return bad(SG_ERR_OOM);
  b->alloc.init((size_t)cfg->arena_bytes);
  if (cudaMalloc(&b->dProbs, b->recBytes * P) != cudaSuccess || cudaMalloc((void**)&b->dTallies, sizeof(BatchTally) * P) != cudaSuccess ||
      cudaMalloc((void**)&b->dOne, sizeof(double)) != cudaSuccess)
    return bad(SG_ERR_OOM);
  for (int m = 0; m < 2; ++m) {
    if (cudaMalloc((void**)&b->dItems[m], sizeof(WorkItem) * W) != cudaSuccess ||
        cudaMalloc((void**)&b->dInts[m], 4 * sizeof(int)) != cudaSuccess ||
        cudaMalloc((void**)&b->dClose[m], sizeof(int) * P) != cudaSuccess ||
        cudaMalloc((void**)&b->dCtr[m], sizeof(DCounters)) != cudaSuccess)
      return bad(SG_ERR_OOM);
    if (cudaStreamCreateWithFlags(&b->ws[m], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->kdone[m], cudaEventDisableTiming) != cudaSuccess)
      return bad(SG_ERR_CUDA);
  }
  if (cudaStreamCreateWithFlags(&b->cstream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->upl, cudaEventDisableTiming) != cudaSuccess)
    return bad(SG_ERR_CUDA);
  if (cudaMallocHost((void**)&b->hRec, b->recBytes * P) != cudaSuccess ||
      cudaMallocHost((void**)&b->hTl, sizeof(BatchTally) * P) != cudaSuccess)
    return bad(SG_ERR_OOM);
  for (int m = 0; m < 2; ++m)
    if (cudaMallocHost((void**)&b->hItems[m], sizeof(WorkItem) * W) != cudaSuccess ||
        cudaMallocHost((void**)&b->hInts[m], 4 * sizeof(int)) != cudaSuccess ||
        cudaMallocHost((void**)&b->hClose[m], sizeof(int) * P) != cudaSuccess ||
        cudaMallocHost((void**)&b->hCtr[m], sizeof(DCounters)) != cudaSuccess)
      return bad(SG_ERR_OOM);
  const double one = 1.0;
  if (cudaMemcpy(b->dOne, &one, sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) return bad(SG_ERR_CUDA);
  for (auto& e : b->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return bad(SG_ERR_CUDA);
  b->slots.resize(P);
  *out = b;
  return SG_OK;
}

int32_t sg_batch_destroy(sg_batch b) {
  if (!b) return SG_ERR_BAD_ARG;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& w : b->waves) cudaEventDestroy(w.done);
  if (b->ref) cudaEventDestroy(b->ref);
  for (auto& plane : b->graph)
    for (auto& row : plane)
      for (auto& g : row) drop_graph(g);
  if (b->plainWork) sg_destroy(b->plainWork);
  cudaFree(b->arena);
  cudaFree(b->dProbs);
  cudaFree(b->dTallies);
  for (int m = 0; m < 2; ++m) {
    if (b->ws[m]) cudaStreamSynchronize(b->ws[m]);
    cudaFree(b->dItems[m]);
    cudaFree(b->dInts[m]);
    cudaFree(b->dClose[m]);
    cudaFree(b->dCtr[m]);
    if (b->kdone[m]) cudaEventDestroy(b->kdone[m]);
    if (b->ws[m]) cudaStreamDestroy(b->ws[m]);
  }
  if (b->cstream) { cudaStreamSynchronize(b->cstream); cudaStreamDestroy(b->cstream); }
  if (b->upl) cudaEventDestroy(b->upl);
  cudaFree(b->dOne);
  for (int m = 0; m < 2; ++m) {
    cudaFreeHost(b->hItems[m]);
    cudaFreeHost(b->hInts[m]);
    cudaFreeHost(b->hClose[m]);
    cudaFreeHost(b->hCtr[m]);
  }
  cudaFreeHost(b->hRec);
  cudaFreeHost(b->hTl);
  for (auto& e : b->ev) if (e) cudaEventDestroy(e);
  if (b->rstream) cudaStreamDestroy(b->rstream);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return SG_OK;
}

int32_t sg_batch_last_error(sg_batch b, char* buf, size_t len) {
  if (!b || !buf || len == 0) return SG_ERR_BAD_ARG;
  std::snprintf(buf, len, "%s", b->err.c_str());
  return SG_OK;
}

int32_t sg_batch_add(sg_batch b, const sg_problem_desc* p, int32_t* slot_out) {
  if (!b || !p || !slot_out || !p->geometry || !p->mg || !p->source || !p->tally) return SG_ERR_BAD_ARG;
  if (p->pop <= 0 || p->cycles <= 0 || (long long)p->pop * p->cycles > 0x7fffffffLL)
    return b->fail(SG_ERR_BAD_ARG, "batch: pop and cycles must be positive with pop * cycles < 2^31");
  if (p->tally->batch_size > 1) return b->fail(SG_ERR_BAD_ARG, "batch: tally batch_size must be 1");
  int slot = -1;
  for (int i = 0; i < (int)b->slots.size(); ++i)
    if (!b->slots[i].used) { slot = i; break; }
  if (slot < 0) return b->fail(SG_ERR_OOM, "batch: every problem slot is in use");
  Slot S;
  size_t bytes = 0;
  std::string err;
  int rc = stage_problem(p->geometry, p->mg, p->source, p->tally, nullptr, nullptr, 0, &bytes, &S.sp, &err);
  if (rc) return b->fail(rc, err);
  const size_t tallyBytes = sizeof(double) * (size_t)S.sp.n_bins * (size_t)(p->cycles + 3);
  if (!b->alloc.take(bytes, &S.dataOff)) return b->fail(SG_ERR_OOM, "batch: arena full (problem data)");
  S.dataBytes = bytes;
  if (!b->alloc.take(tallyBytes, &S.tallyOff)) {
    b->alloc.give(S.dataOff, S.dataBytes);
    return b->fail(SG_ERR_OOM, "batch: arena full (score memory)");
  }
  S.tallyBytes = tallyBytes;
  size_t used = 0;
  rc = stage_problem(p->geometry, p->mg, p->source, p->tally, b->arena + S.dataOff, &b->staging, S.dataBytes,
                     &used, &S.sp, &err);
  if (rc || used > S.dataBytes) {
    release_slot_memory(b, S);
    return b->fail(rc ? rc : SG_ERR_STATE, rc ? err : "batch: staged size changed");
  }
  BCK(cudaMemcpyAsync(b->arena + S.dataOff, b->staging.data(), used, cudaMemcpyHostToDevice, b->stream));
  S.used = true;
  S.src = *p->source;
  S.src.prob_g = nullptr;
  S.pop = p->pop;
  S.cycles = p->cycles;
  S.master = p->master_state;
  b->slots[slot] = S;
  rc = clear_tally(b, slot);
  if (!rc) rc = write_record(b, slot);
  if (rc) {
    release_slot_memory(b, b->slots[slot]);
    return rc;
  }
  BCK(cudaStreamSynchronize(b->stream));           // the staging image is reused by the next add
  *slot_out = slot;
  return SG_OK;
}

int32_t sg_batch_instance(sg_batch b, int32_t parent, int32_t pop, int32_t cycles, uint64_t master, int32_t* slot_out) {
  if (!b || !slot_out) return SG_ERR_BAD_ARG;
  int rc = check_slot(b, parent);
  if (rc) return rc;
  if (b->slots[parent].parent >= 0) return b->fail(SG_ERR_BAD_ARG, "batch: an instance cannot be a parent");
  if (pop <= 0 || cycles <= 0 || (long long)pop * cycles > 0x7fffffffLL)
    return b->fail(SG_ERR_BAD_ARG, "batch: pop and cycles must be positive with pop * cycles < 2^31");
  int slot = -1;
  for (int i = 0; i < (int)b->slots.size(); ++i)
    if (!b->slots[i].used) { slot = i; break; }
  if (slot < 0) return b->fail(SG_ERR_OOM, "batch: every problem slot is in use");
  Slot S = b->slots[parent];
  S.children = 0;
  S.parent = parent;
  S.pop = pop;
  S.cycles = cycles;
  S.master = master;
  S.tallyBytes = sizeof(double) * (size_t)S.sp.n_bins * (size_t)(cycles + 3);
  if (!b->alloc.take(S.tallyBytes, &S.tallyOff)) return b->fail(SG_ERR_OOM, "batch: arena full (score memory)");
  b->slots[parent].children += 1;
  b->slots[slot] = S;
  rc = clear_tally(b, slot);
  if (!rc) rc = write_record(b, slot);
  if (rc) {
    release_slot_memory(b, b->slots[slot]);
    return rc;
  }
  *slot_out = slot;
  return SG_OK;
}

int32_t sg_batch_remove(sg_batch b, int32_t slot) {
  if (!b) return SG_ERR_BAD_ARG;
  int rc = check_slot(b, slot);
  if (rc) return rc;
  for (const Request& r : b->active)
    if (r.slot == slot) return b->fail(SG_ERR_STATE, "batch: the slot is an active request");
  for (const Wave& w : b->waves)
    for (const Request& q : w.closing)
      if (q.slot == slot) return b->fail(SG_ERR_STATE, "batch: the slot's request is still in flight");
  if (b->slots[slot].children > 0) return b->fail(SG_ERR_STATE, "batch: instances still share this slot's data");
  // no wave in flight reads this slot, so its memory can go back to the arena at once; later uses
  // of it are ordered on the batch stream
  if (!b->serving) BCK(cudaStreamSynchronize(b->stream));
  return release_slot_memory(b, b->slots[slot]);
}

int32_t sg_batch_memory(sg_batch b, int64_t* used, int64_t* capacity) {
  if (!b) return SG_ERR_BAD_ARG;
  if (used) *used = (int64_t)b->alloc.used();
  if (capacity) *capacity = (int64_t)b->alloc.cap();
  return SG_OK;
}

int32_t sg_batch_set_tuning(sg_batch b, const sg_batch_tuning* t) {
  if (!b || !t) return SG_ERR_BAD_ARG;
  if (t->item_histories < 32 || t->block_threads < 32 || t->block_threads > 128 || t->block_threads % 32 ||
      t->blocks_per_sm < 0 || t->order < 0 || t->order > 2)
    return b->fail(SG_ERR_BAD_ARG, "batch: bad tuning");
  b->tune = *t;
  return SG_OK;
}

int32_t sg_batch_get_tuning(sg_batch b, sg_batch_tuning* t) {
  if (!b || !t) return SG_ERR_BAD_ARG;
  *t = b->tune;
  return SG_OK;
}

int32_t sg_batch_run(sg_batch b, const int32_t* slots, int32_t n, sg_batch_stats* stats) {
  if (!b || (n > 0 && !slots) || n < 0) return SG_ERR_BAD_ARG;
  if (b->serving) return b->fail(SG_ERR_STATE, "batch: serving is active");
  if (n > b->cfg.max_problems) return b->fail(SG_ERR_BAD_ARG, "batch: too many problems");
  std::vector<int> order(slots, slots + n);
  std::vector<char> seen(b->slots.size(), 0);
  int maxl = 2;
  bool lean = true;
  long long hist = 0;
  for (int s : order) {
    int rc = check_slot(b, s);
    if (rc) return rc;
    if (seen[s]) return b->fail(SG_ERR_BAD_ARG, "batch: a slot is listed twice");
    seen[s] = 1;
    maxl = std::max(maxl, b->slots[s].sp.maxl);
    lean = lean && slot_lean(b->slots[s]);
    hist += (long long)b->slots[s].pop * b->slots[s].cycles;
  }
  auto size_of = [&](int x) { return (long long)b->slots[x].pop * b->slots[x].cycles; };
  if (b->tune.order == 1)
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return size_of(x) > size_of(y); });
  else if (b->tune.order == 2)      // problems of one kind together (nesting, group count), largest first
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      const Slot &X = b->slots[x], &Y = b->slots[y];
      if (X.sp.maxl != Y.sp.maxl) return X.sp.maxl < Y.sp.maxl;
      if (X.sp.t64.mg.nG != Y.sp.t64.mg.nG) return X.sp.t64.mg.nG < Y.sp.t64.mg.nG;
      return size_of(x) > size_of(y);
    });
  std::vector<WorkItem> items;
  for (int s : order) cut_items(items, s, 0, (long long)b->slots[s].pop * b->slots[s].cycles, b->tune.item_histories);
  if ((long long)items.size() > b->cfg.max_work_items) return b->fail(SG_ERR_BAD_ARG, "batch: more work items than the queue holds");
  const int m = 0;
  std::memcpy(b->hItems[m], items.data(), sizeof(WorkItem) * items.size());
  b->hInts[m][0] = (int)items.size();
  b->hInts[m][1] = 0;
  b->hInts[m][2] = n;
  b->hInts[m][3] = 0;
  for (int i = 0; i < n; ++i) b->hClose[m][i] = order[i];
  BCK(cudaEventRecord(b->ev[2], b->stream));
  int rc = launch_graph(b, m, maxl, lean, b->stream);
  if (rc) return rc;
  rc = run_closes(b, m, b->stream);
  if (rc) return rc;
  BCK(cudaEventRecord(b->ev[3], b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  rc = read_counters(b, m);
  if (rc) return rc;
  if (stats) {
    // events bracket the graph launch: the kernel time includes the work-list copy and the closes
    // (microseconds beside the transport kernel)
    float r = 0.f;
    BCK(cudaEventElapsedTime(&r, b->ev[2], b->ev[3]));
    const float k = r;
    stats->n_histories = hist;
    stats->n_events = (int64_t)b->hCtr[m]->events;
    stats->n_collisions = (int64_t)b->hCtr[m]->collisions;
    stats->n_problems = n;
    stats->n_items = (int32_t)items.size();
    stats->kernel_ms = k;
    stats->run_ms = r;
    stats->n_kernels = 2;
  }
  return SG_OK;
}

int32_t sg_batch_run_plain(sg_batch b, const int32_t* slots, int32_t n, int32_t form, sg_batch_stats* stats) {
  if (!b || (n > 0 && !slots) || n < 0) return SG_ERR_BAD_ARG;
  if (form != SG_FORM_EVENT && form != SG_FORM_HISTORY) return b->fail(SG_ERR_BAD_ARG, "batch: bad form");
  if (b->serving) return b->fail(SG_ERR_STATE, "batch: serving is active");
  int maxPop = 1;
  for (int i = 0; i < n; ++i) {
    int rc = check_slot(b, slots[i]);
    if (rc) return rc;
    maxPop = std::max(maxPop, b->slots[slots[i]].pop);
  }
  if (!b->plainWork || b->plainForm != form || maxPop > b->plainCap) {
    if (b->plainWork) sg_destroy(b->plainWork);
    b->plainWork = nullptr;
    sg_config c{};
    c.precision = b->cfg.precision;
    c.transport = b->cfg.transport;
    c.device = b->cfg.device;
    c.max_bank = std::max(maxPop, 1024);
    c.record_histories = 0;
    c.form = form;
    c.ht_cutoff = b->cfg.ht_cutoff;
    int rc = sg_create(&c, &b->plainWork);
    if (rc) return b->fail(rc, "batch: cannot create the plain-form work handle");
    b->plainForm = form;
    b->plainCap = c.max_bank;
  }
  if (sg_set_event_tuning(b->plainWork, &b->plainTune) != SG_OK) return b->fail(SG_ERR_BAD_ARG, "batch: bad event tuning");
  BCK(cudaStreamSynchronize(b->stream));
  sg_batch_stats tot{};
  const double t0 = host_now();
  for (int i = 0; i < n; ++i) {
    Slot& S = b->slots[slots[i]];
    sg_cycle_stats st{};
    int rc = plain_fixed_source(b->plainWork, S.sp, &S.src, S.tl.acc, S.tl.bin, S.tl.csum, S.tl.csum2, S.pop, S.cycles,
                                S.master, &st);
    if (rc) {
      char msg[512];
      sg_last_error(b->plainWork, msg, sizeof(msg));
      return b->fail(rc, std::string("batch (plain): ") + msg);
    }
    tot.n_histories += st.n_histories;
    tot.n_events += st.n_events;
    tot.n_collisions += st.n_collisions;
    tot.kernel_ms += st.transport_ms;
    tot.n_kernels += st.n_kernels;
  }
  tot.run_ms = 1e3 * (host_now() - t0);
  tot.n_problems = n;
  if (stats) *stats = tot;
  return SG_OK;
}

int32_t sg_batch_autotune(sg_batch b, const int32_t* slots, int32_t n, sg_batch_tuning* best) {
  if (!b || !slots || n <= 0) return SG_ERR_BAD_ARG;
  if (b->serving) return b->fail(SG_ERR_STATE, "batch: serving is active");
  // coordinate search from the current shape: work-item size, then block shape, then blocks per
  // SM, then item order; each candidate timed (kernel events) on the listed problems, best of 2
  sg_batch_tuning cur = b->tune;
  auto time_it = [&](const sg_batch_tuning& t, double* ms) -> int {
    b->tune = t;
    double bestMs = 1e300;
    for (int r = 0; r < 2; ++r) {
      sg_batch_stats st{};
      int rc = sg_batch_run(b, slots, n, &st);
      if (rc) return rc;
      bestMs = std::min(bestMs, st.kernel_ms);
    }
    *ms = bestMs;
    return SG_OK;
  };
  double curMs = 0.0;
  int rc = time_it(cur, &curMs);
  if (rc) return rc;
  const int items[] = {256, 512, 1024, 2048, 4096, 8192};
  const int blocks[] = {64, 96, 128};
  for (int pass = 0; pass < 4; ++pass) {
    std::vector<sg_batch_tuning> cands;
    if (pass == 0) for (int v : items) { sg_batch_tuning t = cur; t.item_histories = v; cands.push_back(t); }
    if (pass == 1) for (int v : blocks) { sg_batch_tuning t = cur; t.block_threads = v; cands.push_back(t); }
    if (pass == 2) {
      int maxl = 2, lean = 1;
      for (int i = 0; i < n; ++i) {
        maxl = std::max(maxl, b->slots[slots[i]].sp.maxl);
        lean = lean && slot_lean(b->slots[slots[i]]);
      }
      const int dt = transport_op(b->cfg.transport);
      const int occ = fp64(b) ? batch_occupancy<double>(maxl, lean, dt, cur.block_threads)
                              : batch_occupancy<float>(maxl, lean, dt, cur.block_threads);
      for (int v = std::max(1, occ / 2); v <= occ; ++v) { sg_batch_tuning t = cur; t.blocks_per_sm = v; cands.push_back(t); }
    }
    if (pass == 3) for (int v = 0; v <= 2; ++v) { sg_batch_tuning t = cur; t.order = v; cands.push_back(t); }
    for (const auto& t : cands) {
      if (std::memcmp(&t, &cur, sizeof(t)) == 0) continue;
      double ms = 0.0;
      rc = time_it(t, &ms);
      if (rc == SG_ERR_BAD_ARG) { b->tune = cur; continue; }   // e.g. too many work items for the queue
      if (rc) return rc;
      if (ms < curMs) { cur = t; curMs = ms; }
    }
  }
  b->tune = cur;
  for (int i = 0; i < n; ++i) {
    rc = clear_tally(b, slots[i]);
    if (rc) return rc;
  }
  BCK(cudaStreamSynchronize(b->stream));
  if (best) *best = cur;
  return SG_OK;
}

int32_t sg_batch_autotune_plain(sg_batch b, const int32_t* slots, int32_t n, sg_event_tuning* best) {
  if (!b || !slots || n <= 0) return SG_ERR_BAD_ARG;
  // coordinate search over the queue-check interval and the tail threshold; wall time of the
  // plain event form on the listed problems, best of 2
  sg_event_tuning cur = b->plainTune;
  auto time_it = [&](const sg_event_tuning& t, double* ms) -> int {
    b->plainTune = t;
    double bestMs = 1e300;
    for (int r = 0; r < 2; ++r) {
      sg_batch_stats st{};
      int rc = sg_batch_run_plain(b, slots, n, SG_FORM_EVENT, &st);
      if (rc) return rc;
      bestMs = std::min(bestMs, st.run_ms);
    }
    *ms = bestMs;
    return SG_OK;
  };
  double curMs = 0.0;
  int rc = time_it(cur, &curMs);
  if (rc) return rc;
  const int rounds[] = {1, 2, 4, 8, 16};
  const int tmin[] = {0, 1024, 4096, 16384, 65536};
  const int tdiv[] = {8, 16, 64, 256};
  for (int pass = 0; pass < 3; ++pass) {
    std::vector<sg_event_tuning> cands;
    if (pass == 0) for (int v : rounds) { sg_event_tuning t = cur; t.rounds_per_check = v; cands.push_back(t); }
    if (pass == 1) for (int v : tmin) { sg_event_tuning t = cur; t.tail_min = v; cands.push_back(t); }
    if (pass == 2) for (int v : tdiv) { sg_event_tuning t = cur; t.tail_divisor = v; cands.push_back(t); }
    for (const auto& t : cands) {
      if (std::memcmp(&t, &cur, sizeof(t)) == 0) continue;
      double ms = 0.0;
      rc = time_it(t, &ms);
      if (rc) return rc;
      if (ms < curMs) { cur = t; curMs = ms; }
    }
  }
  b->plainTune = cur;
  for (int i = 0; i < n; ++i) {
    rc = clear_tally(b, slots[i]);
    if (rc) return rc;
  }
  BCK(cudaStreamSynchronize(b->stream));
  if (best) *best = cur;
  return SG_OK;
}

int32_t sg_batch_tally_size(sg_batch b, int32_t slot, int64_t* n_bins) {
  if (!b || !n_bins) return SG_ERR_BAD_ARG;
  int rc = check_slot(b, slot);
  if (rc) return rc;
  *n_bins = b->slots[slot].sp.n_bins;
  return SG_OK;
}

int32_t sg_batch_get_bins(sg_batch b, int32_t slot, double* bins, int64_t n) {
  if (!b || !bins) return SG_ERR_BAD_ARG;
  int rc = check_slot(b, slot);
  if (rc) return rc;
  const Slot& S = b->slots[slot];
  const long long N = S.sp.n_bins;
  if (n < N) return b->fail(SG_ERR_BAD_ARG, "batch: buffer smaller than the tally");
  if (N == 0) return SG_OK;
  if (!b->serving) BCK(cudaStreamSynchronize(b->stream));
  else {
    for (const Request& r : b->active)
      if (r.slot == slot) return b->fail(SG_ERR_STATE, "batch: the slot is an active request");
    for (const Wave& w : b->waves)
      for (const Request& q : w.closing)
        if (q.slot == slot) return b->fail(SG_ERR_STATE, "batch: the slot's request is still in flight");
  }
  // a completed request's score memory is final: read it on the read-back stream, beside running waves
  cudaStream_t r = b->rstream;
  BCK(cudaMemcpyAsync(bins, S.tl.bin, N * sizeof(double), cudaMemcpyDeviceToHost, r));
  BCK(cudaMemcpyAsync(bins + n, S.tl.csum, N * sizeof(double), cudaMemcpyDeviceToHost, r));
  BCK(cudaMemcpyAsync(bins + 2 * n, S.tl.csum2, N * sizeof(double), cudaMemcpyDeviceToHost, r));
  BCK(cudaStreamSynchronize(r));
  return SG_OK;
}

int32_t sg_batch_clear_tally(sg_batch b, int32_t slot) {
  if (!b) return SG_ERR_BAD_ARG;
  int rc = check_slot(b, slot);
  if (rc) return rc;
  rc = clear_tally(b, slot);
  if (rc) return rc;
  BCK(cudaStreamSynchronize(b->stream));
  return SG_OK;
}

// ------------------------------------------------------------------ serving

double sg_serve_clock(void) { return host_now(); }

int32_t sg_serve_start(sg_batch b, int64_t wave_histories, int32_t item_histories) {
  if (!b || wave_histories < 32 || item_histories < 0 || (item_histories > 0 && item_histories < 32))
    return SG_ERR_BAD_ARG;
  if (b->serving) return b->fail(SG_ERR_STATE, "serve: already started");
  b->serving = true;
  b->waveHist = wave_histories;
  b->servedEvents = b->servedHistories = 0;
  b->serveItem = item_histories > 0 ? item_histories : b->tune.item_histories;
  b->wavesLaunched = 0;
  b->mirror = 0;
  if (!b->ref) BCK(cudaEventCreate(&b->ref));
  // map device event time onto the host clock: record, wait, read the host clock
  BCK(cudaEventRecord(b->ref, b->stream));
  BCK(cudaEventSynchronize(b->ref));
  b->refHost = host_now();
  return SG_OK;
}

int32_t sg_serve_submit(sg_batch b, int32_t slot) {
  if (!b) return SG_ERR_BAD_ARG;
  if (!b->serving) return b->fail(SG_ERR_STATE, "serve: call sg_serve_start first");
  int rc = check_slot(b, slot);
  if (rc) return rc;
  for (const Request& r : b->active)
    if (r.slot == slot) return b->fail(SG_ERR_STATE, "serve: the slot is already an active request");
  for (const Wave& w : b->waves)
    for (const Request& q : w.closing)
      if (q.slot == slot) return b->fail(SG_ERR_STATE, "serve: the slot's previous request is still in flight");
  const Slot& S = b->slots[slot];
  BCK(cudaMemsetAsync(b->arena + S.tallyOff, 0, S.tallyBytes, b->stream));
  Request r;
  r.slot = slot;
  r.next = 0;
  r.total = (long long)S.pop * S.cycles;
  r.submit = host_now();
  b->active.push_back(r);
  return SG_OK;
}

namespace {

// Retires the oldest in-flight wave (waiting for it when `block`).  Its closing requests complete
// at the wave's device end time, mapped onto the host clock through the reference event.
int retire_wave(sg_batch b, bool block, bool* retired) {
  *retired = false;
  if (b->waves.empty()) return SG_OK;
  Wave& w = b->waves.front();
  if (!block) {
    cudaError_t q = cudaEventQuery(w.done);
    if (q == cudaErrorNotReady) return SG_OK;
    if (q != cudaSuccess) return b->fail(SG_ERR_CUDA, std::string("serve: ") + cudaGetErrorString(q));
  } else {
    BCK(cudaEventSynchronize(w.done));
  }
  float ms = 0.f;
  BCK(cudaEventElapsedTime(&ms, b->ref, w.done));
  const double at = b->refHost + 1e-3 * (double)ms;
  int rc = read_counters(b, w.mirror);
  b->servedEvents += (long long)b->hCtr[w.mirror]->events;
  b->servedHistories += w.histories;
  for (const Request& r : w.closing) {
    b->doneSlots.push_back(r.slot);
    b->doneLat.push_back(std::max(0.0, at - r.submit));
  }
  cudaEventDestroy(w.done);
  b->waves.pop_front();
  *retired = true;
  return rc;
}

// Builds and launches one wave: every active request gets an equal share of the wave's histories
// (whole work items; what a request cannot use goes to the others), oldest request first.
int launch_wave(sg_batch b) {
  const int m = (int)(b->wavesLaunched & 1);
  const int item = b->serveItem;
  std::vector<WorkItem> items;
  Wave w;
  w.mirror = m;
  long long budget = b->waveHist;
  int maxl = 2;
  bool lean = true;
  std::vector<long long> take(b->active.size(), 0);
  // water-filling of the budget over the remaining work of the active requests
  for (int round = 0; round < 8 && budget > 0; ++round) {
    int open = 0;
    for (size_t i = 0; i < b->active.size(); ++i)
      if (b->active[i].total - b->active[i].next - take[i] > 0) ++open;
    if (!open) break;
    long long share = std::max<long long>(item, (budget / open + item - 1) / item * item);
    for (size_t i = 0; i < b->active.size() && budget > 0; ++i) {
      const long long left = b->active[i].total - b->active[i].next - take[i];
      if (left <= 0) continue;
      const long long t = std::min(std::min(left, share), std::max<long long>(budget, item));
      take[i] += t;
      budget -= t;
    }
  }
  std::deque<Request> still;
  for (size_t i = 0; i < b->active.size(); ++i) {
    Request& r = b->active[i];
    if (take[i] > 0) {
      if ((long long)items.size() + (take[i] + item - 1) / item > b->cfg.max_work_items) { still.push_back(r); continue; }
      cut_items(items, r.slot, r.next, r.next + take[i], item);
      r.next += take[i];
      w.histories += take[i];
      maxl = std::max(maxl, b->slots[r.slot].sp.maxl);
      lean = lean && slot_lean(b->slots[r.slot]);
    }
    if (r.next >= r.total) w.closing.push_back(r);
    else still.push_back(r);
  }
  if (items.empty() && w.closing.empty()) return SG_OK;
  b->active.swap(still);
  std::memcpy(b->hItems[m], items.data(), sizeof(WorkItem) * items.size());
  b->hInts[m][0] = (int)items.size();
  b->hInts[m][1] = 0;
  b->hInts[m][2] = (int)w.closing.size();
  b->hInts[m][3] = 0;
  for (size_t i = 0; i < w.closing.size(); ++i) b->hClose[m][i] = w.closing[i].slot;
  // wave k runs on stream m = k mod 2, after everything the batch stream has queued (instances,
  // tally clears); its closes run on the close stream once its own kernel and the previous wave's
  // have ended (a request's earlier histories may be in the previous wave)
  BCK(cudaEventRecord(b->upl, b->stream));
  BCK(cudaStreamWaitEvent(b->ws[m], b->upl, 0));
  int rc = launch_graph(b, m, maxl, lean, b->ws[m]);
  if (rc) return rc;
  BCK(cudaEventRecord(b->kdone[m], b->ws[m]));
  BCK(cudaStreamWaitEvent(b->cstream, b->kdone[m], 0));
  if (b->wavesLaunched > 0) BCK(cudaStreamWaitEvent(b->cstream, b->kdone[1 - m], 0));
  rc = run_closes(b, m, b->cstream);
  if (rc) return rc;
  BCK(cudaEventCreate(&w.done));
  BCK(cudaEventRecord(w.done, b->cstream));
  // the next wave on stream m rewrites this set's lists and counters: after these closes read them
  BCK(cudaStreamWaitEvent(b->ws[m], w.done, 0));
  b->waves.push_back(std::move(w));
  b->wavesLaunched += 1;
  return SG_OK;
}

}  // namespace

int32_t sg_serve_pump(sg_batch b, int32_t wait, int32_t* done_slots, double* latency_s, int32_t cap, int32_t* n_done) {
  if (!b || !n_done || cap < 0 || (cap > 0 && (!done_slots || !latency_s))) return SG_ERR_BAD_ARG;
  if (!b->serving) return b->fail(SG_ERR_STATE, "serve: call sg_serve_start first");
  *n_done = 0;
  bool retired = true;
  int rc;
  while (retired) {                         // everything that has finished
    rc = retire_wave(b, false, &retired);
    if (rc) return rc;
  }
  while (b->waves.size() < 2 && !b->active.empty()) {   // keep two waves in flight
    const long long before = b->wavesLaunched;
    rc = launch_wave(b);
    if (rc) return rc;
    if (b->wavesLaunched == before) break;
  }
  if (wait && !b->waves.empty() && b->doneSlots.empty()) {
    rc = retire_wave(b, true, &retired);
    if (rc) return rc;
    while (b->waves.size() < 2 && !b->active.empty()) {
      const long long before = b->wavesLaunched;
      rc = launch_wave(b);
      if (rc) return rc;
      if (b->wavesLaunched == before) break;
    }
  }
  const int k = std::min<int>(cap, (int)b->doneSlots.size());
  for (int i = 0; i < k; ++i) {
    done_slots[i] = b->doneSlots[i];
    latency_s[i] = b->doneLat[i];
  }
  b->doneSlots.erase(b->doneSlots.begin(), b->doneSlots.begin() + k);
  b->doneLat.erase(b->doneLat.begin(), b->doneLat.begin() + k);
  *n_done = k;
  return SG_OK;
}

int32_t sg_serve_stop(sg_batch b) {
  if (!b) return SG_ERR_BAD_ARG;
  bool retired = true;
  while (!b->waves.empty()) {
    int rc = retire_wave(b, true, &retired);
    if (rc) return rc;
  }
  b->serving = false;
  b->active.clear();
  b->doneSlots.clear();
  b->doneLat.clear();
  return SG_OK;
}

int32_t sg_serve_status(sg_batch b, int64_t* queued, int32_t* active, int64_t* waves) {
  if (!b) return SG_ERR_BAD_ARG;
  long long q = 0;
  for (const Request& r : b->active) q += r.total - r.next;
  if (queued) *queued = q;
  if (active) *active = (int32_t)b->active.size();
  if (waves) *waves = b->wavesLaunched;
  return SG_OK;
}

int32_t sg_serve_share(sg_batch b, int32_t blocks_per_sm, int32_t on) {
  if (!b || blocks_per_sm < 0) return SG_ERR_BAD_ARG;
  if (b->reserve != blocks_per_sm) {
    // a new reserve size: the reserving graphs are rebuilt at their next launch
    for (auto& plane : b->graph)
      for (auto& row : plane) drop_graph(row[1]);
    b->reserve = blocks_per_sm;
  }
  b->reserving = (on && blocks_per_sm > 0) ? 1 : 0;
  return SG_OK;
}

int32_t sg_serve_counts(sg_batch b, int64_t* histories, int64_t* events) {
  if (!b) return SG_ERR_BAD_ARG;
  if (histories) *histories = b->servedHistories;
  if (events) *events = b->servedEvents;
  return SG_OK;
}

}  // extern "C"
