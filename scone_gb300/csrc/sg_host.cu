// sg_host.cu -- host implementation of the C ABI in include/scone_gpu.h.
//
// One handle owns one CUDA stream, the resident geometry / MG data / tally memory and two particle
// banks sized by sg_config.max_bank.  Each eigenvalue cycle runs as: start-weight reduction ->
// history-loop kernel -> brood-ordered site scatter -> end-weight reduction -> tally close ->
// population control, with one host synchronisation (to learn the number of fission sites).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <functional>
#include <type_traits>

#include "sg_device.cuh"
#include "sg_launch.h"
#include "sg_source.cuh"
#include "sg_support.h"
#include "sg_noalloc.h"
#include "sg_batch.h"

using namespace sg;

namespace {

const double INF = 9223372036854775808.0;
const double SURF_TOL = 1.0e-12;          // universalVariables.f90:23
const double NUDGE = 1.0e-8;              // universalVariables.f90:25
const double FP_REL_TOL = 1.0e-7;
// mixed form: tolerances sized to FP32 distance accuracy (a crossing lands within ~1e-7 |d|)
const double SURF_TOL_M = 4.0e-6;
const double NUDGE_M = 1.0e-4;

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) return h->fail(SG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// While a Staging is installed on the calling thread, DArr takes its memory from a caller-owned
// device block instead of cudaMalloc and writes uploads into that block's host image; the caller
// commits the image with one copy.  `dev` null measures: offsets are counted, nothing is written.
struct Staging {
  char* dev = nullptr;
  std::vector<char>* host = nullptr;
  size_t used = 0;
  size_t cap = 0;
};
thread_local Staging* t_staging = nullptr;

template <class T>
struct DArr {
  T* p = nullptr;
  size_t n = 0;
  bool borrowed = false;
  cudaError_t alloc(size_t count) {
    free();
    n = count;
    if (count == 0) return cudaSuccess;
    if (Staging* st = t_staging) {
      const size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
      if (st->dev && st->used + bytes > st->cap) return cudaErrorMemoryAllocation;
      p = reinterpret_cast<T*>((st->dev ? st->dev : reinterpret_cast<char*>(256)) + st->used);
      st->used += bytes;
      if (st->dev && st->host) st->host->resize(st->used, 0);
      borrowed = true;
      return cudaSuccess;
    }
    return cudaMalloc((void**)&p, count * sizeof(T));
  }
  cudaError_t upload(const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = alloc(v.size() ? v.size() : 1);
    if (e != cudaSuccess) return e;
    if (v.empty()) return cudaSuccess;
    if (borrowed) {
      Staging* st = t_staging;
      if (st && st->dev && st->host)
        std::memcpy(st->host->data() + (reinterpret_cast<char*>(p) - st->dev), v.data(), v.size() * sizeof(T));
      return cudaSuccess;
    }
    e = cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
  }
  void free() {
    if (p && !borrowed) cudaFree(p);
    p = nullptr;
    n = 0;
    borrowed = false;
  }
};

struct BankBufs {
  DArr<double> r, dir, wgt, time, E;
  DArr<int> G, brood;
  cudaError_t alloc(size_t cap) {
    cudaError_t e;
    if ((e = r.alloc(3 * cap)) || (e = dir.alloc(3 * cap)) || (e = wgt.alloc(cap)) || (e = time.alloc(cap)) ||
        (e = G.alloc(cap)) || (e = brood.alloc(cap)))
      return e;
    return cudaSuccess;
  }
  DBank view() { return DBank{r.p, dir.p, wgt.p, G.p, brood.p, time.p, E.p}; }
  void free() { r.free(); dir.free(); wgt.free(); time.free(); G.free(); brood.free(); E.free(); }
};

struct Admin {
  std::vector<sg_clerk_desc> clerks;
  std::vector<long long> addr;   // 1-based within the admin
  long long N = 0;
  long long off = 0;             // offset of bin 1 in the handle's tally arrays
  int batchSize = 1, cycles = 0, batchN = 0;
  long long normAddr = -1;
  double normVal = 1.0;
  int atch = -1;
  long long keffAnalog = -1, keffImplicit = -1;   // 0-based admin-relative addresses
  // per clerk and axis ([3 * clerk + axis]): device table of an unstructured grid (FP64 and FP32
  // copies) or of a cell axis (int, both entries), null otherwise
  std::vector<const void*> tab64, tab32;
  bool lastCycle() const { return (cycles + 1) % batchSize == 0; }
};

}  // namespace

struct sg_handle_t {
  sg_config cfg;
  double htCutoff = 0.9;       // transportOperatorHT `cutoff` (transportOperatorHT_class.f90:297)
  cudaStream_t stream = nullptr;
  std::string err;

  // geometry
  bool hasGeom = false;
  int maxl = 4;
  double bounds[6];
  DArr<DSurf> surfs64, surfsMx;
  DArr<DUni> unis64, unisMx;
  DArr<int> uniCells, cellPtr, cellSurf, cellComplex;
  DArr<double> rot64;           // rotation matrices of the universes (when any is rotated)
  DArr<float> rotF;
  DArr<double> pinRsq, pinTol64, pinTolMx;
  DArr<float> pinRsqF, pinTolF;
  DArr<int2> graph;
  std::vector<int2> graphHost;   // host copy of the graph (majorant materials)
  DGeom g64{}, gMx{};

  // MG data
  bool hasMG = false;
  bool anyFissile = false;
  int nMat = 0, nG = 0;
  DArr<double> mgD[11];
  DArr<float> mgF[11];
  DArr<int> fissile;
  DMG<double> mg64{};
  DMG<float> mgMx{};

  // continuous-energy data
  bool hasCE = false;
  DArr<double> ceE, ceUE;
  DArr<double> ceXs64, ceA64, ceKT64, ceDens64, ceMaj64;
  DArr<float> ceXsF, ceAF, ceKTF, ceDensF, ceMajF;
  DArr<long long> ceOff;
  DArr<int2> ceHash, ceUHash, ceLUHash;
  DArr<double> ceLU;
  DArr<int> ceLIdx, ceLMaj;
  DArr<int> ceMatPtr, ceMatNuc, ceAct;
  DCE<double> ce64{};
  DCE<float> ceMx{};

  // tallies
  std::vector<Admin> admins;
  std::vector<DArr<double>> mapTab64;   // map tables of the admins (unstructured bounds, cell bins)
  std::vector<DArr<float>> mapTab32;
  std::vector<DArr<int>> mapTabCell;
  int nCell = 0;                        // cells of the uploaded geometry
  // collision processor variant (neutronMGimp / neutronCEimp) and its weight-window field
  bool collImp = false, collBuf = false;   // collBuf: splitting or weight windows (split buffer)
  Admin wwAdmin;                           // tables of the weight-window map
  DArr<double> wwLo64, wwUp64;
  DArr<float> wwLo32, wwUp32;
  DColl<double> hColl64{};
  DColl<float> hColl32{};
  DArr<DColl<double>> dColl64;
  DArr<DColl<float>> dColl32;
  DArr<double> bufR, bufE;                 // split buffer (the handle's precision)
  DArr<double> bufU64, bufW64, bufT64;
  DArr<float> bufU32, bufW32, bufT32;
  DArr<int> bufG;
  long long totalBins = 0;
  DArr<double> acc, bin, csum, csum2;

  // banks and work buffers
  int cap = 0;
  BankBufs bank[2];
  int cur = 0;                 // index of the "this cycle" bank
  DArr<double> sR, sDir, sWgt, sTime;
  DArr<int> sG, sBrood, sSeq, sCursor;
  int regionCap = 0;
  DArr<int> histN, start, scanTmp, flags, pos, kbuf;
  DArr<unsigned long long> keys, sel, winCnt, winCand;
  DArr<unsigned long long> shardKeys;   // sg_normalise_shard: the draws of all processes' sites
  DArr<unsigned int> hist16;
  DArr<double> sumPart, scal;  // scal: 0 k_eff, 1 k_new, 2 start weight, 3 end weight, 4 k_end
  DArr<int> totals;            // 0 sites total, 1 kept total, 2 dup total, 3 error
  DArr<DCounters> ctr;
  DArr<int> recColl;
  DArr<unsigned long long> recRng;
  // event form: particle state (sized for FP64 and 4 levels), queues and their counters
  DArr<double> pR0, pRl, pU, pW, pW0, pTime, pTrack;
  DArr<int> pGeo, pInts, qT0, qT1, qC, qCtr;
  DArr<double> pE;
  DArr<unsigned long long> pRng;
  int evIterations = 0;
  sg_event_tuning evTune{4, 4096, 64};   // rounds per queue check, tail threshold (min, divisor)
  int lastN = 0;
  long long launches = 0;      // kernels launched since the last reset (cycle stats)
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaStream_t copyStream = nullptr;   // second stream of the bank copies back to the host
  cudaEvent_t copyEv[2] = {nullptr, nullptr};
  float lastTransportMs = 0.f;
  sg_cycle_stats lastStats{};   // the last eigenvalue cycle's statistics

  // point source
  bool hasSource = false;
  PointSourceArgs psrc{};
  // file source (fileSource): the particle table on the device
  bool hasFileSource = false;
  long long fileN = 0;
  DArr<double> fsR, fsDir, fsWgt, fsE;
  DArr<int> fsG;
  DArr<double> probG;

  // eigen state
  bool eigenReady = false;
  int pop = 0;
  unsigned long long master = 0;
  double k = 1.0;

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
};

namespace {

unsigned long long rng_stride(unsigned long long s, long long n) { return lcg_skip(s, 152917LL * n); }

// rotationMatrix (genericProcedures.f90:1098-1140): Euler angles phi, theta, psi in degrees, ZXZ
// convention; m row-major
void rotation_matrix(double phi, double theta, double psi, double m[9]) {
  const double conv = 2.0 * 3.14159265358979323846264338327950288 / 360.0;
  const double sf = std::sin(phi * conv), cf = std::cos(phi * conv);
  const double st = std::sin(theta * conv), ct = std::cos(theta * conv);
  const double sp = std::sin(psi * conv), cp = std::cos(psi * conv);
  m[0] = cp * cf - ct * sf * sp;
  m[1] = cp * sf + ct * cf * sp;
  m[2] = sp * sf;
  m[3] = -sp * cf - ct * sf * cp;
  m[4] = -sp * sf + ct * cf * cp;
  m[5] = cp * st;
  m[6] = st * sf;
  m[7] = -st * cf;
  m[8] = ct;
}

// ------------------------------------------------------------------ unionCell
// unionCell%init (Geometry/Cells/unionCell_class.f90:80-199): the token list of a cell becomes its
// evaluation array.  Implicit intersections are inserted (after a surface or a closing bracket,
// before a surface, an opening bracket or a complement); complements are removed by De Morgan's law
// (deMorgan, :202-262: the complemented surface or bracket flips every surface's sense and swaps
// unions and intersections); mixed unions and intersections without brackets are rejected
// (checkPrecedence, :267-305).  A list without operators is a simpleCell and is kept as it is.
bool cell_eval_array(const std::vector<int>& in, int ns, std::vector<int>& a, bool& complex_, std::string& why) {
  const int COMPLEM = SG_CELL_COMPLEMENT;
  bool hasOp = false;
  for (int t : in) {
    if (t == SG_CELL_OPEN || t == SG_CELL_CLOSE || t == SG_CELL_UNION || t == SG_CELL_COMPLEMENT) hasOp = true;
    else if (t == 0 || std::abs(t) > ns) { why = "bad surface index"; return false; }
  }
  complex_ = false;
  if (!hasOp) { a = in; return true; }
  a.clear();
  bool surfPrev = false, closePrev = false;
  int depth = 0;
  for (int t : in) {
    if (t == SG_CELL_OPEN) {
      depth += 1;
      if (surfPrev || closePrev) a.push_back(CELL_INTERSECT);
      a.push_back(CELL_OPEN);
      closePrev = false;
      surfPrev = false;
    } else if (t == SG_CELL_CLOSE) {
      depth -= 1;
      a.push_back(CELL_CLOSE);
      closePrev = true;
      surfPrev = false;
    } else if (t == SG_CELL_UNION) {
      a.push_back(CELL_UNION);
      closePrev = false;
      surfPrev = false;
    } else if (t == SG_CELL_COMPLEMENT) {
      if (surfPrev || closePrev) a.push_back(CELL_INTERSECT);
      a.push_back(COMPLEM);
      closePrev = false;
      surfPrev = false;
    } else {
      if (surfPrev || closePrev) a.push_back(CELL_INTERSECT);
      a.push_back(t);
      surfPrev = true;
      closePrev = false;
    }
  }
  if (depth != 0) { why = "inconsistent use of parentheses"; return false; }
  if (a.empty() || a.back() == CELL_UNION) { why = "definition ends with a union"; return false; }
  if (a.back() == COMPLEM) { why = "definition ends with a complement"; return false; }
  for (size_t i = 0; i + 1 < a.size(); ++i) {            // De Morgan
    if (a[i] != COMPLEM) continue;
    a.erase(a.begin() + i);
    size_t endPos = i;
    if (a[i] == CELL_OPEN) {
      int d = 1;
      size_t j = i + 1;
      for (; j < a.size(); ++j) {
        if (a[j] == CELL_OPEN) d += 1;
        else if (a[j] == CELL_CLOSE) d -= 1;
        if (d == 0) break;
      }
      endPos = std::min(j, a.size() - 1);
    }
    for (size_t j = i; j <= endPos; ++j) {
      if (!cell_is_op(a[j]) && a[j] != COMPLEM) a[j] = -a[j];
      else if (a[j] == CELL_UNION) a[j] = CELL_INTERSECT;
      else if (a[j] == CELL_INTERSECT) a[j] = CELL_UNION;
    }
  }
  for (size_t i = 0; i + 1 < a.size();) {                // precedence
    const int e1 = a[i];
    if (e1 == CELL_UNION || e1 == CELL_INTERSECT) {
      size_t j = i + 1, next = i + 1;
      for (; j < a.size(); ++j) {
        const int e2 = a[j];
        if (e2 == CELL_UNION || e2 == CELL_INTERSECT) {
          if (e2 != e1) { why = "the order of operations is ambiguous"; return false; }
          next = j;
          break;
        }
        if (e2 == CELL_OPEN || e2 == CELL_CLOSE) { next = j + 1; break; }
      }
      if (j == a.size()) next = i + 1;
      i = next;
      continue;
    }
    i += 1;
  }
  for (int t : a) if (t == CELL_UNION) complex_ = true;
  if (!complex_) {                                      // repeated surfaces of an intersection-only cell
    std::vector<int> ids;
    for (int t : a) if (!cell_is_op(t)) ids.push_back(std::abs(t));
    std::sort(ids.begin(), ids.end());
    if (std::adjacent_find(ids.begin(), ids.end()) != ids.end()) { why = "repeated surfaces in a cell"; return false; }
  }
  return true;
}

// ------------------------------------------------------------------ geometry build
int build_geometry(sg_handle h, const sg_geometry_desc* g) {
  const int ns = g->n_surf, nu = g->n_uni;
  if (ns <= 0 || nu <= 0 || g->root_uni < 0 || g->root_uni >= nu || g->border_surf < 0 || g->border_surf >= ns)
    return h->fail(SG_ERR_BAD_ARG, "geometry: bad counts or root/border index");
  std::vector<DSurf> s64(ns), sMx(ns);
  auto fill_surf = [&](DSurf& s, int type, const double* par, bool mixed) -> bool {
    std::memset(&s, 0, sizeof(s));
    s.type = type;
    for (int i = 0; i < SG_SURF_NPAR; ++i) s.p[i] = par[i];
    s.axis = 2; s.pl0 = 0; s.pl1 = 1;
    switch (type) {
      case SG_SURF_XPLANE: s.axis = 0; break;
      case SG_SURF_YPLANE: s.axis = 1; break;
      case SG_SURF_ZPLANE: s.axis = 2; break;
      case SG_SURF_XCYL: case SG_SURF_XSQCYL: s.axis = 0; s.pl0 = 1; s.pl1 = 2; break;
      case SG_SURF_YCYL: case SG_SURF_YSQCYL: s.axis = 1; s.pl0 = 0; s.pl1 = 2; break;
      case SG_SURF_ZCYL: case SG_SURF_ZSQCYL: s.axis = 2; s.pl0 = 0; s.pl1 = 1; break;
      case SG_SURF_PLANE: case SG_SURF_SPHERE: case SG_SURF_BOX: break;
      default: return false;
    }
    if (type == SG_SURF_PLANE) {   // plane_class.f90:78-84, gfortran NORM2 of coefficients 1-3
      double scale = 1.0, ssq = 0.0;
      for (int i = 0; i < 3; ++i)
        if (par[i] != 0.0) {
          double a = std::fabs(par[i]);
          if (scale < a) { double t = scale / a; ssq = 1.0 + ssq * t * t; scale = a; }
          else { double t = a / scale; ssq = ssq + t * t; }
        }
      double n = scale * std::sqrt(ssq);
      for (int i = 0; i < 4; ++i) s.p[i] = par[i] / n;
    }
    const bool curved = type == SG_SURF_XCYL || type == SG_SURF_YCYL || type == SG_SURF_ZCYL || type == SG_SURF_SPHERE;
    if (!mixed) s.tol = curved ? 2.0 * s.p[3] * SURF_TOL : SURF_TOL;   // cylinder :181, sphere :107
    else {
      double scale = 1.0;
      if (type == SG_SURF_XPLANE || type == SG_SURF_YPLANE || type == SG_SURF_ZPLANE) scale = std::max(1.0, std::fabs(s.p[0]));
      else if (type == SG_SURF_PLANE) scale = std::max(1.0, std::fabs(s.p[3]));
      else if (!curved) for (int i = 0; i < 3; ++i) scale = std::max(scale, std::fabs(s.p[i]) + std::fabs(s.p[3 + i]));
      s.tol = curved ? 2.0 * s.p[3] * SURF_TOL_M : SURF_TOL_M * scale;
    }
    for (int i = 0; i < SG_SURF_NPAR; ++i) s.pf[i] = (float)s.p[i];
    s.tolf = (float)s.tol;
    return true;
  };
  for (int i = 0; i < ns; ++i) {
    if (!fill_surf(s64[i], g->surf_type[i], g->surf_par + SG_SURF_NPAR * i, false) ||
        !fill_surf(sMx[i], g->surf_type[i], g->surf_par + SG_SURF_NPAR * i, true))
      return h->fail(SG_ERR_BAD_ARG, "geometry: unknown surface type");
  }
  for (int i = 0; i < 6; ++i) {
    if (g->bc[i] < 0 || g->bc[i] > 2) return h->fail(SG_ERR_BAD_ARG, "geometry: bad boundary condition");
    s64[g->border_surf].bc[i] = g->bc[i];
    sMx[g->border_surf].bc[i] = g->bc[i];
  }
  // cells: simpleCell surface lists, or unionCell token lists turned into their evaluation arrays
  std::vector<int> cptr(1, 0), csurf, ccomplex(g->n_cell, 0);
  bool anyComplex = false;
  for (int c = 0; c < g->n_cell; ++c) {
    std::vector<int> in(g->cell_surf + g->cell_ptr[c], g->cell_surf + g->cell_ptr[c + 1]), ev;
    bool cx = false;
    std::string why;
    if (!cell_eval_array(in, ns, ev, cx, why))
      return h->fail(SG_ERR_BAD_ARG, "geometry: cell " + std::to_string(c) + ": " + why);
    csurf.insert(csurf.end(), ev.begin(), ev.end());
    cptr.push_back((int)csurf.size());
    ccomplex[c] = cx ? 1 : 0;
    anyComplex |= cx;
  }
  // universes
  std::vector<DUni> u64(nu), uMx(nu);
  std::vector<double> rotM(9 * (size_t)nu, 0.0);
  bool anyRot = false;
  std::vector<std::vector<int>> fills(nu);
  std::vector<int> uniCells;
  std::vector<double> rsq, tol64, tolMx;
  for (int u = 0; u < nu; ++u) {
    DUni U;
    std::memset(&U, 0, sizeof(U));
    U.type = g->uni_type[u];
    for (int i = 0; i < 3; ++i) U.origin[i] = g->uni_origin[3 * u + i];
    std::vector<int> ip(g->uni_ipar + g->uni_iptr[u], g->uni_ipar + g->uni_iptr[u + 1]);
    std::vector<double> dp(g->uni_dpar + g->uni_dptr[u], g->uni_dpar + g->uni_dptr[u + 1]);
    std::vector<int> f(g->uni_fill + g->uni_fptr[u], g->uni_fill + g->uni_fptr[u + 1]);
    DUni Um = U;
    switch (U.type) {
      case SG_UNI_ROOT:                          // rootUniverse_class.f90:100-119: fills [inside, OUTSIDE]
        if (ip.size() != 1 || f.size() != 1) return h->fail(SG_ERR_BAD_ARG, "root universe: ipar/fill");
        if (U.origin[0] != 0.0 || U.origin[1] != 0.0 || U.origin[2] != 0.0)
          return h->fail(SG_ERR_BAD_ARG, "root universe: origin offset is not supported");
        U.i[0] = ip[0];
        f.push_back(0);
        break;
      case SG_UNI_CELL:                          // cellUniverse_class.f90:145-151: + UNDEF, OVERLAP
        if (ip.size() != f.size()) return h->fail(SG_ERR_BAD_ARG, "cell universe: cells/fills mismatch");
        U.i[0] = (int)uniCells.size();
        U.i[1] = (int)ip.size();
        for (int c : ip) {
          if (c < 0 || c >= g->n_cell) return h->fail(SG_ERR_BAD_ARG, "cell universe: bad cell index");
          uniCells.push_back(c);
        }
        f.push_back(SG_UNDEF_MAT);
        f.push_back(SG_OVERLAP_MAT);
        break;
      case SG_UNI_PIN: {                         // pinUniverse_class.f90:76-139
        int N = (int)dp.size() + 1;
        if ((int)f.size() != N) return h->fail(SG_ERR_BAD_ARG, "pin universe: radii/fills mismatch");
        U.i[0] = (int)rsq.size();
        U.i[1] = N;
        for (int i = 0; i < N; ++i) {
          double rad = (i < N - 1) ? dp[i] : INF * 1.1;
          if (i < N - 1 && (rad <= 0.0 || (i > 0 && rad <= dp[i - 1])))
            return h->fail(SG_ERR_BAD_ARG, "pin universe: radii must be positive and ascending");
          rsq.push_back(rad * rad);
          tol64.push_back(2.0 * rad * SURF_TOL);
          tolMx.push_back(2.0 * rad * SURF_TOL_M);
        }
        break;
      }
      case SG_UNI_LAT: {                         // latUniverse_class.f90:113-260
        if (ip.size() < 3 || dp.size() != 3) return h->fail(SG_ERR_BAD_ARG, "lattice: shape/pitch");
        int sizeN[3] = {ip[0], ip[1], ip[2]};
        double pitch[3] = {dp[0], dp[1], dp[2]};
        if (sizeN[2] == 0) { sizeN[2] = 1; pitch[2] = 2.0 * INF; }
        if (sizeN[0] <= 0 || sizeN[1] <= 0) return h->fail(SG_ERR_BAD_ARG, "lattice: zero shape");
        int nloc = sizeN[0] * sizeN[1] * sizeN[2] + 1;
        if ((int)f.size() != nloc) return h->fail(SG_ERR_BAD_ARG, "lattice: fills must be nx*ny*nz + 1");
        for (int i = 0; i < 3; ++i) {
          U.i[i] = sizeN[i];
          U.d[i] = pitch[i];
          U.d[3 + i] = -(sizeN[i] * 0.5 * pitch[i]);
          U.d[6 + i] = pitch[i] * 0.5 - pitch[i] * SURF_TOL;
        }
        U.i[3] = nloc;
        U.i[5] = (ip.size() > 3) ? (ip[3] != 0) : 1;
        // outline box (latUniverse_class.f90:176-183) appended as an extra surface
        double par[SG_SURF_NPAR] = {0, 0, 0, std::fabs(U.d[3]), std::fabs(U.d[4]), std::fabs(U.d[5])};
        DSurf o64, oMx;
        fill_surf(o64, SG_SURF_BOX, par, false);
        fill_surf(oMx, SG_SURF_BOX, par, true);
        U.i[4] = (int)s64.size();
        s64.push_back(o64);
        sMx.push_back(oMx);
        break;
      }
      default:
        return h->fail(SG_ERR_BAD_ARG, "geometry: unknown universe type");
    }
    if (g->uni_rot) {                            // universe%setTransform (universe_inter.f90:358-375)
      const double* a = g->uni_rot + 3 * u;
      if (!(a[0] == 0.0 && a[1] == 0.0 && a[2] == 0.0)) {
        if (U.type == SG_UNI_ROOT) return h->fail(SG_ERR_BAD_ARG, "root universe: rotation is not supported");
        if (!(a[0] >= 0.0 && a[0] < 360.0) || !(a[1] >= 0.0 && a[1] <= 180.0) || !(a[2] >= 0.0 && a[2] < 360.0))
          return h->fail(SG_ERR_BAD_ARG, "universe rotation: angles must be phi, psi in [0,360), theta in [0,180]");
        rotation_matrix(a[0], a[1], a[2], &rotM[9 * (size_t)u]);
        U.rot = 1;
        anyRot = true;
      }
    }
    // level coordinates of an origin-free, unrotated universe equal those of the level above
    U.i[6] = (!U.rot && U.origin[0] == 0.0 && U.origin[1] == 0.0 && U.origin[2] == 0.0) ? 1 : 0;
    Um = U;
    if (U.type == SG_UNI_LAT)
      for (int i = 0; i < 3; ++i) Um.d[6 + i] = U.d[i] * 0.5 - U.d[i] * SURF_TOL_M;
    for (int i = 0; i < 3; ++i) { U.originf[i] = (float)U.origin[i]; Um.originf[i] = (float)Um.origin[i]; }
    for (int i = 0; i < 9; ++i) { U.f[i] = (float)U.d[i]; Um.f[i] = (float)Um.d[i]; }
    if (U.type == SG_UNI_LAT) {
      for (int i = 0; i < 3; ++i) U.invf[i] = Um.invf[i] = (float)(1.0 / U.d[i]);
      for (int i = 0; i < 2; ++i) U.invn[i] = Um.invn[i] = (float)(1.0 / U.i[i]);
    }
    u64[u] = U;
    uMx[u] = Um;
    fills[u] = f;
  }
  // shrunk geomGraph (geomGraph_class.f90:172-232 layout; :309-345 unique IDs)
  std::vector<int> base(nu, -1);
  std::vector<int2> graph;
  auto layout = [&](int u) {
    base[u] = (int)graph.size() + 1;
    for (int f : fills[u]) graph.push_back(make_int2(f, 0));
  };
  layout(g->root_uni);
  for (size_t loc = 0; loc < graph.size(); ++loc) {
    int f = graph[loc].x;
    if (f < 0) {
      int u = -f - 1;
      if (u < 0 || u >= nu) return h->fail(SG_ERR_BAD_ARG, "geometry: fill names a missing universe");
      if (base[u] < 0) layout(u);
      graph[loc].y = base[u];
    }
  }
  int cells = 0;
  for (auto& e : graph) if (e.x > 0) e.y = ++cells;
  // nesting depth
  std::function<int(int, int)> depth = [&](int u, int d) -> int {
    if (d > SG_MAX_NEST) return d;
    int m = d;
    for (int f : fills[u]) if (f < 0) m = std::max(m, depth(-f - 1, d + 1));
    return m;
  };
  int dep = depth(g->root_uni, 1);
  if (dep > 4) return h->fail(SG_ERR_BAD_ARG, "geometry: nesting deeper than 4 levels is not supported");
  h->maxl = dep <= 2 ? 2 : (dep == 3 ? 3 : 4);
  // bounds (geometryStd_class.f90:186-205)
  {
    const DSurf& b = s64[g->border_surf];
    for (int i = 0; i < 3; ++i) { h->bounds[i] = -INF; h->bounds[3 + i] = INF; }
    if (b.type == SG_SURF_BOX) for (int i = 0; i < 3; ++i) { h->bounds[i] = b.p[i] - b.p[3 + i]; h->bounds[3 + i] = b.p[i] + b.p[3 + i]; }
    else if (b.type >= SG_SURF_XSQCYL) { int pl[2] = {b.pl0, b.pl1}; for (int i : pl) { h->bounds[i] = b.p[i] - b.p[3 + i]; h->bounds[3 + i] = b.p[i] + b.p[3 + i]; } }
    else if (b.type == SG_SURF_SPHERE) for (int i = 0; i < 3; ++i) { h->bounds[i] = b.p[i] - b.p[3]; h->bounds[3 + i] = b.p[i] + b.p[3]; }
    else if (b.type >= SG_SURF_XCYL && b.type <= SG_SURF_ZCYL) { int pl[2] = {b.pl0, b.pl1}; for (int i : pl) { h->bounds[i] = b.p[i] - b.p[3]; h->bounds[3 + i] = b.p[i] + b.p[3]; } }
    for (int i = 0; i < 3; ++i)
      if (h->bounds[i] <= -INF && h->bounds[3 + i] >= INF) { h->bounds[i] = 0.0; h->bounds[3 + i] = 0.0; }
  }
  // mixed form: FP32 filter of the root border test.  The FP32 value of the surface function at
  // float(r) differs from the FP64 value by at most a few FP32 ulps of the geometry scale (squared
  // for quadrics); beyond that bound plus the surface tolerance the FP64 test gives the same side.
  {
    double scale = 1.0;
    for (int i = 0; i < 6; ++i) scale = std::max(scale, std::fabs(h->bounds[i]));
    DSurf& b = sMx[g->border_surf];
    const bool quad = b.type == SG_SURF_SPHERE || (b.type >= SG_SURF_XCYL && b.type <= SG_SURF_ZCYL);
    const bool bounded = b.type == SG_SURF_SPHERE || b.type == SG_SURF_BOX || b.type >= SG_SURF_XCYL;
    const double ulp = 0x1p-24;
    const double err = quad ? 128.0 * ulp * scale * scale : 32.0 * ulp * scale;
    b.filt = bounded ? (float)(b.tol + err) : 0.0f;
  }
  cudaStream_t st = h->stream;
  CK(h->surfs64.upload(s64, st));
  CK(h->surfsMx.upload(sMx, st));
  CK(h->unis64.upload(u64, st));
  CK(h->unisMx.upload(uMx, st));
  CK(h->uniCells.upload(uniCells, st));
  CK(h->cellPtr.upload(cptr, st));
  CK(h->cellSurf.upload(csurf, st));
  if (anyComplex) CK(h->cellComplex.upload(ccomplex, st));
  else h->cellComplex.free();
  CK(h->pinRsq.upload(rsq, st));
  CK(h->pinTol64.upload(tol64, st));
  CK(h->pinTolMx.upload(tolMx, st));
  {
    std::vector<float> rf(rsq.size()), tf(tolMx.size());
    for (size_t i = 0; i < rsq.size(); ++i) rf[i] = (float)std::min(rsq[i], 1.0e38);
    for (size_t i = 0; i < tolMx.size(); ++i) tf[i] = (float)std::min(tolMx[i], 1.0e38);
    CK(h->pinRsqF.upload(rf, st));
    CK(h->pinTolF.upload(tf, st));
  }
  CK(h->graph.upload(graph, st));
  h->graphHost = graph;
  if (anyRot) {
    std::vector<float> rf(rotM.begin(), rotM.end());
    CK(h->rot64.upload(rotM, st));
    CK(h->rotF.upload(rf, st));
  } else {
    h->rot64.free();
    h->rotF.free();
  }
  // mixed-form tie tolerance: 16 FP32 ulps of the largest root coordinate
  double scale = 1.0;
  for (int i = 0; i < 6; ++i) scale = std::max(scale, std::fabs(h->bounds[i]));
  const double tie_abs = 16.0 * scale * 0x1p-23;
  const int* cx = anyComplex ? h->cellComplex.p : nullptr;
  h->g64 = DGeom{h->surfs64.p, h->unis64.p, h->uniCells.p, h->cellPtr.p, h->cellSurf.p, h->pinRsq.p,
                 h->pinTol64.p, h->pinRsqF.p, h->pinTolF.p, h->graph.p, g->root_uni, g->border_surf, NUDGE, 0.0, cx,
                 anyRot ? h->rot64.p : nullptr, anyRot ? h->rotF.p : nullptr};
  h->gMx = DGeom{h->surfsMx.p, h->unisMx.p, h->uniCells.p, h->cellPtr.p, h->cellSurf.p, h->pinRsq.p,
                 h->pinTolMx.p, h->pinRsqF.p, h->pinTolF.p, h->graph.p, g->root_uni, g->border_surf, NUDGE_M, tie_abs, cx,
                 anyRot ? h->rot64.p : nullptr, anyRot ? h->rotF.p : nullptr};
  h->nCell = g->n_cell;
  h->hasGeom = true;
  // active materials for the majorant
  return SG_OK;
}

std::vector<int> active_mats(sg_handle h, const std::vector<int2>& graph) {
  std::vector<int> a;
  for (auto& e : graph) if (e.x > 0 && e.x <= h->nMat) a.push_back(e.x);
  std::sort(a.begin(), a.end());
  a.erase(std::unique(a.begin(), a.end()), a.end());
  return a;
}

int build_mg(sg_handle h, const sg_mg_desc* d) {
  const int M = d->n_mat, nG = d->n_g;
  if (M <= 0 || nG <= 0) return h->fail(SG_ERR_BAD_ARG, "mg: bad sizes");
  if (!h->hasGeom) return h->fail(SG_ERR_STATE, "mg: upload the geometry first (majorant uses its materials)");
  h->nMat = M;
  h->nG = nG;
  const size_t MG = (size_t)M * nG;
  std::vector<double> total(MG), scatter(MG), capture(MG), fission(MG, 0), nuf(MG, 0), chi(MG, 0);
  std::vector<double> P0(MG * nG), prod(MG * nG);
  std::vector<int> fis(M);
  h->anyFissile = false;
  for (int m = 0; m < M; ++m) {
    fis[m] = d->fissile[m] ? 1 : 0;
    h->anyFissile |= fis[m] != 0;
    for (size_t k = (size_t)m * nG * nG; k < (size_t)(m + 1) * nG * nG; ++k) { P0[k] = d->p0[k]; prod[k] = d->prod[k]; }
    for (int gi = 0; gi < nG; ++gi) {
      size_t k = (size_t)m * nG + gi;
      double s = 0.0;                              // multiScatterMG: scatterXSs = sum(P0, 1)
      for (int go = 0; go < nG; ++go) s = s + P0[k * nG + go];
      scatter[k] = s;
      capture[k] = d->capture[k];
      if (fis[m]) { fission[k] = d->fission[k]; nuf[k] = d->nu[k] * d->fission[k]; }
      total[k] = scatter[k] + capture[k];          // baseMgNeutronMaterial_class.f90:282-289
      if (fis[m]) total[k] = total[k] + fission[k];
      if (!(total[k] > 0.0)) return h->fail(SG_ERR_BAD_ARG, "mg: non-positive total cross section");
    }
    if (fis[m]) {                                  // fissionMG_class.f90:262-268
      double S = 0.0;
      for (int g = 0; g < nG; ++g) S = S + d->chi[(size_t)m * nG + g];
      for (int g = 0; g < nG; ++g) {
        double c = d->chi[(size_t)m * nG + g];
        if (std::fabs(S - 1.0) > 0.01 * FP_REL_TOL) c = c / S;
        chi[(size_t)m * nG + g] = c;
      }
    }
  }
  std::vector<int> act = active_mats(h, h->graphHost);
  for (int a : act) if (a > M) return h->fail(SG_ERR_BAD_ARG, "mg: geometry uses a material beyond n_mat");
  std::vector<double> maj(nG, 0.0);                // initMajorant (baseMgNeutronDatabase :458-503)
  for (int g = 0; g < nG; ++g) {
    double xs = 0.0;
    for (int a : act) xs = std::max(xs, total[(size_t)(a - 1) * nG + g]);
    maj[g] = xs * 1.0;
  }
  // multiScatterP1MG buildFromDict (multiScatterP1MG_class.f90:96-128): 3 P1/P0 where P0 /= 0
  std::vector<double> P1n;
  if (d->p1) {
    P1n.assign(MG * nG, 0.0);
    for (size_t k = 0; k < MG * nG; ++k) {
      if (P0[k] != 0.0) P1n[k] = d->p1[k] / P0[k] * 3.0;
      if (!(std::fabs(P1n[k]) <= 3.0))                // sampleLegendre_P1 (legendrePoly_func.f90:62-63)
        return h->fail(SG_ERR_BAD_ARG, "mg: P1 must have absolute value below 3 P0");
    }
  }
  const std::vector<double>* src[10] = {&total, &scatter, &capture, &fission, &nuf, &chi, &P0, &prod, &maj, &P1n};
  const int nArr = d->p1 ? 10 : 9;
  cudaStream_t st = h->stream;
  h->mgD[9].free();
  h->mgF[9].free();
  for (int i = 0; i < nArr; ++i) {
    CK(h->mgD[i].upload(*src[i], st));
    std::vector<float> f(src[i]->begin(), src[i]->end());
    CK(h->mgF[i].upload(f, st));
  }
  CK(h->fissile.upload(fis, st));
  double cxs = d->avg_dist > 0.0 ? 1.0 / d->avg_dist : 0.0;
  // 1 / max(majorant, collisionXS) per group, the delta-tracking flight's inverse majorant: the same
  // IEEE division the kernel would make, in each precision
  std::vector<double> majInv(nG);
  std::vector<float> majInvF(nG);
  for (int g = 0; g < nG; ++g) {
    majInv[g] = 1.0 / std::max(maj[g], cxs);
    majInvF[g] = 1.0f / std::max((float)maj[g], (float)cxs);
  }
  CK(h->mgD[10].upload(majInv, st));
  CK(h->mgF[10].upload(majInvF, st));
  h->mg64 = DMG<double>{M, nG, h->mgD[0].p, h->mgD[1].p, h->mgD[2].p, h->mgD[3].p, h->mgD[4].p, h->mgD[5].p,
                        h->mgD[6].p, h->mgD[7].p, h->fissile.p, h->mgD[8].p, cxs, d->p1 ? h->mgD[9].p : nullptr,
                        h->mgD[10].p};
  h->mgMx = DMG<float>{M, nG, h->mgF[0].p, h->mgF[1].p, h->mgF[2].p, h->mgF[3].p, h->mgF[4].p, h->mgF[5].p,
                       h->mgF[6].p, h->mgF[7].p, h->fissile.p, h->mgF[8].p, (float)cxs, d->p1 ? h->mgF[9].p : nullptr,
                       h->mgF[10].p};
  h->hasMG = true;
  return SG_OK;
}

// ------------------------------------------------------------------ continuous-energy data
// Floor index with the reference's rule (genericProcedures.f90:132-166): the largest i with
// e[i] <= x, n-2 for x = e[n-1]; -1 outside [e[0], e[n-1]].
int floor_index(const double* e, int n, double x) {
  if (!(x >= e[0] && x <= e[n - 1])) return -1;
  if (x == e[n - 1]) return n - 2;
  return (int)(std::upper_bound(e, e + n, x) - e) - 1;
}

// Hash brackets over [logMin, logMin + nBins / invStep]: bin b gets (lo, hi) with
// e[lo] <= E < e[hi] for every E whose FP32-computed bin is b (edges widened by 1e-4 relative).
std::vector<int2> hash_brackets(const double* e, int n, int nBins, float logMin, float invStep) {
  std::vector<int2> h(nBins);
  const double step = 1.0 / (double)invStep;
  for (int b = 0; b < nBins; ++b) {
    const double lo_e = std::exp((double)logMin + b * step) * (1.0 - 1.0e-4);
    const double hi_e = std::exp((double)logMin + (b + 1) * step) * (1.0 + 1.0e-4);
    int lo = (b == 0 || lo_e <= e[0]) ? 0 : std::max(0, floor_index(e, n, std::min(lo_e, e[n - 1])));
    int hi = (b == nBins - 1 || hi_e >= e[n - 1]) ? n - 1 : floor_index(e, n, hi_e) + 1;
    hi = std::min(std::max(hi, lo + 1), n - 1);
    h[b] = make_int2(lo, hi);
  }
  return h;
}

// aceNeutronDatabase%init/activate/initMajorant (aceNeutronDatabase_class.f90:873-1163,1291-1621)
// for non-fissile nuclides without URR or S(a,b) tables.
int build_ce(sg_handle h, const sg_ce_desc* d) {
  if (!h->hasGeom) return h->fail(SG_ERR_STATE, "ce: upload the geometry first (majorant uses its materials)");
  if (h->hasMG) return h->fail(SG_ERR_STATE, "ce: the handle already holds MG data");
  const int nN = d->n_nuc, nM = d->n_mat;
  if (nN <= 0 || nM <= 0 || !d->nuc_ptr || !d->e || !d->xs || !d->A || !d->kT || !d->mat_ptr || !d->mat_nuc || !d->mat_dens)
    return h->fail(SG_ERR_BAD_ARG, "ce: bad sizes or missing arrays");
  if (!(d->min_e >= 0.0) || !(d->max_e > d->min_e) || !(d->thresh_e >= 0.0) || !(d->thresh_a >= 0.0))
    return h->fail(SG_ERR_BAD_ARG, "ce: bad neutronCEstd settings");
  const long long nP = d->nuc_ptr[nN];
  std::vector<long long> off(d->nuc_ptr, d->nuc_ptr + nN + 1);
  for (int i = 0; i < nN; ++i) {
    if (off[i + 1] - off[i] < 2) return h->fail(SG_ERR_BAD_ARG, "ce: a nuclide grid needs at least 2 points");
    if (off[i + 1] - off[i] > 0x7fffffff) return h->fail(SG_ERR_BAD_ARG, "ce: nuclide grid too large");
    for (long long j = off[i]; j < off[i + 1]; ++j) {
      if (j > off[i] && !(d->e[j] >= d->e[j - 1])) return h->fail(SG_ERR_BAD_ARG, "ce: energy grid not ascending");
      if (d->xs[4 * j + 2] != 0.0) return h->fail(SG_ERR_BAD_ARG, "ce: inelastic channels are not supported");
    }
    if (!(d->A[i] > 0.0) || !(d->kT[i] > 0.0)) return h->fail(SG_ERR_BAD_ARG, "ce: A and kT must be positive");
  }
  for (int m = 0; m < nM; ++m)
    for (int k = d->mat_ptr[m]; k < d->mat_ptr[m + 1]; ++k)
      if (d->mat_nuc[k] < 0 || d->mat_nuc[k] >= nN) return h->fail(SG_ERR_BAD_ARG, "ce: bad nuclide index");
  const std::vector<int2>& graph = h->graphHost;
  std::vector<int> act;                // materials the geometry uses (VOID, UNDEF and OVERLAP excluded)
  for (auto& e : graph) if (e.x > 0 && e.x < SG_OVERLAP_MAT) act.push_back(e.x);
  std::sort(act.begin(), act.end());
  act.erase(std::unique(act.begin(), act.end()), act.end());
  for (int a : act)
    if (a > nM || d->mat_ptr[a] == d->mat_ptr[a - 1]) return h->fail(SG_ERR_BAD_ARG, "ce: geometry uses an undefined or empty material");
  // energy bounds over all nuclides (:1043-1052)
  double eb0 = d->e[off[0]], eb1 = d->e[off[1] - 1];
  double gmin = eb0, gmax = eb1;
  for (int i = 1; i < nN; ++i) {
    eb0 = std::max(eb0, d->e[off[i]]);
    eb1 = std::min(eb1, d->e[off[i + 1] - 1]);
    gmin = std::min(gmin, d->e[off[i]]);
    gmax = std::max(gmax, d->e[off[i + 1] - 1]);
  }
  if (!(gmin > 0.0)) return h->fail(SG_ERR_BAD_ARG, "ce: energies must be positive");
  auto nuc_total = [&](int n, double E, double& xs) -> bool {   // updateTotalNucXS
    const double* e = d->e + off[n];
    int i = floor_index(e, (int)(off[n + 1] - off[n]), E);
    if (i < 0) return false;
    double f = (E - e[i]) / (e[i + 1] - e[i]);
    const double* x = d->xs + 4 * (off[n] + i);
    xs = x[4] * f + (1.0 - f) * x[0];
    return true;
  };
  // unionised majorant (:1375-1621): every active nuclide's grid points up to its first point
  // outside the bounds, plus eBounds(2); sorted and de-duplicated; value = max over the active
  // materials of their total at that energy, nudged up by 1e-6
  std::vector<double> ue, umaj;
  if (d->majorant) {
    std::vector<int> nucs;
    for (int a : act)
      for (int k = d->mat_ptr[a - 1]; k < d->mat_ptr[a]; ++k) nucs.push_back(d->mat_nuc[k]);
    std::sort(nucs.begin(), nucs.end());
    nucs.erase(std::unique(nucs.begin(), nucs.end()), nucs.end());
    for (int n : nucs)
      for (long long j = off[n]; j < off[n + 1]; ++j) {
        if (d->e[j] < eb0 || d->e[j] > eb1) break;
        ue.push_back(d->e[j]);
      }
    ue.push_back(eb1);
    std::sort(ue.begin(), ue.end());
    ue.erase(std::unique(ue.begin(), ue.end()), ue.end());
    if (ue.size() < 2) return h->fail(SG_ERR_BAD_ARG, "ce: the union energy grid has fewer than 2 points");
    umaj.resize(ue.size());
    for (size_t i = 0; i < ue.size(); ++i) {
      double E = std::min(std::max(ue[i], eb0), eb1);
      double maj = 0.0;
      for (int a : act) {
        double t = 0.0;
        for (int k = d->mat_ptr[a - 1]; k < d->mat_ptr[a]; ++k) {
          double s = 0.0;
          nuc_total(d->mat_nuc[k], E, s);
          t = t + d->mat_dens[k] * s;
        }
        maj = std::max(maj, t * 1.0);
      }
      umaj[i] = maj * (1.0 + 1.0e-6);
    }
  }
  // hash brackets: nuclides share one log range; the union grid has its own
  const int nHash = 8192;
  const float hLogMin = (float)std::log(gmin);
  const float hInvStep = (float)(nHash / (std::log(gmax) - std::log(gmin)));
  std::vector<int2> hash((size_t)nN * nHash);
  for (int n = 0; n < nN; ++n) {
    auto hb = hash_brackets(d->e + off[n], (int)(off[n + 1] - off[n]), nHash, hLogMin, hInvStep);
    std::copy(hb.begin(), hb.end(), hash.begin() + (size_t)n * nHash);
  }
  int nUHash = 0;
  float uLogMin = 0.f, uInvStep = 0.f;
  std::vector<int2> uhash;
  if (d->majorant) {
    nUHash = (int)std::min<size_t>(1u << 18, std::max<size_t>(1024, ue.size() / 4));
    uLogMin = (float)std::log(ue.front());
    uInvStep = (float)(nUHash / (std::log(ue.back()) - std::log(ue.front())));
    uhash = hash_brackets(ue.data(), (int)ue.size(), nUHash, uLogMin, uInvStep);
  }
  // lookup union: every nuclide's grid points, sorted and de-duplicated, with each nuclide's floor
  // index at every union point (a merge walk per nuclide).  Built when the table stays below 2^26
  // entries (256 MB); otherwise the kernels search each nuclide's grid.
  std::vector<double> lu;
  std::vector<int> lidx, lmaj;
  std::vector<int2> luhash;
  int nLUHash = 0;
  float luLogMin = 0.f, luInvStep = 0.f;
  {
    lu.assign(d->e, d->e + nP);
    std::sort(lu.begin(), lu.end());
    lu.erase(std::unique(lu.begin(), lu.end()), lu.end());
    if (lu.size() >= 2 && (double)lu.size() * nN <= (double)(1 << 26)) {
      lidx.resize(lu.size() * (size_t)nN);
      for (int n = 0; n < nN; ++n) {
        const double* en = d->e + off[n];
        const long long cnt = off[n + 1] - off[n];
        long long j = 0;
        for (size_t u = 0; u < lu.size(); ++u) {
          while (j + 1 < cnt && en[j + 1] <= lu[u]) ++j;
          lidx[u * nN + n] = (lu[u] < en[0]) ? -1 : (int)j;
        }
      }
      nLUHash = (int)std::min<size_t>(1u << 18, std::max<size_t>(1024, lu.size() / 4));
      luLogMin = (float)std::log(lu.front());
      luInvStep = (float)(nLUHash / (std::log(lu.back()) - std::log(lu.front())));
      luhash = hash_brackets(lu.data(), (int)lu.size(), nLUHash, luLogMin, luInvStep);
      if (d->majorant) {               // the majorant grid's points are union points too
        lmaj.resize(lu.size());
        long long j = 0;
        const long long cnt = (long long)ue.size();
        for (size_t u = 0; u < lu.size(); ++u) {
          while (j + 1 < cnt && ue[j + 1] <= lu[u]) ++j;
          lmaj[u] = (lu[u] < ue[0]) ? -1 : (int)j;
        }
        for (double x : ue)            // guard: a majorant point outside the union disables the table
          if (!std::binary_search(lu.begin(), lu.end(), x)) { lmaj.clear(); break; }
      }
    } else {
      lu.clear();
    }
  }
  // uploads
  cudaStream_t st = h->stream;
  std::vector<double> e(d->e, d->e + nP), xs(d->xs, d->xs + 4 * nP), A(d->A, d->A + nN), kT(d->kT, d->kT + nN);
  std::vector<int> mp(d->mat_ptr, d->mat_ptr + nM + 1), mn(d->mat_nuc, d->mat_nuc + d->mat_ptr[nM]);
  std::vector<double> dens(d->mat_dens, d->mat_dens + d->mat_ptr[nM]);
  CK(h->ceE.upload(e, st));
  CK(h->ceXs64.upload(xs, st));
  CK(h->ceA64.upload(A, st));
  CK(h->ceKT64.upload(kT, st));
  CK(h->ceDens64.upload(dens, st));
  CK(h->ceXsF.upload(std::vector<float>(xs.begin(), xs.end()), st));
  CK(h->ceAF.upload(std::vector<float>(A.begin(), A.end()), st));
  CK(h->ceKTF.upload(std::vector<float>(kT.begin(), kT.end()), st));
  CK(h->ceDensF.upload(std::vector<float>(dens.begin(), dens.end()), st));
  CK(h->ceOff.upload(off, st));
  CK(h->ceHash.upload(hash, st));
  CK(h->ceMatPtr.upload(mp, st));
  CK(h->ceMatNuc.upload(mn, st));
  CK(h->ceAct.upload(act, st));
  CK(h->ceUE.upload(ue, st));
  CK(h->ceMaj64.upload(umaj, st));
  CK(h->ceMajF.upload(std::vector<float>(umaj.begin(), umaj.end()), st));
  CK(h->ceUHash.upload(uhash, st));
  if (!lidx.empty()) {
    CK(h->ceLU.upload(lu, st));
    CK(h->ceLIdx.upload(lidx, st));
    CK(h->ceLUHash.upload(luhash, st));
    if (!lmaj.empty()) CK(h->ceLMaj.upload(lmaj, st));
  }
  const double cxs = d->avg_dist > 0.0 ? 1.0 / d->avg_dist : 0.0;
  auto fill = [&](auto& D, auto xsP, auto aP, auto ktP, auto densP, auto majP) {
    using RR = std::remove_reference_t<decltype(*xsP)>;
    D.nNuc = nN; D.nMat = nM;
    D.e = h->ceE.p; D.xs = xsP; D.off = h->ceOff.p; D.hash = h->ceHash.p; D.nHash = nHash;
    D.hLogMin = hLogMin; D.hInvStep = hInvStep;
    D.A = aP; D.kT = ktP; D.matPtr = h->ceMatPtr.p; D.matNuc = h->ceMatNuc.p; D.matDens = densP;
    D.hasMajorant = d->majorant ? 1 : 0;
    D.ue = h->ceUE.p; D.umaj = majP; D.uhash = h->ceUHash.p; D.nU = (int)ue.size(); D.nUHash = nUHash;
    D.uLogMin = uLogMin; D.uInvStep = uInvStep;
    D.act = h->ceAct.p; D.nAct = (int)act.size();
    D.lu = lidx.empty() ? nullptr : h->ceLU.p;
    D.lidx = lidx.empty() ? nullptr : h->ceLIdx.p;
    D.luhash = lidx.empty() ? nullptr : h->ceLUHash.p;
    D.lmaj = (lidx.empty() || lmaj.empty()) ? nullptr : h->ceLMaj.p;
    D.nLU = (int)lu.size(); D.nLUHash = nLUHash;
    D.luLogMin = luLogMin; D.luInvStep = luInvStep;
    D.minE = d->min_e; D.threshE = (RR)d->thresh_e; D.threshA = (RR)d->thresh_a; D.collisionXS = (RR)cxs;
  };
  fill(h->ce64, (const double*)h->ceXs64.p, (const double*)h->ceA64.p, (const double*)h->ceKT64.p,
       (const double*)h->ceDens64.p, (const double*)h->ceMaj64.p);
  fill(h->ceMx, (const float*)h->ceXsF.p, (const float*)h->ceAF.p, (const float*)h->ceKTF.p,
       (const float*)h->ceDensF.p, (const float*)h->ceMajF.p);
  // banks carry energies
  for (int b = 0; b < 2; ++b) CK(h->bank[b].E.alloc(h->cap));
  if (h->cfg.form == SG_FORM_EVENT) CK(h->pE.alloc(h->cap));
  h->hasCE = true;
  return SG_OK;
}

int alloc_work(sg_handle h) {
  const size_t cap = (size_t)h->cap;
  for (int b = 0; b < 2; ++b) CK(h->bank[b].alloc(cap));
  h->regionCap = (int)((2 * cap + SITE_REGIONS - 1) / SITE_REGIONS) + 4096;
  const size_t sc = (size_t)h->regionCap * SITE_REGIONS;
  CK(h->sR.alloc(3 * sc)); CK(h->sDir.alloc(3 * sc)); CK(h->sWgt.alloc(sc)); CK(h->sTime.alloc(sc));
  CK(h->sG.alloc(sc)); CK(h->sBrood.alloc(sc)); CK(h->sSeq.alloc(sc)); CK(h->sCursor.alloc(SITE_REGIONS));
  CK(h->histN.alloc(cap + 1)); CK(h->start.alloc(cap + 1)); CK(h->scanTmp.alloc(scan_tmp_size((int)cap + 1) + 16));
  CK(h->flags.alloc(cap + 1)); CK(h->pos.alloc(cap + 1)); CK(h->kbuf.alloc(4));
  CK(h->keys.alloc(cap)); CK(h->sel.alloc(2)); CK(h->hist16.alloc(65536));
  CK(h->winCnt.alloc(2)); CK(h->winCand.alloc(WIN_CAP));
  CK(cudaMemsetAsync(h->hist16.p, 0, 65536 * sizeof(unsigned int), h->stream));
  CK(h->sumPart.alloc(SUM_BLOCKS)); CK(h->scal.alloc(8)); CK(h->totals.alloc(8)); CK(h->ctr.alloc(1));
  if (h->cfg.record_histories) { CK(h->recColl.alloc(cap)); CK(h->recRng.alloc(cap)); }
  if (h->cfg.form == SG_FORM_EVENT) {
    CK(h->pR0.alloc(3 * cap)); CK(h->pRl.alloc(9 * cap)); CK(h->pU.alloc(3 * cap));
    CK(h->pW.alloc(cap)); CK(h->pW0.alloc(cap)); CK(h->pTime.alloc(cap)); CK(h->pTrack.alloc(cap));
    CK(h->pGeo.alloc(15 * cap)); CK(h->pInts.alloc(5 * cap)); CK(h->pRng.alloc(cap));
    CK(h->qT0.alloc(cap)); CK(h->qT1.alloc(cap)); CK(h->qC.alloc(cap)); CK(h->qCtr.alloc(8));
  }
  CK(cudaMemset(h->scal.p, 0, 8 * sizeof(double)));
  return SG_OK;
}

template <class R>
DPart<R> part_view(sg_handle h) {
  DPart<R> p;
  p.r0 = h->pR0.p;
  p.rl = reinterpret_cast<R*>(h->pRl.p);
  p.u = reinterpret_cast<R*>(h->pU.p);
  p.geo = h->pGeo.p;
  p.rng = h->pRng.p;
  p.w = reinterpret_cast<R*>(h->pW.p);
  p.w0 = reinterpret_cast<R*>(h->pW0.p);
  p.time = reinterpret_cast<R*>(h->pTime.p);
  p.trackXS = reinterpret_cast<R*>(h->pTrack.p);
  p.ints = h->pInts.p;
  p.E = h->pE.p;
  p.cap = h->cap;
  return p;
}

template <class R> const DColl<R>* coll_view(sg_handle h);
template <> const DColl<double>* coll_view<double>(sg_handle h) { return h->dColl64.p; }
template <> const DColl<float>* coll_view<float>(sg_handle h) { return h->dColl32.p; }

DSites site_view(sg_handle h) {
  return DSites{h->sR.p, h->sDir.p, h->sWgt.p, h->sG.p, h->sBrood.p, h->sSeq.p, h->sTime.p, h->sCursor.p, h->regionCap,
                SITE_REGIONS - 1};
}

// Bins of one map axis: cellMap has n cells plus the `undefBin` rest bin (cellMap_class.f90:129-136)
long long axis_bins(const sg_axis_desc& x) {
  return x.kind == SG_AXIS_CELL ? (long long)x.n + (x.cell_rest ? 1 : 0) : x.n;
}

// The multiMap axes of one clerk (or of the weight-window map) as the kernels read them; tables
// from A.tab64 / A.tab32 at [tab + axis].  Returns the number of map bins.
template <class R>
long long fill_axes(DClerk& K, const sg_axis_desc* axes, int n, const Admin& A, size_t tab) {
  long long mul = 1;
  K.n_axes = n;
  for (int i = 0; i < n; ++i) {
    const sg_axis_desc& x = axes[i];
    K.ax_kind[i] = x.kind;
    K.ax_n[i] = x.n;
    K.ax_min[i] = x.min;
    int grid = x.grid;
    if (grid == SG_GRID_DEFAULT) grid = x.kind == SG_AXIS_ENERGY ? SG_GRID_LOG : SG_GRID_LIN;
    K.ax_grid[i] = grid;
    if (grid == SG_GRID_LOG)                         // grid step (grid_class.f90:60-90)
      K.ax_step[i] = std::log(x.max / x.min) / x.n;
    else K.ax_step[i] = (x.max - x.min) / x.n;
    K.ax_inv_step[i] = 1.0 / K.ax_step[i];
    // the FP32 copy of a log grid holds log(min): the mixed form bins log(E) - log(min) directly
    K.ax_minf[i] = grid == SG_GRID_LOG ? (float)std::log(x.min) : (float)K.ax_min[i];
    K.ax_inv_stepf[i] = (float)K.ax_inv_step[i];
    K.ax_tab[i] = (sizeof(R) == 8 ? A.tab64 : A.tab32)[tab + i];
    K.multi[i] = mul;
    mul *= axis_bins(x);
  }
  return mul;
}

// clerks of admin `a` and its attachment flattened for one launch (attachment first)
template <class R>
int build_clerks(sg_handle h, int a, TransportArgs<R>& t, long long& lo, long long& hi) {
  std::vector<int> chain;
  for (int x = a; x >= 0; x = h->admins[x].atch) {
    if (chain.size() > 4) return h->fail(SG_ERR_BAD_ARG, "tally: attachment cycle");
    chain.push_back(x);
  }
  std::reverse(chain.begin(), chain.end());
  lo = 0; hi = 0;
  bool first = true;
  for (int x : chain) {
    const Admin& A = h->admins[x];
    if (A.N == 0) continue;
    if (first) { lo = A.off; hi = A.off + A.N; first = false; }
    lo = std::min(lo, A.off);
    hi = std::max(hi, A.off + A.N);
  }
  t.n_clerks = 0;
  t.keff_clerk = -1;
  t.has_current = 0;
  t.has_cellmap = 0;
  for (int x : chain) {
    const Admin& A = h->admins[x];
    for (size_t c = 0; c < A.clerks.size(); ++c) {
      const sg_clerk_desc& d = A.clerks[c];
      if (d.type == SG_CLERK_KEFF_ANALOG) continue;   // scored at cycle start/end only
      if (t.n_clerks >= MAX_CLERKS) return h->fail(SG_ERR_BAD_ARG, "tally: too many clerks in one launch");
      DClerk& K = t.clerks[t.n_clerks];
      std::memset(&K, 0, sizeof(K));
      K.type = d.type;
      K.handle_virtual = d.handle_virtual;
      K.width = d.n_resp > 0 ? d.n_resp : 1;
      for (int i = 0; i < 4; ++i) K.resp[i] = d.resp[i];
      K.n_axes = d.n_axes;
      const long long mul = fill_axes<R>(K, d.axes, d.n_axes, A, 3 * c);
      for (int i = 0; i < d.n_axes; ++i)
        if (d.axes[i].kind == SG_AXIS_CELL) t.has_cellmap = 1;
      K.g_top = d.filter_g_top;
      K.g_low = d.filter_g_low;
      K.acc_off = A.off + (A.addr[c] - 1) - lo;
      K.nbins = mul;
      if (d.type == SG_CLERK_SURFACE_CURRENT) {
        K.cur_axis = d.current_axis - SG_AXIS_X;
        K.n_planes = d.n_planes;
        for (int q = 0; q < d.n_planes; ++q) K.planes[q] = d.planes[q];
        t.has_current = 1;
      }
      if (d.type == SG_CLERK_KEFF_IMPLICIT) {
        if (t.keff_clerk >= 0) return h->fail(SG_ERR_BAD_ARG, "tally: one k-implicit clerk per launch");
        t.keff_clerk = t.n_clerks;
      }
      t.n_clerks++;
    }
  }
  return SG_OK;
}

// Whether a launch can run the lean history loop: multigroup data and none of rotated universes,
// cell maps, surface-current clerks, neutronMGimp or P1 scattering.
template <class R>
bool lean_launch(sg_handle h, const TransportArgs<R>& t) {
  return !h->hasCE && t.geom.rot == nullptr && !t.has_cellmap && !t.has_current && !t.coll_imp &&
         t.mg.P1n == nullptr;
}

// The gen loop over `n` histories of bank `in` on the device; fission sites are written into bank
// `out` in brood order.  Returns SG_OK and the number of sites.
template <class R>
int gen_loop_t(sg_handle h, int admin, DBank in, int n, unsigned long long master, const double* d_k,
               DBank out, int outcap, int* S_out, sg_cycle_stats* st, const DGeom& geom, const DMG<R>& mg,
               const DCE<R>& ce) {
  cudaStream_t s = h->stream;
  TransportArgs<R> t;
  std::memset(&t, 0, sizeof(t));
  long long lo = 0, hi = 0;
  int rc = build_clerks<R>(h, admin, t, lo, hi);
  if (rc) return rc;
  t.geom = geom;
  t.mg = mg;
  t.ce = ce;
  t.in = in;
  t.n = n;
  t.master = master;
  t.k_eff = d_k;
  t.acc = h->acc.p + lo;
  t.acc_n = (int)(hi - lo);
  size_t smem = (size_t)t.acc_n * sizeof(double);
  t.use_smem = scores_in_shared_memory(t.acc_n) ? 1 : 0;
  if (!t.use_smem) smem = 0;
  t.sites = site_view(h);
  t.hist_nsites = h->histN.p;
  t.rec_coll = h->cfg.record_histories ? h->recColl.p : nullptr;
  t.rec_rng = h->cfg.record_histories ? h->recRng.p : nullptr;
  t.coll_imp = h->collImp ? 1 : 0;
  t.coll = h->collImp ? coll_view<R>(h) : nullptr;
  if (h->collImp && h->collBuf && h->cfg.form == SG_FORM_EVENT)
    return h->fail(SG_ERR_BAD_ARG, "splitting and weight windows need the history-loop form");
  t.ctr = h->ctr.p;
  t.use_cache = transport_cache(h->cfg.transport);
  t.max_segments = 1000000;
  t.ht_cutoff = (R)h->htCutoff;
  t.lean = lean_launch(h, t) ? 1 : 0;
  CK(cudaMemsetAsync(h->ctr.p, 0, sizeof(DCounters), s));
  CK(cudaMemsetAsync(h->sCursor.p, 0, SITE_REGIONS * sizeof(int), s));
  CK(cudaMemsetAsync(h->histN.p, 0, (size_t)(n + 1) * sizeof(int), s));
  CK(cudaMemsetAsync(h->totals.p, 0, 8 * sizeof(int), s));
  CK(cudaEventRecord(h->ev[0], s));
  const int dt = transport_op(h->cfg.transport);
  auto launch_kind = [&](int kind, const TransportArgs<R>& a, int maxl, int opk, size_t sm, cudaStream_t ss, int* g) {
    return h->hasCE ? launch_kind_ce<R>(kind, a, maxl, opk, sm, ss, g) : sg::launch_kind<R>(kind, a, maxl, opk, sm, ss, g);
  };
  if (h->cfg.form == SG_FORM_HISTORY) {
    CK(launch_kind(K_HISTORY, t, h->maxl, dt, smem, s, nullptr));
    h->launches += 1;
  } else {
    // event form: start, then transit / collide rounds over compacted queues, then the tail
    t.use_smem = 0;
    t.part = part_view<R>(h);
    int* qc = h->qCtr.p;              // [0] transit count A, [1] transit count B, [2] collision count, [3] work
    int* qT[2] = {h->qT0.p, h->qT1.p};
    CK(cudaMemsetAsync(qc, 0, 8 * sizeof(int), s));
    t.q = DQueues{nullptr, nullptr, qT[0], qc + 0, qc + 3};
    CK(launch_kind(K_EV_START, t, h->maxl, dt, 0, s, nullptr));
    int cur = 0, it = 0;
    const int tail = std::max(h->evTune.tail_min, n / h->evTune.tail_divisor);
    const int CHUNK = h->evTune.rounds_per_check;
    h->launches += 1;
    while (true) {
      for (int k = 0; k < CHUNK; ++k, ++it) {
        CK(cudaMemsetAsync(qc + 2, 0, 2 * sizeof(int), s));
        t.q = DQueues{qT[cur], qc + cur, h->qC.p, qc + 2, qc + 3};
        CK(launch_kind(K_EV_TRANSIT, t, h->maxl, dt, 0, s, nullptr));
        CK(cudaMemsetAsync(qc + (1 - cur), 0, sizeof(int), s));
        t.q = DQueues{h->qC.p, qc + 2, qT[1 - cur], qc + (1 - cur), qc + 3};
        CK(launch_kind(K_EV_COLLIDE, t, h->maxl, dt, 0, s, nullptr));
        cur = 1 - cur;
        h->launches += 2;
      }
      int left = 0;
      CK(cudaMemcpyAsync(&left, qc + cur, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (left <= tail || it > 4096) break;
    }
    CK(cudaMemsetAsync(qc + 3, 0, sizeof(int), s));
    t.q = DQueues{qT[cur], qc + cur, nullptr, nullptr, qc + 3};
    CK(launch_kind(K_EV_TAIL, t, h->maxl, dt, 0, s, nullptr));
    h->launches += 1;
    h->evIterations = it;
  }
  CK(cudaEventRecord(h->ev[1], s));
  CK(exclusive_scan(h->histN.p, n + 1, h->start.p, h->scanTmp.p, h->totals.p + 0, s));
  CK(launch_site_scatter(site_view(h), h->start.p, out, outcap, h->totals.p + 3, s));
  h->launches += 4;
  DCounters c;
  int tot[8];
  CK(cudaMemcpyAsync(&c, h->ctr.p, sizeof(c), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(tot, h->totals.p, sizeof(tot), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaEventElapsedTime(&h->lastTransportMs, h->ev[0], h->ev[1]));
  h->lastN = n;
  if (c.err_code) {
    char m[160];
    std::snprintf(m, sizeof(m), "transport: error %d raised in history %d", c.err_code, c.err_hist);
    return h->fail(c.err_code, m);
  }
  if (tot[3] || tot[0] > outcap) return h->fail(SG_ERR_BANK_OVERFLOW, "transport: fission bank overflow");
  *S_out = tot[0];
  if (st) {
    st->n_histories = n;
    st->n_events = (int64_t)c.events;
    st->n_collisions = (int64_t)c.collisions;
    st->n_next = tot[0];
    st->transport_ms = h->lastTransportMs;
  }
  return SG_OK;
}

int gen_loop(sg_handle h, int admin, DBank in, int n, unsigned long long master, const double* d_k, DBank out,
             int outcap, int* S, sg_cycle_stats* st) {
  if (!h->hasGeom || !(h->hasMG || h->hasCE)) return h->fail(SG_ERR_STATE, "upload geometry and nuclear data first");
  if (admin < 0 || admin >= (int)h->admins.size()) return h->fail(SG_ERR_BAD_ARG, "bad tally admin");
  if (n < 0 || n > h->cap) return h->fail(SG_ERR_BANK_OVERFLOW, "bank larger than max_bank");
  if (h->hasCE) {
    for (int x = admin; x >= 0; x = h->admins[x].atch)
      for (const auto& d : h->admins[x].clerks) {
        if (d.type == SG_CLERK_KEFF_IMPLICIT) return h->fail(SG_ERR_BAD_ARG, "tally: k-implicit clerks need fissile MG data");
        if (d.filter_g_top > 0) return h->fail(SG_ERR_BAD_ARG, "tally: group filters apply to MG problems only");
      }
  }
  if (h->cfg.precision == SG_PREC_MIXED)
    return gen_loop_t<float>(h, admin, in, n, master, d_k, out, outcap, S, st, h->gMx, h->mgMx, h->ceMx);
  return gen_loop_t<double>(h, admin, in, n, master, d_k, out, outcap, S, st, h->g64, h->mg64, h->ce64);
}

// tallyAdmin%reportCycleStart: keffAnalog START_POP (keffAnalogClerk_class.f90:140-147)
int cycle_start(sg_handle h, int admin, const double* d_w, double w) {
  for (int x = admin; x >= 0; x = h->admins[x].atch) {
    const Admin& A = h->admins[x];
    if (A.keffAnalog >= 0) { CK(add_scalar(h->acc.p + A.off + A.keffAnalog, d_w, w, h->stream)); h->launches += 1; }
  }
  return SG_OK;
}

// tallyAdmin%reportCycleEnd for the chain (attachment first); k of `kadmin` is written to k_out
int cycle_end(sg_handle h, int admin, const double* d_endw, const double* d_kend, int kadmin, double* k_out) {
  std::vector<int> chain;
  for (int x = admin; x >= 0; x = h->admins[x].atch) chain.push_back(x);
  std::reverse(chain.begin(), chain.end());
  for (int x : chain) {
    Admin& A = h->admins[x];
    TallyCloseArgs a;
    std::memset(&a, 0, sizeof(a));
    a.acc = h->acc.p + A.off;
    a.bin = h->bin.p + A.off;
    a.csum = h->csum.p + A.off;
    a.csum2 = h->csum2.p + A.off;
    a.N = A.N;
    a.last_cycle = A.lastCycle();
    a.close_batch = (A.cycles + 1) % A.batchSize == 0;
    a.keff_analog = A.keffAnalog;
    a.keff_implicit = A.keffImplicit;
    a.norm_addr = A.normAddr >= 1 ? A.normAddr - 1 : -1;
    a.norm_val = A.normVal;
    a.end_weight = d_endw;
    a.k_end = d_kend;
    int batchN = A.batchN + (a.close_batch ? 1 : 0);
    a.batchN = batchN;
    a.k_out = (x == kadmin) ? k_out : nullptr;
    a.k_addr = A.keffImplicit >= 0 ? A.keffImplicit + 4 : (A.keffAnalog >= 0 ? A.keffAnalog + 2 : -1);
    if (A.N > 0) { CK(launch_tally_close(a, h->stream)); h->launches += 1; }
    A.cycles += 1;
    A.batchN = batchN;
  }
  return SG_OK;
}

// particleDungeon%normSize_Repr on the device: sites (sorted by brood) in `in`, result in `out`
int norm_size(sg_handle h, DBank in, int S, int totPop, unsigned long long master, DBank out, int n_hist) {
  cudaStream_t s = h->stream;
  if (S <= 0) return h->fail(SG_ERR_STATE, "normSize: empty fission bank");
  int excess = S - totPop;
  int heap = excess > 0 ? excess : (excess < 0 ? (-excess) % S : 0);
  if (heap > 0) {
    k_rn_keys<<<((S + 31) / 32 + 127) / 128, 128, 0, s>>>(master, S, h->keys.p);
    CK(cudaGetLastError());
    CK(quantile_select(h->keys.p, S, heap, h->sel.p, h->kbuf.p, h->hist16.p, h->winCnt.p, h->winCand.p, s));
    h->launches += 11;
  }
  if (excess > 0) {
    CK(launch_flags(h->keys.p, S, h->sel.p, 1, h->flags.p, s));
    CK(cudaMemsetAsync(h->flags.p + S, 0, sizeof(int), s));
    CK(exclusive_scan(h->flags.p, S + 1, h->pos.p, h->scanTmp.p, h->totals.p + 1, s));
    CK(launch_compact(in, S, h->flags.p, h->pos.p, out, s));
    h->launches += 5;
    int kept = 0;
    CK(cudaMemcpyAsync(&kept, h->totals.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (kept != totPop) return h->fail(SG_ERR_STATE, "normSize: normalisation failed (ties at the threshold)");
  } else if (excess < 0) {
    int n_copies = (-excess) / S;
    if ((long long)(n_copies + 1) * S + heap > h->cap) return h->fail(SG_ERR_BANK_OVERFLOW, "normSize: bank overflow");
    if (heap > 0) CK(launch_flags(h->keys.p, S, h->sel.p, 0, h->flags.p, s));
    else CK(cudaMemsetAsync(h->flags.p, 0, (size_t)S * sizeof(int), s));
    CK(cudaMemsetAsync(h->flags.p + S, 0, sizeof(int), s));
    CK(exclusive_scan(h->flags.p, S + 1, h->pos.p, h->scanTmp.p, h->totals.p + 2, s));
    CK(launch_replicate(in, S, h->flags.p, h->pos.p, h->start.p, n_copies, out, s));
    h->launches += (heap > 0 ? 5 : 4);
    (void)n_hist;
  } else {
    CK(cudaMemcpyAsync(out.r, in.r, 3 * sizeof(double) * S, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(out.dir, in.dir, 3 * sizeof(double) * S, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(out.wgt, in.wgt, sizeof(double) * S, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(out.time, in.time, sizeof(double) * S, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(out.G, in.G, sizeof(int) * S, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(out.brood, in.brood, sizeof(int) * S, cudaMemcpyDeviceToDevice, s));
  }
  return SG_OK;
}

int h2d_bank(sg_handle h, const sg_bank* b, int n, DBank d) {
  cudaStream_t s = h->stream;
  if (!b->r || !b->dir) return h->fail(SG_ERR_BAD_ARG, "bank: r and dir are required");
  CK(cudaMemcpyAsync(d.r, b->r, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.dir, b->dir, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, s));
  if (b->wgt) CK(cudaMemcpyAsync(d.wgt, b->wgt, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  else {
    std::vector<double> one(n, 1.0);
    CK(cudaMemcpyAsync(d.wgt, one.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
  }
  if (h->hasCE) {
    if (!b->E) return h->fail(SG_ERR_BAD_ARG, "bank: E is required for CE transport");
    CK(cudaMemcpyAsync(d.E, b->E, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    if (b->G) CK(cudaMemcpyAsync(d.G, b->G, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    else CK(cudaMemsetAsync(d.G, 0, sizeof(int) * n, s));
  } else if (b->G) CK(cudaMemcpyAsync(d.G, b->G, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  else return h->fail(SG_ERR_BAD_ARG, "bank: G is required for MG transport");
  if (b->time) CK(cudaMemcpyAsync(d.time, b->time, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  else CK(cudaMemsetAsync(d.time, 0, sizeof(double) * n, s));
  return SG_OK;
}

// The arrays go back in two halves on two streams, so two copy engines share the transfer (the
// second stream waits for the bank to be complete and the first waits for the second's copies).
int d2h_bank(sg_handle h, DBank d, int n, const sg_bank* b) {
  cudaStream_t s = h->stream, s2 = h->copyStream;
  if (n <= 0) return SG_OK;
  CK(cudaEventRecord(h->copyEv[0], s));
  CK(cudaStreamWaitEvent(s2, h->copyEv[0], 0));
  if (b->r) CK(cudaMemcpyAsync(b->r, d.r, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (b->dir) CK(cudaMemcpyAsync(b->dir, d.dir, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, s2));
  if (b->wgt) CK(cudaMemcpyAsync(b->wgt, d.wgt, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (b->G) CK(cudaMemcpyAsync(b->G, d.G, sizeof(int) * n, cudaMemcpyDeviceToHost, s2));
  if (b->time) CK(cudaMemcpyAsync(b->time, d.time, sizeof(double) * n, cudaMemcpyDeviceToHost, s2));
  if (b->brood_id) CK(cudaMemcpyAsync(b->brood_id, d.brood, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  if (b->E && d.E) CK(cudaMemcpyAsync(b->E, d.E, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(h->copyEv[1], s2));
  CK(cudaStreamWaitEvent(s, h->copyEv[1], 0));
  CK(cudaStreamSynchronize(s));
  return SG_OK;
}

// A host bank in page-locked memory that the device can address (cudaHostAlloc / cudaHostRegister
// with mapping, the default under unified addressing) is read by the kernels in place, across the
// C2C link of a Grace-Blackwell node, while they run: no staging copy before the gen loop.  True and
// the device view when every array the gen loop reads (r, dir, wgt, G, time; E for CE) is such
// memory; false otherwise (the bank is then copied).
bool mapped_host_bank(sg_handle h, const sg_bank* b, DBank* d) {
  auto dev = [](const void* p, void** out) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
    *out = a.devicePointer;
    return true;
  };
  void *r, *dir, *wgt, *G, *time, *E = nullptr;
  if (!dev(b->r, &r) || !dev(b->dir, &dir) || !dev(b->wgt, &wgt) || !dev(b->time, &time)) return false;
  if (h->hasCE) { if (!dev(b->E, &E)) return false; G = nullptr; }
  else if (!dev(b->G, &G)) return false;
  *d = DBank{(double*)r, (double*)dir, (double*)wgt, (int*)G, nullptr, (double*)time, (double*)E};
  return true;
}

// Checks one map axis and uploads its table: the bounds of an unstructured grid (grid%init_unstruct,
// grid_class.f90:100-113: sorted, at least 2 bounds) or the bin of every cell for a cellMap
// (cellMap%build, cellMap_class.f90:87-138: listed cells take bins 1..n in order, every other cell
// and the places outside any cellUniverse take the rest bin n+1 or none).
int build_axis(sg_handle h, const sg_axis_desc& x, Admin& A) {
  const void *t64 = nullptr, *t32 = nullptr;
  if (x.n < 1 || x.kind < SG_AXIS_X || x.kind > SG_AXIS_CELL) return h->fail(SG_ERR_BAD_ARG, "tally: bad map axis");
  if (x.kind <= SG_AXIS_Z || x.kind == SG_AXIS_ENERGY) {
    const bool energy = x.kind == SG_AXIS_ENERGY;
    const int grid = x.grid == SG_GRID_DEFAULT ? (energy ? SG_GRID_LOG : SG_GRID_LIN) : x.grid;
    if (!energy && grid == SG_GRID_LOG) return h->fail(SG_ERR_BAD_ARG, "tally: spaceMap grids are lin or unstruct");
    if (grid == SG_GRID_LIN) {
      if (!(x.max > x.min)) return h->fail(SG_ERR_BAD_ARG, "tally: lin grid needs max > min");
    } else if (grid == SG_GRID_LOG) {
      if (!(x.min > 0.0 && x.max > x.min)) return h->fail(SG_ERR_BAD_ARG, "tally: log grid needs 0 < min < max");
    } else if (grid == SG_GRID_UNSTRUCT) {
      if (!x.bounds) return h->fail(SG_ERR_BAD_ARG, "tally: unstructured grid without bounds");
      std::vector<double> b(x.bounds, x.bounds + x.n + 1);
      for (int i = 0; i < x.n; ++i)
        if (!(b[i] <= b[i + 1])) return h->fail(SG_ERR_BAD_ARG, "tally: unstructured grid is not sorted");
      std::vector<float> f(b.begin(), b.end());
      h->mapTab64.emplace_back();
      h->mapTab32.emplace_back();
      if (h->mapTab64.back().upload(b, h->stream) != cudaSuccess || h->mapTab32.back().upload(f, h->stream) != cudaSuccess)
        return h->fail(SG_ERR_OOM, "tally: grid table");
      t64 = h->mapTab64.back().p;
      t32 = h->mapTab32.back().p;
    } else return h->fail(SG_ERR_BAD_ARG, "tally: unknown grid type");
  } else if (x.kind == SG_AXIS_CELL) {
    if (!h->hasGeom) return h->fail(SG_ERR_STATE, "tally: a cellMap needs the geometry uploaded first");
    if (!x.cells) return h->fail(SG_ERR_BAD_ARG, "tally: cellMap without cells");
    std::vector<int> bin(h->nCell + 1, x.cell_rest ? x.n + 1 : 0);
    bin[0] = x.cell_rest ? x.n + 1 : 0;
    for (int i = 0; i < x.n; ++i) {
      const int c = x.cells[i];
      if (c < 0 || c >= h->nCell) return h->fail(SG_ERR_BAD_ARG, "tally: cellMap names a cell the geometry lacks");
      bin[c + 1] = i + 1;     // a cell listed twice keeps its last bin (intMap%add replaces)
    }
    h->mapTabCell.emplace_back();
    if (h->mapTabCell.back().upload(bin, h->stream) != cudaSuccess) return h->fail(SG_ERR_OOM, "tally: cell table");
    t64 = t32 = h->mapTabCell.back().p;
  }
  A.tab64.push_back(t64);
  A.tab32.push_back(t32);
  return SG_OK;
}

// tallyAdmin%init (tallyAdmin_class.f90:162-255): clerk validation and scoreMemory layout of one admin
int build_admin(sg_handle h, const sg_tally_desc* t, Admin& A) {
  long long loc = 1;
  for (int i = 0; i < t->n_clerks; ++i) {
    const sg_clerk_desc& d = t->clerks[i];
    long long size;
    if (d.type == SG_CLERK_KEFF_ANALOG) { size = 3; A.keffAnalog = loc - 1; }
    else if (d.type == SG_CLERK_KEFF_IMPLICIT) { size = 5; A.keffImplicit = loc - 1; }
    else if (d.type == SG_CLERK_COLLISION || d.type == SG_CLERK_TRACK || d.type == SG_CLERK_SURFACE_CURRENT) {
      const bool cur = d.type == SG_CLERK_SURFACE_CURRENT;
      if ((!cur && (d.n_resp < 1 || d.n_resp > 4)) || d.n_axes < 0 || d.n_axes > 3) return h->fail(SG_ERR_BAD_ARG, "tally: bad clerk");
      if (cur && (d.current_axis < SG_AXIS_X || d.current_axis > SG_AXIS_Z || d.n_planes < 1 || d.n_planes > 8))
        return h->fail(SG_ERR_BAD_ARG, "tally: surface-current clerk needs an axis and 1-8 planes");
      long long nb = 1;
      for (int a = 0; a < d.n_axes; ++a) {
        const int rc = build_axis(h, d.axes[a], A);
        if (rc) return rc;
        nb *= axis_bins(d.axes[a]);
      }
      for (int a = d.n_axes; a < 3; ++a) { A.tab64.push_back(nullptr); A.tab32.push_back(nullptr); }
      size = cur ? nb * d.n_planes * 2 : nb * d.n_resp;
    } else return h->fail(SG_ERR_BAD_ARG, "tally: unknown clerk type");
    if (A.tab64.size() < 3 * (A.clerks.size() + 1))
      for (int a = 0; a < 3; ++a) { A.tab64.push_back(nullptr); A.tab32.push_back(nullptr); }
    A.clerks.push_back(d);
    A.addr.push_back(loc);
    loc += size;
  }
  A.N = loc - 1;
  A.batchSize = t->batch_size > 0 ? t->batch_size : 1;
  if (t->norm_clerk >= 0) {
    if (t->norm_clerk >= t->n_clerks) return h->fail(SG_ERR_BAD_ARG, "tally: bad norm clerk");
    A.normAddr = A.addr[t->norm_clerk];
    A.normVal = t->norm_val;
  }
  return SG_OK;
}

// One whole eigenvalue cycle (eigenPhysicsPackage_class.f90:203-338) on device banks: `in` is
// thisCycle (h->pop particles), the fission sites go to `sites` in brood order, normSize_Repr writes
// the next-cycle bank to `out` (which may be `in`).  h->master and h->k advance; the k used is in
// scal[0] and end%k_eff in scal[4].  The caller recorded ev[2] at its start.
int eigen_cycle_core(sg_handle h, int admin, int atch, DBank A, DBank B, DBank out, sg_cycle_stats* stats) {
  cudaStream_t s = h->stream;
  const int n = h->pop;
  CK(deterministic_sum(A.wgt, n, h->sumPart.p, h->scal.p + 2, s));       // popWeight(thisCycle)
  h->launches += 2;
  int rc = cycle_start(h, admin, h->scal.p + 2, 0.0);
  if (rc) return rc;
  int S = 0;
  sg_cycle_stats st{};
  rc = gen_loop(h, admin, A, n, h->master, h->scal.p + 0, B, h->cap, &S, &st);
  if (rc) return rc;
  h->master = rng_stride(h->master, (long long)h->pop + 1);              // :257
  CK(deterministic_sum(B.wgt, S, h->sumPart.p, h->scal.p + 3, s));       // popWeight(nextCycle)
  h->launches += 2;
  rc = cycle_end(h, admin, h->scal.p + 3, h->scal.p + 4, atch, h->scal.p + 1);
  if (rc) return rc;
  rc = norm_size(h, B, S, h->pop, h->master, out, n);                    // :269
  if (rc) return rc;
  h->master = rng_stride(h->master, 1);                                  // :275
  CK(cudaMemcpyAsync(h->scal.p + 0, h->scal.p + 1, sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(h->scal.p + 4, h->scal.p + 1, sizeof(double), cudaMemcpyDeviceToDevice, s));
  double sc[5];
  CK(cudaMemcpyAsync(sc, h->scal.p, sizeof(sc), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(h->ev[3], s));
  CK(cudaStreamSynchronize(s));
  float cyc = 0.f;
  CK(cudaEventElapsedTime(&cyc, h->ev[2], h->ev[3]));
  double kUsed = h->k;
  h->k = sc[1];
  st.start_weight = sc[2];
  st.end_weight = sc[3];
  st.k_eff = kUsed;
  st.k_new = sc[1];
  st.cycle_ms = cyc;
  st.n_kernels = h->launches;
  h->lastStats = st;
  if (stats) *stats = st;
  return SG_OK;
}

}  // namespace

// Bridge for sg_transport_bank_noalloc (sg_noalloc.cu): the launch arguments that do not depend on
// the call.  Reads the handle only; allocates nothing.
int sg::noalloc_view(sg_handle h, int admin, NoAllocView* v, TransportArgs<double>* t64, TransportArgs<float>* t32,
                     long long* lo) {
  if (h->hasCE)
    return h->fail(SG_ERR_STATE, "sg_transport_bank_noalloc: multigroup handles only (this handle holds "
                                 "continuous-energy data; use sg_transport_bank)");
  if (!h->hasGeom || !h->hasMG) return h->fail(SG_ERR_STATE, "upload geometry and MG data first");
  if (admin < 0 || admin >= (int)h->admins.size()) return h->fail(SG_ERR_BAD_ARG, "bad tally admin");
  v->stream = h->stream;
  v->precision = h->cfg.precision;
  v->transport = h->cfg.transport;
  v->maxl = h->maxl;
  v->err = &h->err;
  std::memset(t64, 0, sizeof(*t64));
  std::memset(t32, 0, sizeof(*t32));
  long long hi = 0;
  int rc = build_clerks<double>(h, admin, *t64, *lo, hi);
  if (rc) return rc;
  rc = build_clerks<float>(h, admin, *t32, *lo, hi);
  if (rc) return rc;
  t64->geom = h->g64;
  t64->mg = h->mg64;
  t32->geom = h->gMx;
  t32->mg = h->mgMx;
  t64->acc = h->acc.p + *lo;
  t32->acc = h->acc.p + *lo;
  t64->acc_n = t32->acc_n = (int)(hi - *lo);
  t64->use_cache = t32->use_cache = transport_cache(h->cfg.transport);
  t64->max_segments = t32->max_segments = 1000000;
  t64->ht_cutoff = h->htCutoff;
  t32->ht_cutoff = (float)h->htCutoff;
  t64->coll_imp = t32->coll_imp = h->collImp ? 1 : 0;
  t64->coll = h->collImp ? h->dColl64.p : nullptr;
  t32->coll = h->collImp ? h->dColl32.p : nullptr;
  t64->lean = lean_launch(h, *t64) ? 1 : 0;
  t32->lean = lean_launch(h, *t32) ? 1 : 0;
  return SG_OK;
}

// Bridge for the batched form (sg_batch_host.cu): builds one problem's resident data with the
// single-problem builders, into a caller-owned device block through a host image (no allocation).
int sg::stage_problem(const sg_geometry_desc* g, const sg_mg_desc* mg, const sg_point_source_desc* src,
                      const sg_tally_desc* tally, char* dev, std::vector<char>* host, size_t cap, size_t* bytes,
                      StagedProblem* out, std::string* err) {
  sg_handle_t H;
  H.cfg = sg_config{};
  Staging st;
  st.dev = dev;
  st.host = host;
  st.cap = cap;
  if (dev && host) host->clear();
  Staging* prev = t_staging;
  t_staging = &st;
  int rc = build_geometry(&H, g);
  if (!rc) rc = build_mg(&H, mg);
  if (!rc && src->n_prob_g > 0) {
    std::vector<double> v(src->prob_g, src->prob_g + src->n_prob_g);
    if (H.probG.upload(v, nullptr) != cudaSuccess) rc = H.fail(SG_ERR_OOM, "batch: problem larger than its block");
  }
  Admin A;
  if (!rc) rc = build_admin(&H, tally, A);
  if (!rc)
    for (const auto& d : A.clerks)
      if (d.type == SG_CLERK_KEFF_ANALOG || d.type == SG_CLERK_KEFF_IMPLICIT)
        rc = H.fail(SG_ERR_BAD_ARG, "batch: k clerks need an eigenvalue run; batched problems are fixed-source");
  if (!rc && H.anyFissile) rc = H.fail(SG_ERR_BAD_ARG, "batch: fixed-source problems with fissile materials are not supported");
  if (!rc) {
    A.off = 0;
    H.admins.push_back(A);
    long long lo = 0, hi = 0;
    std::memset(&out->t64, 0, sizeof(out->t64));
    std::memset(&out->t32, 0, sizeof(out->t32));
    rc = build_clerks<double>(&H, 0, out->t64, lo, hi);
    if (!rc) rc = build_clerks<float>(&H, 0, out->t32, lo, hi);
  }
  t_staging = prev;
  *bytes = st.used;
  if (rc) {
    if (err) *err = H.err;
    return rc;
  }
  out->t64.geom = H.g64;
  out->t64.mg = H.mg64;
  out->t32.geom = H.gMx;
  out->t32.mg = H.mgMx;
  out->maxl = H.maxl;
  out->n_bins = A.N;
  out->norm_addr = A.normAddr >= 1 ? A.normAddr - 1 : -1;
  out->norm_val = A.normVal;
  out->prob_g = H.probG.p;
  out->any_fissile = H.anyFissile;
  out->clerks = A.clerks;
  out->addr = A.addr;
  out->tab64 = A.tab64;
  out->tab32 = A.tab32;
  return SG_OK;
}

int sg::plain_fixed_source(sg_handle h, const StagedProblem& p, const sg_point_source_desc* src, double* acc,
                           double* bin, double* csum, double* csum2, int pop, int cycles,
                           unsigned long long master, sg_cycle_stats* total) {
  if (pop > h->cap) return h->fail(SG_ERR_BANK_OVERFLOW, "plain: population larger than the work handle's banks");
  // bind
  const DGeom g64 = h->g64, gMx = h->gMx;
  const DMG<double> mg64 = h->mg64;
  const DMG<float> mgMx = h->mgMx;
  const int maxl = h->maxl;
  const bool hasGeom = h->hasGeom, hasMG = h->hasMG, hasCE = h->hasCE, anyFissile = h->anyFissile, hasSource = h->hasSource;
  const PointSourceArgs psrc = h->psrc;
  std::vector<Admin> admins;
  admins.swap(h->admins);
  DArr<double>* arrs[4] = {&h->acc, &h->bin, &h->csum, &h->csum2};
  double* mine[4] = {acc, bin, csum, csum2};
  DArr<double> kept[4];
  for (int i = 0; i < 4; ++i) {
    kept[i] = *arrs[i];
    arrs[i]->p = mine[i];
    arrs[i]->n = (size_t)p.n_bins;
    arrs[i]->borrowed = true;
  }
  h->g64 = p.t64.geom;
  h->gMx = p.t32.geom;
  h->mg64 = p.t64.mg;
  h->mgMx = p.t32.mg;
  h->maxl = p.maxl;
  h->hasGeom = h->hasMG = true;
  h->hasCE = false;
  h->anyFissile = p.any_fissile;
  PointSourceArgs& q = h->psrc;
  for (int i = 0; i < 3; ++i) { q.r[i] = src->r[i]; q.dir[i] = src->dir[i]; }
  q.isotropic = src->isotropic;
  q.G = src->G;
  q.E = 0.0;
  q.n_prob_g = src->n_prob_g;
  q.prob_g = src->n_prob_g > 0 ? p.prob_g : nullptr;
  h->hasSource = true;
  Admin A;
  A.clerks = p.clerks;
  A.addr = p.addr;
  A.tab64 = p.tab64;
  A.tab32 = p.tab32;
  A.N = p.n_bins;
  A.off = 0;
  A.normAddr = p.norm_addr >= 0 ? p.norm_addr + 1 : -1;
  A.normVal = p.norm_val;
  h->admins.push_back(A);
  // run: fixedSourcePhysicsPackage%cycles, one call per cycle
  int rc = SG_OK;
  std::memset(total, 0, sizeof(*total));
  uint64_t m = master;
  for (int c = 0; c < cycles && rc == SG_OK; ++c) {
    sg_cycle_stats st{};
    rc = sg_fixed_source_cycle(h, 0, pop, &m, &st);
    total->n_histories += st.n_histories;
    total->n_events += st.n_events;
    total->n_collisions += st.n_collisions;
    total->transport_ms += st.transport_ms;
    total->cycle_ms += st.cycle_ms;
    total->n_kernels += st.n_kernels;
  }
  // restore
  h->admins.swap(admins);
  for (int i = 0; i < 4; ++i) *arrs[i] = kept[i];
  h->g64 = g64; h->gMx = gMx; h->mg64 = mg64; h->mgMx = mgMx; h->maxl = maxl;
  h->hasGeom = hasGeom; h->hasMG = hasMG; h->hasCE = hasCE; h->anyFissile = anyFissile;
  h->psrc = psrc; h->hasSource = hasSource;
  return rc;
}

// ====================================================================== C ABI
extern "C" {

int32_t sg_create(const sg_config* cfg, sg_handle* out) {
  if (!cfg || !out) return SG_ERR_BAD_ARG;
  *out = nullptr;
  if (cfg->precision != SG_PREC_FP64 && cfg->precision != SG_PREC_MIXED) return SG_ERR_BAD_ARG;
  if (cfg->transport < SG_TRANSPORT_ST || cfg->transport > SG_TRANSPORT_HT_NOCACHE) return SG_ERR_BAD_ARG;
  if (!(cfg->ht_cutoff >= 0.0 && cfg->ht_cutoff < 1.0)) return SG_ERR_BAD_ARG;
  if (cfg->max_bank <= 0) return SG_ERR_BAD_ARG;
  if (cfg->form != SG_FORM_EVENT && cfg->form != SG_FORM_HISTORY) return SG_ERR_BAD_ARG;
  sg_handle h = new sg_handle_t();
  h->cfg = *cfg;
  h->cap = cfg->max_bank;
  h->htCutoff = cfg->ht_cutoff > 0.0 ? cfg->ht_cutoff : 0.9;
  if (cudaSetDevice(cfg->device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return SG_ERR_CUDA;
  }
  int rc = alloc_work(h);
  if (rc) { delete h; return rc; }
  for (auto& e : h->ev)
    if (cudaEventCreate(&e) != cudaSuccess) { delete h; return SG_ERR_CUDA; }
  if (cudaStreamCreateWithFlags(&h->copyStream, cudaStreamNonBlocking) != cudaSuccess) { delete h; return SG_ERR_CUDA; }
  for (auto& e : h->copyEv)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) { delete h; return SG_ERR_CUDA; }
  *out = h;
  return SG_OK;
}

int32_t sg_destroy(sg_handle h) {
  if (!h) return SG_ERR_BAD_ARG;
  cudaStreamSynchronize(h->stream);
  for (auto& b : h->bank) b.free();
  h->surfs64.free(); h->surfsMx.free(); h->unis64.free(); h->unisMx.free(); h->uniCells.free();
  h->cellPtr.free(); h->cellSurf.free(); h->cellComplex.free(); h->rot64.free(); h->rotF.free();
  h->fsR.free(); h->fsDir.free(); h->fsWgt.free(); h->fsE.free(); h->fsG.free(); h->pinRsq.free(); h->pinTol64.free(); h->pinTolMx.free(); h->graph.free();
  h->pinRsqF.free(); h->pinTolF.free();
  for (auto& a : h->mgD) a.free();
  for (auto& a : h->mgF) a.free();
  h->fissile.free(); h->acc.free(); h->bin.free(); h->csum.free(); h->csum2.free();
  h->sR.free(); h->sDir.free(); h->sWgt.free(); h->sTime.free(); h->sG.free(); h->sBrood.free(); h->sSeq.free();
  h->sCursor.free(); h->histN.free(); h->start.free(); h->scanTmp.free(); h->flags.free(); h->pos.free();
  h->kbuf.free(); h->keys.free(); h->sel.free(); h->hist16.free(); h->winCnt.free(); h->winCand.free(); h->shardKeys.free(); h->sumPart.free(); h->scal.free();
  h->totals.free(); h->ctr.free(); h->recColl.free(); h->recRng.free(); h->probG.free();
  h->pR0.free(); h->pRl.free(); h->pU.free(); h->pW.free(); h->pW0.free(); h->pTime.free(); h->pTrack.free();
  h->pGeo.free(); h->pInts.free(); h->pRng.free(); h->qT0.free(); h->qT1.free(); h->qC.free(); h->qCtr.free();
  h->ceE.free(); h->ceUE.free(); h->ceXs64.free(); h->ceA64.free(); h->ceKT64.free(); h->ceDens64.free();
  h->ceMaj64.free(); h->ceXsF.free(); h->ceAF.free(); h->ceKTF.free(); h->ceDensF.free(); h->ceMajF.free();
  h->ceOff.free(); h->ceHash.free(); h->ceUHash.free(); h->ceLUHash.free(); h->ceLU.free(); h->ceLIdx.free(); h->ceLMaj.free(); h->ceMatPtr.free(); h->ceMatNuc.free(); h->ceAct.free();
  h->pE.free();
  h->wwLo64.free(); h->wwUp64.free(); h->wwLo32.free(); h->wwUp32.free(); h->dColl64.free(); h->dColl32.free();
  h->bufR.free(); h->bufE.free(); h->bufU64.free(); h->bufW64.free(); h->bufT64.free(); h->bufU32.free();
  h->bufW32.free(); h->bufT32.free(); h->bufG.free();
  for (auto& a : h->mapTab64) a.free();
  for (auto& a : h->mapTab32) a.free();
  for (auto& a : h->mapTabCell) a.free();
  for (auto& e : h->ev) if (e) cudaEventDestroy(e);
  for (auto& e : h->copyEv) if (e) cudaEventDestroy(e);
  if (h->copyStream) cudaStreamDestroy(h->copyStream);
  cudaStreamDestroy(h->stream);
  delete h;
  return SG_OK;
}

int32_t sg_last_error(sg_handle h, char* buf, size_t len) {
  if (!h || !buf || len == 0) return SG_ERR_BAD_ARG;
  std::snprintf(buf, len, "%s", h->err.c_str());
  return SG_OK;
}

int32_t sg_upload_geometry(sg_handle h, const sg_geometry_desc* g) {
  if (!h || !g) return SG_ERR_BAD_ARG;
  return build_geometry(h, g);
}

int32_t sg_upload_mg(sg_handle h, const sg_mg_desc* mg) {
  if (!h || !mg) return SG_ERR_BAD_ARG;
  if (h->hasCE) return h->fail(SG_ERR_STATE, "mg: the handle already holds CE data");
  return build_mg(h, mg);
}

int32_t sg_upload_ce(sg_handle h, const sg_ce_desc* ce) {
  if (!h || !ce) return SG_ERR_BAD_ARG;
  return build_ce(h, ce);
}

int32_t sg_upload_tally(sg_handle h, const sg_tally_desc* t, int32_t* admin_out) {
  if (!h || !t || !admin_out || t->n_clerks < 0) return SG_ERR_BAD_ARG;
  Admin A;
  int rc = build_admin(h, t, A);
  if (rc) return rc;
  A.off = h->totalBins;
  // grow the device score memory, keeping what earlier admins hold
  long long newTotal = h->totalBins + A.N;
  DArr<double>* arrs[4] = {&h->acc, &h->bin, &h->csum, &h->csum2};
  for (DArr<double>* a : arrs) {
    std::vector<double> old(h->totalBins);
    if (h->totalBins) { cudaError_t e = cudaMemcpy(old.data(), a->p, h->totalBins * sizeof(double), cudaMemcpyDeviceToHost); if (e) return h->fail(SG_ERR_CUDA, "tally copy"); }
    old.resize(newTotal > 0 ? newTotal : 1, 0.0);
    CK(a->upload(old, h->stream));
  }
  h->totalBins = newTotal;
  h->admins.push_back(A);
  *admin_out = (int32_t)h->admins.size() - 1;
  return SG_OK;
}

int32_t sg_attach_tally(sg_handle h, int32_t admin, int32_t atch) {
  if (!h || admin < 0 || admin >= (int)h->admins.size() || atch < 0 || atch >= (int)h->admins.size() || admin == atch)
    return SG_ERR_BAD_ARG;
  h->admins[admin].atch = atch;
  return SG_OK;
}

int32_t sg_set_point_source(sg_handle h, const sg_point_source_desc* src) {
  if (!h || !src) return SG_ERR_BAD_ARG;
  PointSourceArgs& p = h->psrc;
  for (int i = 0; i < 3; ++i) { p.r[i] = src->r[i]; p.dir[i] = src->dir[i]; }
  p.isotropic = src->isotropic;
  p.G = src->G;
  p.E = src->E;
  if (h->hasCE && !(src->E > 0.0)) return h->fail(SG_ERR_BAD_ARG, "point source: CE problems need E > 0");
  p.n_prob_g = src->n_prob_g;
  if (src->n_prob_g > 0) {
    std::vector<double> v(src->prob_g, src->prob_g + src->n_prob_g);
    CK(h->probG.upload(v, h->stream));
    p.prob_g = h->probG.p;
  } else p.prob_g = nullptr;
  h->hasSource = true;
  return SG_OK;
}

int32_t sg_generate_source(sg_handle h, uint64_t master_state, int32_t n, sg_bank* out) {
  if (!h || !out || n < 0 || n > h->cap) return SG_ERR_BAD_ARG;
  if (!h->hasSource) return h->fail(SG_ERR_STATE, "no point source set");
  PointSourceArgs a = h->psrc;
  a.out = h->bank[h->cur].view();
  a.n = n;
  a.master = master_state;
  if (n > 0) CK(launch_point_source(a, h->stream));
  return d2h_bank(h, a.out, n, out);
}

int32_t sg_transport_bank(sg_handle h, int32_t admin, const sg_bank* in, int32_t n, uint64_t master_state,
                          double k_eff, sg_bank* next, int32_t next_cap, sg_cycle_stats* stats) {
  if (!h || !in || n < 0 || n > h->cap) return SG_ERR_BAD_ARG;
  DBank A = h->bank[0].view(), B = h->bank[1].view();
  h->launches = 0;
  CK(cudaEventRecord(h->ev[2], h->stream));
  int rc = SG_OK;
  if (!mapped_host_bank(h, in, &A)) {
    A = h->bank[0].view();
    rc = h2d_bank(h, in, n, A);
    if (rc) return rc;
  }
  CK(cudaMemcpyAsync(h->scal.p + 0, &k_eff, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  // popWeight of the bank given (particleDungeon_class.f90:358-375), summed on the device
  CK(deterministic_sum(A.wgt, n, h->sumPart.p, h->scal.p + 2, h->stream));
  h->launches += 2;
  int S = 0;
  sg_cycle_stats st{};
  rc = gen_loop(h, admin, A, n, master_state, h->scal.p + 0, B, h->cap, &S, &st);
  if (rc) return rc;
  h->eigenReady = false;   // the resident banks were overwritten
  if (next && S > 0) {
    if (S > next_cap) return h->fail(SG_ERR_BANK_OVERFLOW, "next bank capacity too small");
    CK(deterministic_sum(B.wgt, S, h->sumPart.p, h->scal.p + 3, h->stream));
    h->launches += 2;
    rc = d2h_bank(h, B, S, next);
    if (rc) return rc;
  }
  CK(cudaEventRecord(h->ev[3], h->stream));
  CK(cudaStreamSynchronize(h->stream));
  float cyc = 0.f;
  CK(cudaEventElapsedTime(&cyc, h->ev[2], h->ev[3]));
  if (stats) {
    double w[2] = {0.0, 0.0};
    CK(cudaMemcpy(w, h->scal.p + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost));
    *stats = st;
    stats->cycle_ms = cyc;
    stats->n_kernels = h->launches;
    stats->k_eff = k_eff;
    stats->k_new = k_eff;
    stats->start_weight = n > 0 ? w[0] : 0.0;
    stats->end_weight = (next && S > 0) ? w[1] : 0.0;
  }
  return SG_OK;
}

int32_t sg_tally_cycle_start(sg_handle h, int32_t admin, double w) {
  if (!h || admin < 0 || admin >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  return cycle_start(h, admin, nullptr, w);
}

int32_t sg_tally_cycle_end(sg_handle h, int32_t admin, double w, double k_end) {
  if (!h || admin < 0 || admin >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  CK(cudaMemcpyAsync(h->scal.p + 3, &w, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->scal.p + 4, &k_end, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int rc = cycle_end(h, admin, h->scal.p + 3, h->scal.p + 4, -1, nullptr);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return SG_OK;
}

int32_t sg_tally_size(sg_handle h, int32_t admin, int64_t* n) {
  if (!h || !n || admin < 0 || admin >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  *n = h->admins[admin].N;
  return SG_OK;
}

int32_t sg_get_bins(sg_handle h, int32_t admin, double* bins, int64_t n) {
  if (!h || !bins || admin < 0 || admin >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  const Admin& A = h->admins[admin];
  if (n < A.N) return h->fail(SG_ERR_BAD_ARG, "get_bins: buffer smaller than the tally");
  if (A.N == 0) return SG_OK;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(bins, h->bin.p + A.off, A.N * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(bins + n, h->csum.p + A.off, A.N * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(bins + 2 * n, h->csum2.p + A.off, A.N * sizeof(double), cudaMemcpyDeviceToHost));
  return SG_OK;
}

int32_t sg_get_keff(sg_handle h, int32_t admin, double* k, double* sd) {
  if (!h || !k || !sd || admin < 0 || admin >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  const Admin& A = h->admins[admin];
  long long addr = A.keffImplicit >= 0 ? A.keffImplicit + 4 : (A.keffAnalog >= 0 ? A.keffAnalog + 2 : -1);
  if (addr < 0) return h->fail(SG_ERR_BAD_ARG, "admin has no k clerk");
  double cs[2];
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(&cs[0], h->csum.p + A.off + addr, sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&cs[1], h->csum2.p + A.off + addr, sizeof(double), cudaMemcpyDeviceToHost));
  int N = A.batchN;                                  // scoreMemory%getResult (:537-573)
  double mean = cs[0] / N;
  double inv_N = 1.0 / N;
  double inv_Nm1 = (N != 1) ? 1.0 / (N - 1) : 1.0;
  double var = cs[1] * inv_N * inv_Nm1 - mean * mean * inv_Nm1;
  *k = mean;
  *sd = std::sqrt(var);
  return SG_OK;
}

int32_t sg_eigen_init(sg_handle h, int32_t pop, uint64_t master_state, double k0) {
  if (!h || pop <= 0 || pop > h->cap) return SG_ERR_BAD_ARG;
  if (!h->hasGeom || !h->hasMG) return h->fail(SG_ERR_STATE, "eigenvalue runs need geometry and fissile MG data");
  h->cur = 0;
  CK(cudaMemsetAsync(h->totals.p, 0, 8 * sizeof(int), h->stream));
  CK(launch_fission_source(h->g64, h->mg64, h->bank[0].view(), pop, master_state, h->bounds, h->maxl,
                           h->totals.p + 3, h->stream));
  int e = 0;
  CK(cudaMemcpyAsync(&e, h->totals.p + 3, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (e) return h->fail(e, "fission source: no fissile material found");
  h->pop = pop;
  h->master = rng_stride(master_state, pop);        // generateInitialState (:363-364)
  h->k = k0;
  double kk[2] = {k0, 1.0};                          // k used, and nextCycle%k_eff (dungeon default 1)
  CK(cudaMemcpyAsync(h->scal.p + 0, &kk[0], sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->scal.p + 4, &kk[1], sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->eigenReady = true;
  return SG_OK;
}

int32_t sg_eigen_cycle(sg_handle h, int32_t admin, int32_t atch, sg_cycle_stats* stats) {
  if (!h || !h->eigenReady) return h ? h->fail(SG_ERR_STATE, "call sg_eigen_init first") : SG_ERR_BAD_ARG;
  if (admin < 0 || admin >= (int)h->admins.size() || atch < 0 || atch >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  h->launches = 0;
  CK(cudaEventRecord(h->ev[2], h->stream));
  DBank A = h->bank[h->cur].view();
  return eigen_cycle_core(h, admin, atch, A, h->bank[1 - h->cur].view(), A, stats);
}

int32_t sg_eigen_cycle_bank(sg_handle h, int32_t admin, int32_t atch, const sg_bank* in, int32_t pop,
                            uint64_t* master_state, double* k_eff, double k_end, sg_bank* out,
                            sg_cycle_stats* stats) {
  if (!h || !in || !out || !master_state || !k_eff || pop <= 0 || pop > h->cap) return SG_ERR_BAD_ARG;
  if (admin < 0 || admin >= (int)h->admins.size() || atch < 0 || atch >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  if (!h->hasGeom || !h->hasMG) return h->fail(SG_ERR_STATE, "eigenvalue cycles need geometry and fissile MG data");
  if (!out->r || !out->dir || !out->wgt || !out->G)
    return h->fail(SG_ERR_BAD_ARG, "sg_eigen_cycle_bank: the output bank needs r, dir, wgt and G");
  cudaStream_t s = h->stream;
  h->launches = 0;
  CK(cudaEventRecord(h->ev[2], s));
  // thisCycle: read in place from mapped host memory, else staged in bank 0; the fission sites go to
  // bank 1 and the normalised next-cycle bank to bank 0 (the staged input is consumed by then)
  DBank res = h->bank[0].view(), in_d;
  if (!mapped_host_bank(h, in, &in_d)) {
    in_d = res;
    int rc = h2d_bank(h, in, pop, in_d);
    if (rc) return rc;
  }
  double kk[2] = {*k_eff, k_end};                    // k used this cycle, end%k_eff
  CK(cudaMemcpyAsync(h->scal.p + 0, &kk[0], sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(h->scal.p + 4, &kk[1], sizeof(double), cudaMemcpyHostToDevice, s));
  h->pop = pop;
  h->master = *master_state;
  h->k = *k_eff;
  h->cur = 0;
  int rc = eigen_cycle_core(h, admin, atch, in_d, h->bank[1].view(), res, nullptr);
  h->eigenReady = false;   // the device banks hold no resident run for sg_eigen_cycle
  if (rc) return rc;
  rc = d2h_bank(h, res, pop, out);
  if (rc) return rc;
  CK(cudaEventRecord(h->ev[3], s));
  CK(cudaStreamSynchronize(s));
  *master_state = h->master;
  *k_eff = h->k;
  if (stats) {
    *stats = h->lastStats;
    float cyc = 0.f;
    CK(cudaEventElapsedTime(&cyc, h->ev[2], h->ev[3]));
    stats->cycle_ms = cyc;
  }
  return SG_OK;
}

int32_t sg_eigen_state(sg_handle h, uint64_t* master, double* k) {
  if (!h || !master || !k) return SG_ERR_BAD_ARG;
  *master = h->master;
  *k = h->k;
  return SG_OK;
}

int32_t sg_eigen_get_bank(sg_handle h, sg_bank* out, int32_t cap, int32_t* pop) {
  if (!h || !out || !pop) return SG_ERR_BAD_ARG;
  *pop = h->pop;
  return d2h_bank(h, h->bank[h->cur].view(), std::min(cap, h->pop), out);
}

int32_t sg_fixed_source_cycle(sg_handle h, int32_t admin, int32_t n, uint64_t* master_state, sg_cycle_stats* stats) {
  return sg_fixed_source_cycle_shard(h, admin, n, n, master_state, stats);
}

int32_t sg_fixed_source_cycle_shard(sg_handle h, int32_t admin, int32_t n, int32_t total, uint64_t* master_state,
                                    sg_cycle_stats* stats) {
  if (!h || !master_state || n <= 0 || n > h->cap || total < n) return SG_ERR_BAD_ARG;
  if (!h->hasSource && !h->hasFileSource) return h->fail(SG_ERR_STATE, "no point or file source set");
  if (h->anyFissile) return h->fail(SG_ERR_BAD_ARG, "fixed-source runs with fissile materials are not supported");
  cudaStream_t s = h->stream;
  DBank A = h->bank[0].view(), B = h->bank[1].view();
  h->launches = 0;
  CK(cudaEventRecord(h->ev[2], s));
  h->launches += 1;                                                      // fixedSource%generate
  if (h->hasFileSource) {
    FileSourceArgs f;
    f.geom = h->g64;
    f.r = h->fsR.p; f.dir = h->fsDir.p; f.wgt = h->fsWgt.p;
    f.E = h->hasCE ? h->fsE.p : nullptr;
    f.G = h->hasCE ? nullptr : h->fsG.p;
    f.N = h->fileN;
    f.out = A;
    f.n = n;
    f.master = *master_state;
    f.err = h->totals.p + 5;
    CK(cudaMemsetAsync(h->totals.p + 5, 0, sizeof(int), s));
    CK(launch_file_source(f, h->maxl, s));
    int ferr = 0;
    CK(cudaMemcpyAsync(&ferr, h->totals.p + 5, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (ferr) return h->fail(ferr, "file source: a particle is outside the geometry or in an undefined cell");
  } else {
    PointSourceArgs a = h->psrc;
    a.out = A;
    a.n = n;
    a.master = *master_state;
    CK(launch_point_source(a, s));
  }
  unsigned long long m = rng_stride(*master_state, total);               // :189
  int rc = cycle_start(h, admin, nullptr, (double)n);
  if (rc) return rc;
  const double one = 1.0;
  CK(cudaMemcpyAsync(h->scal.p + 0, &one, sizeof(double), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(h->scal.p + 4, &one, sizeof(double), cudaMemcpyHostToDevice, s));
  int S = 0;
  sg_cycle_stats st{};
  rc = gen_loop(h, admin, A, n, m, h->scal.p + 0, B, h->cap, &S, &st);
  if (rc) return rc;
  m = rng_stride(m, total);                                              // :264
  const double wn = (double)n;
  CK(cudaMemcpyAsync(h->scal.p + 3, &wn, sizeof(double), cudaMemcpyHostToDevice, s));
  rc = cycle_end(h, admin, h->scal.p + 3, h->scal.p + 4, -1, nullptr);   // :267
  if (rc) return rc;
  CK(cudaEventRecord(h->ev[3], s));
  CK(cudaStreamSynchronize(s));
  float cyc = 0.f;
  CK(cudaEventElapsedTime(&cyc, h->ev[2], h->ev[3]));
  h->eigenReady = false;
  *master_state = m;
  if (stats) {
    *stats = st;
    stats->start_weight = n;
    stats->end_weight = n;
    stats->k_eff = 1.0;
    stats->k_new = 1.0;
    stats->cycle_ms = cyc;
    stats->n_kernels = h->launches;
  }
  return SG_OK;
}

// particleDungeon%normSize_Repr, one process's part (particleDungeon_class.f90:431-590 with MPI).
// The keys of all tot_sites sites are the master stream's draws in process order (:469-494), so
// every process generates them all and finds the same heap threshold; its own sites take the keys
// from sites_before on (the seed the master would have broadcast, :497-500).
int32_t sg_normalise_shard(sg_handle h, const sg_bank* sites, int32_t n, int64_t sites_before, int64_t tot_sites,
                           int32_t tot_pop, uint64_t master_state, sg_bank* out, int32_t out_cap, int32_t* n_out) {
  if (!h || !sites || !out || !n_out) return SG_ERR_BAD_ARG;
  if (!h->hasGeom || !h->hasMG) return h->fail(SG_ERR_STATE, "sg_normalise_shard: multigroup eigenvalue banks only");
  if (n < 0 || n > h->cap || sites_before < 0 || tot_sites < sites_before + n || tot_sites > INT32_MAX || tot_pop <= 0)
    return h->fail(SG_ERR_BAD_ARG, "sg_normalise_shard: bad sizes");
  if (tot_sites == 0) return h->fail(SG_ERR_STATE, "normSize: empty fission bank");
  if (n > 0 && (!sites->r || !sites->dir || !sites->G || !sites->brood_id))
    return h->fail(SG_ERR_BAD_ARG, "sg_normalise_shard: the sites need r, dir, G and brood_id");
  if (!out->r || !out->dir || !out->wgt || !out->G)
    return h->fail(SG_ERR_BAD_ARG, "sg_normalise_shard: the output bank needs r, dir, wgt and G");
  for (int i = 0; i < n; ++i)
    if (sites->brood_id[i] < 1 || sites->brood_id[i] > h->cap || (i > 0 && sites->brood_id[i] < sites->brood_id[i - 1]))
      return h->fail(SG_ERR_BAD_ARG, "sg_normalise_shard: brood IDs must be sorted and within 1..max_bank");
  const int S = (int)tot_sites;
  const long long excess = tot_sites - tot_pop;
  const int heap = excess > 0 ? (int)excess : (excess < 0 ? (int)((-excess) % tot_sites) : 0);
  const int n_copies = excess < 0 ? (int)((-excess) / tot_sites) : 0;
  cudaStream_t s = h->stream;
  h->eigenReady = false;   // the device banks are used as scratch
  DBank in = h->bank[1].view(), res = h->bank[0].view();
  *n_out = 0;
  if (n > 0) {
    int rc = h2d_bank(h, sites, n, in);
    if (rc) return rc;
    CK(cudaMemcpyAsync(in.brood, sites->brood_id, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  }
  if (heap > 0) {
    if (h->shardKeys.n < (size_t)S) CK(h->shardKeys.alloc(S));
    k_rn_keys<<<((S + 31) / 32 + 127) / 128, 128, 0, s>>>(master_state, S, h->shardKeys.p);
    CK(cudaGetLastError());
    CK(quantile_select(h->shardKeys.p, S, heap, h->sel.p, h->kbuf.p, h->hist16.p, h->winCnt.p, h->winCand.p, s));
  }
  const unsigned long long* keys = heap > 0 ? h->shardKeys.p + sites_before : nullptr;
  int m = n;
  if (n > 0 && excess > 0) {
    CK(launch_flags(keys, n, h->sel.p, 1, h->flags.p, s));
    CK(cudaMemsetAsync(h->flags.p + n, 0, sizeof(int), s));
    CK(exclusive_scan(h->flags.p, n + 1, h->pos.p, h->scanTmp.p, h->totals.p + 1, s));
    CK(launch_compact(in, n, h->flags.p, h->pos.p, res, s));
    CK(cudaMemcpyAsync(&m, h->totals.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  } else if (n > 0 && excess < 0) {
    if (heap > 0) CK(launch_flags(keys, n, h->sel.p, 0, h->flags.p, s));
    else CK(cudaMemsetAsync(h->flags.p, 0, (size_t)n * sizeof(int), s));
    CK(cudaMemsetAsync(h->flags.p + n, 0, sizeof(int), s));
    CK(exclusive_scan(h->flags.p, n + 1, h->pos.p, h->scanTmp.p, h->totals.p + 2, s));
    int dups = 0;
    CK(cudaMemcpyAsync(&dups, h->totals.p + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if ((long long)n * (n_copies + 1) + dups > h->cap) return h->fail(SG_ERR_BANK_OVERFLOW, "normSize: bank overflow");
    m = n * (n_copies + 1) + dups;
    CK(launch_brood_starts(in.brood, n, sites->brood_id[n - 1], h->start.p, s));
    CK(launch_replicate(in, n, h->flags.p, h->pos.p, h->start.p, n_copies, res, s));
  } else if (n > 0) {
    res = in;
  }
  if (m > out_cap) return h->fail(SG_ERR_BANK_OVERFLOW, "sg_normalise_shard: output bank too small");
  int rc = d2h_bank(h, res, m, out);
  if (rc) return rc;
  *n_out = m;
  return SG_OK;
}

int32_t sg_tally_get_scores(sg_handle h, int32_t admin, double* scores, int64_t n) {
  if (!h || !scores || admin < 0 || admin >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  const Admin& A = h->admins[admin];
  if (n < A.N) return h->fail(SG_ERR_BAD_ARG, "get_scores: buffer smaller than the tally");
  if (A.N == 0) return SG_OK;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(scores, h->acc.p + A.off, A.N * sizeof(double), cudaMemcpyDeviceToHost));
  return SG_OK;
}

int32_t sg_tally_set_scores(sg_handle h, int32_t admin, const double* scores, int64_t n) {
  if (!h || !scores || admin < 0 || admin >= (int)h->admins.size()) return SG_ERR_BAD_ARG;
  const Admin& A = h->admins[admin];
  if (n < A.N) return h->fail(SG_ERR_BAD_ARG, "set_scores: buffer smaller than the tally");
  if (A.N == 0) return SG_OK;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(h->acc.p + A.off, scores, A.N * sizeof(double), cudaMemcpyHostToDevice));
  return SG_OK;
}

// ------------------------------------------------------------------ bank files
int32_t sg_bank_write_file(const char* path, const sg_bank* b, int32_t n, int32_t binary) {
  if (!path || !b || n < 0 || (n > 0 && (!b->r || !b->dir))) return SG_ERR_BAD_ARG;
  std::string name = std::string(path) + (binary ? ".bin" : ".txt");
  FILE* f = std::fopen(name.c_str(), binary ? "wb" : "w");
  if (!f) return SG_ERR_BAD_ARG;
  for (int i = 0; i < n; ++i) {                 // r, dir, E, real(G), real(broodID), wgt
    double v[10];
    for (int k = 0; k < 3; ++k) { v[k] = b->r[3 * i + k]; v[3 + k] = b->dir[3 * i + k]; }
    v[6] = b->E ? b->E[i] : 0.0;
    v[7] = b->G ? (double)b->G[i] : 0.0;
    v[8] = b->brood_id ? (double)b->brood_id[i] : 0.0;
    v[9] = b->wgt ? b->wgt[i] : 1.0;
    bool ok;
    if (binary) ok = std::fwrite(v, sizeof(double), 10, f) == 10;
    else ok = std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", v[0], v[1], v[2],
                           v[3], v[4], v[5], v[6], v[7], v[8], v[9]) > 0;
    if (!ok) { std::fclose(f); return SG_ERR_BAD_ARG; }
  }
  return std::fclose(f) == 0 ? SG_OK : SG_ERR_BAD_ARG;
}

namespace {
// readArray (genericProcedures.f90) of fileSource: ten numbers per particle
bool read_particle(FILE* f, bool binary, double v[10]) {
  if (binary) return std::fread(v, sizeof(double), 10, f) == 10;
  for (int k = 0; k < 10; ++k)
    if (std::fscanf(f, "%lf", &v[k]) != 1) return false;
  return true;
}
}  // namespace

int32_t sg_bank_count_file(const char* path, int32_t binary, int64_t* n) {
  if (!path || !n) return SG_ERR_BAD_ARG;
  FILE* f = std::fopen(path, binary ? "rb" : "r");
  if (!f) return SG_ERR_BAD_ARG;
  double v[10];
  long long c = 0;
  while (read_particle(f, binary != 0, v)) ++c;
  std::fclose(f);
  *n = c;
  return SG_OK;
}

int32_t sg_bank_read_file(const char* path, int32_t binary, sg_bank* b, int32_t cap, int32_t* n) {
  if (!path || !b || !n || cap < 0) return SG_ERR_BAD_ARG;
  FILE* f = std::fopen(path, binary ? "rb" : "r");
  if (!f) return SG_ERR_BAD_ARG;
  double v[10];
  int c = 0;
  while (c < cap && read_particle(f, binary != 0, v)) {
    for (int k = 0; k < 3; ++k) {
      if (b->r) b->r[3 * c + k] = v[k];
      if (b->dir) b->dir[3 * c + k] = v[3 + k];
    }
    if (b->E) b->E[c] = v[6];
    if (b->G) b->G[c] = (int)v[7];
    if (b->brood_id) b->brood_id[c] = (int)v[8];
    if (b->wgt) b->wgt[c] = v[9];
    if (b->time) b->time[c] = 0.0;
    ++c;
  }
  std::fclose(f);
  *n = c;
  return SG_OK;
}

// neutronMGimp / neutronCEimp%init (neutronCEimp_class.f90:160-232) and weightWindowsField%init
// (weightWindowsField_class.f90:75-111).  The split buffer is allocated here, not when a cycle runs:
// it holds `depth` particles for every thread a persistent launch can have (SMs x threads per SM).
int32_t sg_set_collision(sg_handle h, const sg_collision_desc* d) {
  if (!h || !d) return SG_ERR_BAD_ARG;
  if (d->kind == SG_COLL_STD) { h->collImp = false; h->collBuf = false; return SG_OK; }
  if (d->kind != SG_COLL_IMP) return h->fail(SG_ERR_BAD_ARG, "collision: unknown processor");
  if (d->max_split < 1) return h->fail(SG_ERR_BAD_ARG, "collision: maxSplit must be at least 1");
  if (d->split && d->max_wgt < 2 * d->min_wgt)
    return h->fail(SG_ERR_BAD_ARG, "collision: upper weight bound must be at least twice the lower weight bound");
  if (d->imp_abs && !d->roulette && !d->weight_windows)
    return h->fail(SG_ERR_BAD_ARG, "collision: implicit absorption needs Russian roulette or weight windows");
  if ((d->roulette && !(d->av_wgt > 0.0)) || (d->split && !(d->max_wgt > 0.0)))
    return h->fail(SG_ERR_BAD_ARG, "collision: weights must be positive");
  DColl<double> c64{};
  DColl<float> c32{};
  c64.imp_abs = c32.imp_abs = d->imp_abs != 0;
  c64.roulette = c32.roulette = d->roulette != 0;
  c64.split = c32.split = d->split != 0;
  c64.ww = c32.ww = d->weight_windows != 0;
  c64.max_split = c32.max_split = d->max_split;
  c64.min_wgt = d->min_wgt; c64.max_wgt = d->max_wgt; c64.av_wgt = d->av_wgt;
  c32.min_wgt = (float)d->min_wgt; c32.max_wgt = (float)d->max_wgt; c32.av_wgt = (float)d->av_wgt;
  if (d->weight_windows) {
    if (d->ww_n_axes < 1 || d->ww_n_axes > 3) return h->fail(SG_ERR_BAD_ARG, "weight windows: map needs 1-3 axes");
    if (!d->ww_lower || !d->ww_upper) return h->fail(SG_ERR_BAD_ARG, "weight windows: wLower and wUpper are required");
    if (!(d->ww_const_survival > 1.0)) return h->fail(SG_ERR_BAD_ARG, "weight windows: survival constant must be bigger than one");
    Admin W;
    long long N = 1;
    for (int a = 0; a < d->ww_n_axes; ++a) {
      const int rc = build_axis(h, d->ww_axes[a], W);
      if (rc) return rc;
      N *= axis_bins(d->ww_axes[a]);
    }
    for (int a = d->ww_n_axes; a < 3; ++a) { W.tab64.push_back(nullptr); W.tab32.push_back(nullptr); }
    std::vector<double> lo(d->ww_lower, d->ww_lower + N), up(d->ww_upper, d->ww_upper + N);
    for (long long i = 0; i < N; ++i) {
      if (lo[i] < 0.0 || up[i] < 0.0) return h->fail(SG_ERR_BAD_ARG, "weight windows: negative weights");
      if (lo[i] * d->ww_const_survival > up[i])
        return h->fail(SG_ERR_BAD_ARG, "weight windows: roulette survival weight above the upper weight");
    }
    std::vector<float> lof(lo.begin(), lo.end()), upf(up.begin(), up.end());
    CK(h->wwLo64.upload(lo, h->stream));
    CK(h->wwUp64.upload(up, h->stream));
    CK(h->wwLo32.upload(lof, h->stream));
    CK(h->wwUp32.upload(upf, h->stream));
    fill_axes<double>(c64.ww_map, d->ww_axes, d->ww_n_axes, W, 0);
    fill_axes<float>(c32.ww_map, d->ww_axes, d->ww_n_axes, W, 0);
    c64.ww_lower = h->wwLo64.p; c64.ww_upper = h->wwUp64.p; c64.ww_cs = d->ww_const_survival;
    c32.ww_lower = h->wwLo32.p; c32.ww_upper = h->wwUp32.p; c32.ww_cs = (float)d->ww_const_survival;
    h->wwAdmin = W;
  }
  const bool buf = d->split || d->weight_windows;
  if (buf) {
    const int depth = d->buffer_depth > 0 ? d->buffer_depth : 32;
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, h->cfg.device));
    const size_t n = (size_t)prop.multiProcessorCount * prop.maxThreadsPerMultiProcessor * depth;
    CK(h->bufR.alloc(3 * n));
    CK(h->bufE.alloc(n));
    CK(h->bufG.alloc(n));
    if (h->cfg.precision == SG_PREC_FP64) {
      CK(h->bufU64.alloc(3 * n)); CK(h->bufW64.alloc(n)); CK(h->bufT64.alloc(n));
      h->bufU32.free(); h->bufW32.free(); h->bufT32.free();
    } else {
      CK(h->bufU32.alloc(3 * n)); CK(h->bufW32.alloc(n)); CK(h->bufT32.alloc(n));
      h->bufU64.free(); h->bufW64.free(); h->bufT64.free();
    }
    c64.b_r = c32.b_r = h->bufR.p;
    c64.b_E = c32.b_E = h->bufE.p;
    c64.b_G = c32.b_G = h->bufG.p;
    c64.b_u = h->bufU64.p; c64.b_w = h->bufW64.p; c64.b_time = h->bufT64.p;
    c32.b_u = h->bufU32.p; c32.b_w = h->bufW32.p; c32.b_time = h->bufT32.p;
    c64.depth = c32.depth = depth;
  }
  std::vector<DColl<double>> v64(1, c64);
  std::vector<DColl<float>> v32(1, c32);
  CK(h->dColl64.upload(v64, h->stream));
  CK(h->dColl32.upload(v32, h->stream));
  h->hColl64 = c64;
  h->hColl32 = c32;
  h->collImp = true;
  h->collBuf = buf;
  return SG_OK;
}

int32_t sg_set_file_source(sg_handle h, const sg_bank* p, int32_t n) {
  if (!h || !p || n <= 0 || !p->r || !p->dir) return SG_ERR_BAD_ARG;
  if (!h->hasGeom) return h->fail(SG_ERR_STATE, "file source: upload the geometry first");
  if (h->hasCE && !p->E) return h->fail(SG_ERR_BAD_ARG, "file source: CE problems need E");
  if (!h->hasCE && !p->G) return h->fail(SG_ERR_BAD_ARG, "file source: MG problems need G");
  cudaStream_t s = h->stream;
  CK(h->fsR.upload(std::vector<double>(p->r, p->r + 3 * (size_t)n), s));
  CK(h->fsDir.upload(std::vector<double>(p->dir, p->dir + 3 * (size_t)n), s));
  std::vector<double> w(n, 1.0);
  if (p->wgt) w.assign(p->wgt, p->wgt + n);
  CK(h->fsWgt.upload(w, s));
  if (p->E) CK(h->fsE.upload(std::vector<double>(p->E, p->E + n), s));
  if (p->G) CK(h->fsG.upload(std::vector<int>(p->G, p->G + n), s));
  h->fileN = n;
  h->hasFileSource = true;
  return SG_OK;
}

int32_t sg_set_event_tuning(sg_handle h, const sg_event_tuning* t) {
  if (!h || !t) return SG_ERR_BAD_ARG;
  if (t->rounds_per_check < 1 || t->rounds_per_check > 64 || t->tail_min < 0 || t->tail_divisor < 1)
    return h->fail(SG_ERR_BAD_ARG, "event tuning: rounds 1-64, tail_min >= 0, tail_divisor >= 1");
  h->evTune = *t;
  return SG_OK;
}

int32_t sg_get_event_tuning(sg_handle h, sg_event_tuning* t) {
  if (!h || !t) return SG_ERR_BAD_ARG;
  *t = h->evTune;
  return SG_OK;
}

int32_t sg_get_history_records(sg_handle h, int32_t* collisions, uint64_t* rng_end, int32_t n) {
  if (!h || !h->cfg.record_histories) return h ? h->fail(SG_ERR_STATE, "record_histories is off") : SG_ERR_BAD_ARG;
  int m = std::min(n, h->lastN);
  if (m <= 0) return SG_OK;
  CK(cudaStreamSynchronize(h->stream));
  if (collisions) CK(cudaMemcpy(collisions, h->recColl.p, sizeof(int) * m, cudaMemcpyDeviceToHost));
  if (rng_end) CK(cudaMemcpy(rng_end, h->recRng.p, sizeof(unsigned long long) * m, cudaMemcpyDeviceToHost));
  return SG_OK;
}

int32_t sg_rng_draws(uint64_t* state, double* out, int32_t n) {
  if (!state || (!out && n > 0)) return SG_ERR_BAD_ARG;
  uint64_t s = *state;
  for (int i = 0; i < n; ++i) {
    s = (2806196910506780709ULL * s) & 0x7FFFFFFFFFFFFFFFULL;
    s = (s + 1ULL) & 0x7FFFFFFFFFFFFFFFULL;
    out[i] = (double)(int64_t)s * 0x1p-63;
  }
  *state = s;
  return SG_OK;
}

uint64_t sg_rng_skip(uint64_t state, int64_t k) { return lcg_skip(state, k); }

}  // extern "C"
