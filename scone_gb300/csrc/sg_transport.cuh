// sg_transport.cuh -- the history loop kernel: the `gen:` loop of SCONE's physics packages with
// transportOperatorST/DT, neutronMGstd collisions and tally reports fused into one persistent kernel.
//
// The same tracker serves multigroup (neutronMGstd, baseMgNeutronDatabase) and continuous-energy
// (neutronCEstd, aceNeutronDatabase) problems: template parameter CE selects the nuclear data and
// collision physics; geometry, transport operators and tallies are shared.
//
// Execution model: a persistent grid (a multiple of the SM count); each thread carries one particle
// history at a time and takes the next one as soon as its history ends, so a warp stays full until
// the bank runs dry.  Warps take histories from a global counter in chunks of 32 (one atomic per
// chunk).  Each loop iteration advances every live lane by one flight segment, so lanes diverge
// only inside collision processing.  Map-based tallies are accumulated in a shared-memory copy of
// the launch's score memory (SCONE's per-thread parallelBins, scoreMemory_class.f90:215-233,
// become per-block bins) and flushed with FP64 atomics at the end; the k-implicit estimator is
// accumulated in registers.
#pragma once
#include "sg_device.cuh"
#include "sg_ce.cuh"

namespace sg {

static constexpr unsigned FULL = 0xffffffffu;
enum { SEG_MORE = 0, SEG_END = 1, SEG_COLLIDE = 2 };

// fates (tallyCodes.f90:23-27)
enum { FATE_NONE = 5000, FATE_ABS = 5001, FATE_LEAK = 5002 };
// macro MTs (endfConstants.f90:116-130)
enum { MT_TOTAL = -1, MT_DISAP = -2, MT_ESCATTER = -3, MT_IESCATTER = -4, MT_FISSION = -6,
       MT_NUFISSION = -7, MT_ALLSCATTER = -20, MT_ABSORPTION = -21, MT_NONELASTIC = -22 };

__device__ __forceinline__ void raise_error(DCounters* ctr, int code, int hist) {
  if (atomicCAS(&ctr->err_code, 0, code) == 0) ctr->err_hist = hist;
}

// ---- bulk asynchronous copies global -> shared (cp.async.bulk, completion counted in bytes on an
// mbarrier); every wait is bounded
static constexpr int BULK_WAIT_LIMIT = 1 << 22;   // try_wait rounds before a chunk is given up

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}
// bounded wait for phase `parity` of the barrier; false if it did not complete in time
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  for (int it = 0; it < BULK_WAIT_LIMIT; ++it)
    if (mbar_test(bar, parity)) return true;
  return false;
}

// Start states of the histories of a warp's chunk.  History h starts from master + stride(h)
// (RNG_class.f90:251-316), i.e. T^(152917 h)(master) with T the LCG step s -> g s + 1 mod 2^63, an
// affine map; powers of one affine map compose in any order, so for h = b + off the state is
// T^(152917 off) applied to T^(152917 b)(master).  The table holds (A, C) of T^(152917 off) for
// off = 0..31 (A = g^(152917 off), C = T^(152917 off)(0)); a warp then makes one full skip per chunk
// of 32 histories and each history one multiply-add, bit for bit the states of lcg_skip.
struct RngJump {
  unsigned long long a[32], c[32];
};
// fills the table (the block's first warp; the caller synchronises the block afterwards)
__device__ __forceinline__ void rng_jump_table(RngJump& J) {
  if (threadIdx.x < 32) {
    const long long k = RNG_STRIDE * (long long)threadIdx.x;
    const unsigned long long c = lcg_skip(0ULL, k);
    J.c[threadIdx.x] = c;
    J.a[threadIdx.x] = (lcg_skip(1ULL, k) - c) & RNG_MASK;
  }
}
// T^(152917 off)(s), off in 0..31
__device__ __forceinline__ unsigned long long rng_jump(const RngJump& J, int off, unsigned long long s) {
  return (J.a[off] * s + J.c[off]) & RNG_MASK;
}

// LEAN: the history loop compiled for launches without rotated universes, cell maps, surface-current
// clerks, neutronMGimp / neutronCEimp or P1 scattering (TransportArgs::lean): their uniform branches
// are left out, which shortens the loop the instruction caches have to hold.
template <class R, int MAXL, int OP, bool CE, bool LEAN = false>
struct Tracker {
  const TransportArgs<R>& A;
  const Geom<R, MAXL, LEAN> geom;
  const DMG<R>& mg;
  const DCE<R>& ce;
  double* acc;
  R k_eff;

  // particle state
  Coords<R, MAXL> c;
  R cdist[MAXL];
  int csurf[MAXL];
  DistCache cache;
  Rng<R> rng;
  R w, w0;
  int G;
  int collN;
  int hist;
  int nsites;
  R time;            // particle time (MG speed 1: path length); FP32 in the mixed form
  int segs;
  R trackXS;         // tracking XS of the segment that ended in a real collision
  // CE state: energy, and the cross sections cached for it (invalidated when E changes)
  double E;
  CEPoint ep;
  R ceTot;           // total XS of material ceTotMat at E
  int ceTotMat;      // -1: none cached
  R ceMaj;           // majorant at E
  bool ceMajOK;
  R invSpeed;        // 1 / speed at E
  // k-implicit per-thread partial sums (keffImplicitClerk bins IMP_PROD, SCATTER_PROD, IMP_ABS,
  // ANA_LEAK), in R; the batch sums they are added to are FP64
  R kprod, kscat, kabs, kleak;
  unsigned long long nEv, nColl;
  int splitCount;    // particle%splitCount (neutronCEimp / neutronMGimp)
  int nbuf;          // split particles of this history waiting in the buffer
  bool htDT;         // hybrid tracking: the current transit uses delta tracking
  bool onSurf;       // the particle reached its position by a surface crossing or boundary hit

  __device__ __forceinline__ bool imp() const { return !LEAN && A.coll_imp; }
  __device__ __forceinline__ bool current() const { return !LEAN && A.has_current; }
  __device__ __forceinline__ bool cellmap() const { return !LEAN && A.has_cellmap; }

  __device__ __forceinline__ Tracker(const TransportArgs<R>& a, double* accp)
      : A(a), geom(a.geom), mg(a.mg), ce(a.ce), acc(accp) {
    k_eff = (R)(*a.k_eff);
    kprod = kscat = kabs = kleak = R(0);
    nEv = nColl = 0;
    htDT = false;
    onSurf = false;
    splitCount = 0;
    nbuf = 0;
  }

  __device__ __forceinline__ R xs(const R* t, int mat, int g) const { return t[(mat - 1) * mg.nG + (g - 1)]; }

  // neutronMacroXSs%get for the MG material (neutronXsPackages_class.f90:143-190)
  __device__ __forceinline__ R macro(int mat, int g, int MT) const {
    if (mat <= 0 || mat == SG_VOID_MAT) return R(0);
    int k = (mat - 1) * mg.nG + (g - 1);
    bool f = mg.fissile[mat - 1] != 0;
    switch (MT) {
      case MT_TOTAL: return mg.total[k];
      case MT_DISAP: return mg.capture[k];
      case MT_ESCATTER: return R(0);
      case MT_NONELASTIC: return mg.scatter[k] + (f ? mg.fission[k] : R(0)) + mg.capture[k];
      case MT_IESCATTER: return mg.scatter[k];
      case MT_ALLSCATTER: return R(0) + mg.scatter[k];
      case MT_FISSION: return f ? mg.fission[k] : R(0);
      case MT_NUFISSION: return f ? mg.nuFission[k] : R(0);
      case MT_ABSORPTION: return mg.capture[k] + (f ? mg.fission[k] : R(0));
      default: return R(0);
    }
  }
  // neutronMacroXSs%get for a CE material at the particle's energy
  __device__ __forceinline__ R macro_ce(int mat, int MT) const {
    if (mat <= 0 || mat == SG_VOID_MAT) return R(0);
    R x[4];
    if (!ce_mat_macro<R>(ce, mat, ep, x)) return R(0);
    switch (MT) {
      case MT_TOTAL: return x[0];
      case MT_DISAP: return x[3];
      case MT_ESCATTER: return x[1];
      case MT_NONELASTIC: return x[2] + R(0) + x[3];
      case MT_IESCATTER: return x[2];
      case MT_ALLSCATTER: return x[1] + x[2];
      case MT_ABSORPTION: return R(0) + x[3];
      default: return R(0);
    }
  }
  __device__ __forceinline__ R response(int code, int mat, int g) const {
    if (code == SG_RESP_FLUX) return R(1);
    if constexpr (CE) return macro_ce(mat, code);
    else return macro(mat, g, code);
  }

  // the cell the particle is in at its lowest level, as a 1-based index of the geometry's cells; 0
  // when that level is not a cellUniverse (coord%cell, coord_class.f90:419-425)
  __device__ __forceinline__ int lowest_cell() const {
    // the lowest level's universe and local cell, selected with compile-time indices only (a
    // runtime index would put the level arrays in local memory for the whole kernel)
    int u = c.uni[0], loc = c.local[0];
#pragma unroll
    for (int l = 1; l < MAXL; ++l)
      if (l < c.nest) { u = c.uni[l]; loc = c.local[l]; }
    const DUni& U = geom.g.unis[u];
    if (U.type != SG_UNI_CELL || loc > U.i[1]) return 0;   // local n+1: no cell of the universe
    return geom.g.uni_cells[U.i[0] + loc - 1] + 1;
  }

  // binaryFloorIdxClosed (genericProcedures.f90:132-166) on an unstructured grid of nb ascending
  // bounds, as grid%search (grid_class.f90:154-175): 1-based bin, 0 outside
  template <class T>
  __device__ __forceinline__ static int grid_floor(const T* a, int nb, T v) {
    if (!(v >= a[0] && v <= a[nb - 1])) return 0;
    int lo = 0, hi = nb - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (a[mid] <= v) lo = mid;
      else hi = mid;
    }
    return lo + 1;
  }

  // multiMap (multiMap_class.f90:153-173) of spaceMap / energyMap (lin, log and unstructured grids,
  // grid_class.f90:154-175) / group / material / cell axes; `cell` from lowest_cell()
  __device__ __forceinline__ int map_bin(const DClerk& K, const double r[3], int g, int mat, int cell) const {
    return map_bin_e(K, r, g, mat, cell, E);
  }
  __device__ __forceinline__ int map_bin_e(const DClerk& K, const double r[3], int g, int mat, int cell,
                                           double En) const {
    long long idx = 1;
    for (int a = 0; a < K.n_axes; ++a) {
      int b = 0;
      const int kind = K.ax_kind[a];
      if (kind <= SG_AXIS_Z || kind == SG_AXIS_ENERGY) {
        if (kind == SG_AXIS_ENERGY && !CE) return 0;     // energyMap of an MG particle
        const double v = (kind == SG_AXIS_ENERGY) ? En : at3(r, kind - 1);
        const int grid = K.ax_grid[a];
        if (grid == SG_GRID_UNSTRUCT) {
          if constexpr (sizeof(R) == 8) b = grid_floor<double>((const double*)K.ax_tab[a], K.ax_n[a] + 1, v);
          else b = grid_floor<float>((const float*)K.ax_tab[a], K.ax_n[a] + 1, (float)v);
        } else if (grid == SG_GRID_LOG) {
          if (!(v > 0.0)) return 0;
          if constexpr (sizeof(R) == 8) b = (int)floor(log(v / K.ax_min[a]) / K.ax_step[a]) + 1;
          else b = (int)floorf((__logf((float)v) - K.ax_minf[a]) * K.ax_inv_stepf[a]) + 1;   // ax_minf: log(min)
        } else {
          if constexpr (sizeof(R) == 8) b = (int)floor((v - K.ax_min[a]) / K.ax_step[a]) + 1;
          else b = (int)floorf(((float)v - K.ax_minf[a]) * K.ax_inv_stepf[a]) + 1;
        }
        if (b < 1 || b >= K.ax_n[a] + 1) b = 0;
      } else if (kind == SG_AXIS_GROUP) {
        b = (CE ? 0 : ((g >= 1 && g <= K.ax_n[a]) ? g : 0));
      } else if (kind == SG_AXIS_CELL) {
        b = ((const int*)K.ax_tab[a])[cell];
      } else {
        b = (mat >= 1 && mat <= K.ax_n[a]) ? mat : 0;
      }
      if (b == 0) return 0;
      idx += (long long)(b - 1) * K.multi[a];
    }
    return (int)idx;
  }

  __device__ __forceinline__ void score(long long at, double v) { atomicAdd(acc + at, v); }

  // tallyAdmin%reportInColl -> collisionClerk (collisionClerk_class.f90:192-242) and
  // keffImplicitClerk (keffImplicitClerk_class.f90:180-227)
  // invTrack = 1 / trackXS: the mixed form multiplies by it; the FP64 form divides, as SCONE does
  __device__ __forceinline__ void report_in_coll(bool virt, R trackXS, R invTrack) {
    const int cell = cellmap() ? lowest_cell() : 0;
    R fluxTrack;                                       // collision estimator with handleVirtual
    if constexpr (sizeof(R) == 4) fluxTrack = w * invTrack;
    else fluxTrack = w / trackXS;
    for (int k = 0; k < A.n_clerks; ++k) {
      const DClerk& K = A.clerks[k];
      if (K.type == SG_CLERK_COLLISION) {
        if (!K.handle_virtual && virt) continue;
        if (K.g_top > 0 && !(K.g_top <= G && G <= K.g_low)) continue;
        int bin = map_bin(K, c.r0, G, c.mat, cell);
        if (bin == 0) continue;
        R flux;
        if (K.handle_virtual) flux = fluxTrack;
        else if constexpr (CE) flux = w / ce_total(c.mat);
        else flux = w / xs(mg.total, c.mat, G);
        long long at = K.acc_off + (long long)K.width * (bin - 1);
        for (int i = 0; i < K.width; ++i) score(at + i, (double)(response(K.resp[i], c.mat, G) * flux));
      } else if (K.type == SG_CLERK_KEFF_IMPLICIT) {
        if constexpr (CE) continue;                    // rejected for CE problems at upload
        if (c.mat == SG_VOID_MAT) continue;
        const R flux = fluxTrack;
        // fission and nuFission are zero for non-fissile materials, so no fissile test is needed
        // (capture + 0 is capture exactly)
        const int xk = (c.mat - 1) * mg.nG + (G - 1);
        const R nuF = mg.nuFission[xk];
        const R absXS = mg.capture[xk] + mg.fission[xk];
        kprod += nuF * flux;
        kabs += absXS * flux;
      }
    }
  }
  // trackClerk%reportPath (trackClerk_class.f90:185-232): pre-path position and material
  __device__ __forceinline__ void report_path(const double rpre[3], int matPre, int cellPre, R L) {
    for (int k = 0; k < A.n_clerks; ++k) {
      const DClerk& K = A.clerks[k];
      if (K.type != SG_CLERK_TRACK) continue;
      if (K.g_top > 0 && !(K.g_top <= G && G <= K.g_low)) continue;
      int bin = map_bin(K, rpre, G, matPre, cellPre);
      if (bin == 0) continue;
      long long at = K.acc_off + (long long)K.width * (bin - 1);
      for (int i = 0; i < K.width; ++i) score(at + i, (double)(response(K.resp[i], matPre, G) * w * L));
    }
  }

  // Surface-current clerk (no SCONE counterpart): each tally plane crossed by the flight from rpre
  // to the current position scores the weight in [plane][bin of the pre-flight state][direction].
  // Side of a plane: coordinate < plane.  A leaking flight crosses every plane ahead of rpre.
  __device__ __forceinline__ void report_current(const double rpre[3], int matPre, int cellPre, const R u0[3],
                                                 bool leaked) {
    for (int k = 0; k < A.n_clerks; ++k) {
      const DClerk& K = A.clerks[k];
      if (K.type != SG_CLERK_SURFACE_CURRENT) continue;
      const double a0 = at3(rpre, K.cur_axis), a1 = at3(c.r0, K.cur_axis);
      const R u = at3(u0, K.cur_axis);
      int bin = -1;
      for (int q = 0; q < K.n_planes; ++q) {
        const double pl = K.planes[q];
        const bool crossed = leaked ? ((u > R(0)) ? (a0 < pl) : (u < R(0) && a0 >= pl)) : ((a0 < pl) != (a1 < pl));
        if (!crossed) continue;
        if (bin < 0) bin = map_bin(K, rpre, G, matPre, cellPre);
        if (bin == 0) break;
        const int dirBin = (leaked ? (u > R(0)) : (a1 > a0)) ? 1 : 0;
        score(K.acc_off + ((long long)q * K.nbins + (bin - 1)) * 2 + dirBin, (double)w);
      }
    }
  }

  // ---- CE cross sections at the particle's energy (cached until E changes)
  __device__ __forceinline__ void set_energy(double En) {
    E = En;
    ep = ce_point<R>(ce, En);
    ceTotMat = -1;
    ceMajOK = false;
    // particle_class.f90:481-503: speed = sqrt(2E/m) c; the mixed form keeps time in FP32 and takes
    // 1/speed from an FP32 reciprocal square root
    if constexpr (sizeof(R) == 8) invSpeed = 1.0 / (sqrt(2.0 * En / 939.56542194) * 2.99792458e10);
    else invSpeed = rsqrtf((float)(En * (2.0 / 939.56542194))) * (1.0f / 2.99792458e10f);
  }
  __device__ __forceinline__ R ce_total(int mat) {
    if (mat != ceTotMat) {
      if (!ce_mat_total<R>(ce, mat, ep, ceTot)) { raise_error(A.ctr, SG_ERR_NAN, hist); ceTot = R(1); }
      ceTotMat = mat;
    }
    return ceTot;
  }
  __device__ __forceinline__ R ce_major() {
    if (!ceMajOK) {
      if (!ce_majorant<R>(ce, ep, ceMaj)) { raise_error(A.ctr, SG_ERR_NAN, hist); ceMaj = R(1); }
      ceMajOK = true;
    }
    return ceMaj;
  }

  // collisionProcessor%collide with neutronCEstd (collisionProcessor_inter.f90:114-195,
  // neutronCEstd_class.f90:157-588) for non-fissile nuclides with CM-isotropic elastic scattering.
  // Returns true if the particle died.
  __device__ __forceinline__ bool collide_ce(R trackXS) {
    const int mat = c.mat;
    const R total = ce_total(mat);
    (void)rng.get();                                     // alpha test (alpha = 0), always drawn
    // sampleNuclide (ceNeutronMaterial_class.f90:338-455), TMS off
    R xi = total * rng.get();
    int nuc = -1;
    long long gi = -1;
    R f = R(0);
    const int k0 = ce.matPtr[mat - 1], k1 = ce.matPtr[mat];
    for (int k = k0; k < k1; ++k) {
      const int n = ce.matNuc[k];
      gi = ce_nuc_search<R>(ce, n, ep, f);
      const R tot = ce_interp<R>(ce.xs, gi, f, 0);
      xi = xi - tot * ce.matDens[k];
      if (xi < R(0) || k == k1 - 1) { nuc = n; break; }
    }
    // microXSs (aceNeutronNuclide_class.f90:419-453) and neutronMicroXSs%invert (:273-310)
    const R mt = ce_interp<R>(ce.xs, gi, f, 0), mel = ce_interp<R>(ce.xs, gi, f, 1);
    const R min_ = ce_interp<R>(ce.xs, gi, f, 2), mcap = ce_interp<R>(ce.xs, gi, f, 3);
    const R rr = rng.get();
    int C = 1;
    R x = mt * rr - mel;
    if (x > R(0)) C = C + 1;
    x = x - min_;
    if (x > R(0)) C = C + 1;
    x = x - mcap;
    if (x > R(0)) C = C + 1;
    report_in_coll(false, trackXS, R(1) / trackXS);
    if (imp() && A.coll->imp_abs) {                 // neutronCEimp implicit (:406-424)
      const R scat = mel + min_;
      w = w * scat / mt;
      C = (rng.get() < mel / scat) ? 1 : 2;
    }
    bool dead;
    if (C == 1) {                                        // elastic (:340-384)
      const R Anuc = ce.A[nuc], kT = ce.kT[nuc];
      const bool isFixed = ((R)E > kT * ce.threshE) && (Anuc > ce.threshA);
      double Eout;
      if (isFixed) {                                     // scatterFromFixed + asymptoticScatter
        R mu = R(2) * rng.get() - R(1);
        R sp, cp;
        sincos_phi<R>(rng.get(), sp, cp);
        R muL;
        if constexpr (sizeof(R) == 8) {
          const double Ad = (double)Anuc, mud = (double)mu;
          const double inv_Ap1 = 1.0 / (Ad + 1.0);
          Eout = (1.0 + Ad * Ad + 2 * Ad * mud) * E * inv_Ap1 * inv_Ap1;
          muL = (R)((Ad * mud + 1) * sqrt(E / Eout) * inv_Ap1);
        } else {                                         // the same kinematics with an FP32 ratio
          const float inv_Ap1 = 1.0f / (Anuc + 1.0f);
          const float ratio = (1.0f + Anuc * Anuc + 2.0f * Anuc * mu) * inv_Ap1 * inv_Ap1;   // Eout / E
          Eout = E * (double)ratio;
          muL = (Anuc * mu + 1.0f) * rsqrtf(ratio) * inv_Ap1;
        }
        if (muL > R(1)) muL = R(1);
        rotate_vector<R>(c.u[0], c.u[1], c.u[2], muL, sp, cp);
      } else {                                           // scatterFromMoving (:495-585)
        const R d0 = c.u[0], d1 = c.u[1], d2 = c.u[2];
        R sE;
        if constexpr (sizeof(R) == 8) sE = sqrt(E);
        else sE = sqrtf((float)E);
        R Vn[3] = {d0 * sE, d1 * sE, d2 * sE};
        R Vt[3], Vcm[3];
        bool bad = false;
        target_velocity<R>((R)E, d0, d1, d2, Anuc, kT, rng, Vt, &bad);
        if (bad) raise_error(A.ctr, SG_ERR_TIMEOUT, hist);
#pragma unroll
        for (int i = 0; i < 3; ++i) Vcm[i] = (Vn[i] + Vt[i] * Anuc) / (Anuc + R(1));
#pragma unroll
        for (int i = 0; i < 3; ++i) Vn[i] = Vn[i] - Vcm[i];
        R Un = norm3<R>(Vn[0], Vn[1], Vn[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) Vn[i] = Vn[i] / Un;
        const R mu = R(2) * rng.get() - R(1);
        R sp, cp;
        sincos_phi<R>(rng.get(), sp, cp);
        rotate_vector<R>(Vn[0], Vn[1], Vn[2], mu, sp, cp);
#pragma unroll
        for (int i = 0; i < 3; ++i) Vn[i] = Vn[i] * Un + Vcm[i];
        Un = norm3<R>(Vn[0], Vn[1], Vn[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) c.u[i] = Vn[i] / Un;
        Eout = (double)(Un * Un);
      }
      set_energy(Eout);
      dead = false;
    } else if (C == 2) {                                 // no inelastic channels in the data
      raise_error(A.ctr, SG_ERR_BAD_ARG, hist);
      dead = true;
    } else {
      dead = true;                                       // capture / fission
    }
    if (imp()) dead = imp_cutoffs(dead);
    else if (E < ce.minE) dead = true;                   // cutoffs (:434-444)
    collN += 1;
    nColl += 1;
    return dead;
  }

  // ---- neutronCEimp / neutronMGimp cutoffs (neutronCEimp_class.f90:633-734,
  // neutronMGimp_class.f90:319-407).  Returns whether the particle is dead afterwards.
  __device__ __forceinline__ bool imp_cutoffs(bool dead) {
    if (dead) return true;
    const DColl<R>& K = *A.coll;
    if constexpr (CE) { if (E < ce.minE) return true; }
    if (K.ww) {                                          // weightWindowsField%atP (:148-171)
      const int bin = map_bin_e(K.ww_map, c.r0, G, c.mat, lowest_cell(), E);
      R lo = R(0), up = R(0), av = R(0);
      if (bin > 0) { lo = K.ww_lower[bin - 1]; up = K.ww_upper[bin - 1]; av = lo * K.ww_cs; }
      if (w > up && up != R(0) && splitCount < K.max_split) split(up);
      else if (w < lo) return roulette(av);
      return false;
    }
    if constexpr (CE) {
      if (K.split && w > K.max_wgt) split(K.max_wgt);
      else if (K.roulette && w < K.min_wgt) return roulette(K.av_wgt);
    }
    return false;
  }
  // russianRoulette (:683-694)
  __device__ __forceinline__ bool roulette(R av) {
    if (rng.get() < (R(1) - w / av)) return true;
    w = av;
    return false;
  }
  // split (:699-734): mult - 1 copies of weight w / mult into the history's buffer
  __device__ __forceinline__ void split(R maxW) {
    const DColl<R>& K = *A.coll;
    int mult = (int)ceil((double)(w / maxW));
    if (mult + splitCount > K.max_split) mult = K.max_split - splitCount + 1;
    const R ws = w / (R)mult;
    const long long lane = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = 1; i < mult; ++i) {
      if (nbuf >= K.depth) { raise_error(A.ctr, SG_ERR_BANK_OVERFLOW, hist); break; }
      const long long e = lane * K.depth + nbuf;
#pragma unroll
      for (int k = 0; k < 3; ++k) { K.b_r[3 * e + k] = c.r0[k]; K.b_u[3 * e + k] = c.u[k]; }
      K.b_w[e] = ws;
      K.b_E[e] = CE ? E : 0.0;
      K.b_G[e] = G;
      K.b_time[e] = time;
      nbuf += 1;
    }
    splitCount += mult;
    w = w / (R)mult;
  }
  // buffer%release and the restart of the gen loop's bufferLoop (fixedSourcePhysicsPackage_class.f90
  // :209-216,235-239): the last split particle, placed, with its weight as the pre-history weight;
  // the RNG stream continues
  __device__ __forceinline__ void release() {
    const DColl<R>& K = *A.coll;
    nbuf -= 1;
    const long long e = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * K.depth + nbuf;
#pragma unroll
    for (int k = 0; k < 3; ++k) { c.r0[k] = K.b_r[3 * e + k]; c.u[k] = K.b_u[3 * e + k]; }
    w = K.b_w[e];
    w0 = w;
    G = K.b_G[e];
    if constexpr (CE) set_energy(K.b_E[e]);
    time = K.b_time[e];
    splitCount = 0;
    cache.lvl = 0;
    onSurf = false;
    if (!geom.place(c, false)) raise_error(A.ctr, SG_ERR_UNDEF_MAT, hist);
    select_ht();
  }

  __device__ __forceinline__ void write_site(const R dir[3], int gout, R wgt) {
    int region = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) & A.sites.region_mask;
    int slot = atomicAdd(&A.sites.cursor[region], 1);
    if (slot >= A.sites.region_cap) { raise_error(A.ctr, SG_ERR_BANK_OVERFLOW, hist); return; }
    long long i = (long long)region * A.sites.region_cap + slot;
    A.sites.r[3 * i + 0] = c.r0[0];
    A.sites.r[3 * i + 1] = c.r0[1];
    A.sites.r[3 * i + 2] = c.r0[2];
    A.sites.dir[3 * i + 0] = (double)dir[0];
    A.sites.dir[3 * i + 1] = (double)dir[1];
    A.sites.dir[3 * i + 2] = (double)dir[2];
    A.sites.wgt[i] = (double)wgt;
    A.sites.G[i] = gout;
    A.sites.brood[i] = hist;
    A.sites.seq[i] = nsites;
    A.sites.time[i] = (double)time;
    nsites += 1;
  }

  // A CDF walk (multiScatterMG%sampleGout, fissionMG%sampleOut) that ran past the last group.  In
  // FP64 this is SCONE's fatal error (multiScatterMG_class.f90:250-251).  In the mixed form the FP32
  // table total can exceed the FP32 running sum of its entries by a few ulps, so a number xi within
  // a few ulps of 1 can outlast the walk: it belongs to the last group with a nonzero entry.
  __device__ __forceinline__ int walk_failed(const R* entries, int stride) {
    if constexpr (sizeof(R) == 8) {
      raise_error(A.ctr, SG_ERR_NAN, hist);
      return mg.nG;
    } else {
      int g = mg.nG;
      while (g > 1 && !(entries[(g - 1) * stride] > R(0))) --g;
      return g;
    }
  }

  // collisionProcessor%collide with neutronMGstd (collisionProcessor_inter.f90:114-195,
  // neutronMGstd_class.f90:85-297).  Returns true if the particle died.
  __device__ __forceinline__ bool collide(R trackXS) {
    if constexpr (CE) return collide_ce(trackXS);
    const int mat = c.mat;
    (void)rng.get();                                     // alpha test, drawn even for alpha = 0
    const int k = (mat - 1) * mg.nG + (G - 1);
    const bool fiss = mg.fissile[mat - 1] != 0;
    const R total = mg.total[k], inel = mg.scatter[k], capture = mg.capture[k];
    const R rr = rng.get();
    int C = 1;                                           // neutronMacroXSs%invert (:211-250)
    R x = total * rr - R(0);
    if (x > R(0)) C = C + 1;
    x = x - inel;
    if (x > R(0)) C = C + 1;
    x = x - capture;
    if (x > R(0)) C = C + 1;
    report_in_coll(false, trackXS, R(1) / trackXS);
    const R preCollW = w;
    if (fiss) {                                          // implicit (:134-201)
      R rand1 = rng.get();
      R nuF = mg.nuFission[k];
      int n = (int)(fabs((w * nuF) / (w0 * total * k_eff)) + rand1);
      if (n >= 1) {
        R sw = sgn(w0, w);
        for (int s = 0; s < n; ++s) {                    // fissionMG%sampleOut (:183-206)
          R mu = R(2) * rng.get() - R(1);
          R sp, cp;
          sincos_phi<R>(rng.get(), sp, cp);
          R rem = rng.get();
          int go = 1;
          for (go = 1; go <= mg.nG; ++go) {
            rem = rem - mg.chi[(mat - 1) * mg.nG + (go - 1)];
            if (rem < R(0)) break;
          }
          if (go > mg.nG) go = walk_failed(mg.chi + (mat - 1) * mg.nG, 1);
          R d[3] = {c.u[0], c.u[1], c.u[2]};
          rotate_vector<R>(d[0], d[1], d[2], mu, sp, cp);
          write_site(d, go, sw);
        }
      }
    }
    bool dead;
    int MT;
    if (C <= 2) {                                        // inelastic (:221-252), multiScatterMG%sampleOut
      R rem = rng.get() * inel;
      const R* row = mg.P0 + (long long)k * mg.nG;
      int go;
      for (go = 1; go <= mg.nG; ++go) {
        rem = rem - row[go - 1];
        if (rem < R(0)) break;
      }
      if (go > mg.nG) go = walk_failed(row, 1);
      R mu;                                              // multiScatterP1MG%sampleOut (:69-85)
      if (!LEAN && mg.P1n) mu = sample_legendre_p1<R>(mg.P1n[(long long)k * mg.nG + (go - 1)], rng);
      else mu = R(2) * rng.get() - R(1);
      R sp, cp;
      sincos_phi<R>(rng.get(), sp, cp);
      R w_mul = mg.prod[(long long)k * mg.nG + (go - 1)];
      G = go;
      w = w * w_mul;
      rotate_vector<R>(c.u[0], c.u[1], c.u[2], mu, sp, cp);
      MT = MT_IESCATTER;
      dead = false;
    } else {                                             // capture / fission
      MT = (C == 3) ? MT_DISAP : MT_FISSION;
      dead = true;
    }
    if (imp()) dead = imp_cutoffs(dead);            // neutronMGimp cutoffs (:319-351)
    collN += 1;
    nColl += 1;
    if (A.keff_clerk >= 0 && MT == MT_IESCATTER) {       // keffImplicit reportOutColl (:241-268)
      R sc = fmax(w - preCollW, R(0));
      if (sc > R(0)) kscat += sc;
    }
    return dead;
  }

  __device__ __forceinline__ void start(int h) { start_from(h, lcg_skip(A.master, RNG_STRIDE * (long long)h)); }
  // history h of the bank, its RNG already at master + stride(h)
  __device__ __forceinline__ void start_from(int h, unsigned long long s0) {
    hist = h;
    const int i = h - 1;
    c.r0[0] = A.in.r[3 * i + 0];
    c.r0[1] = A.in.r[3 * i + 1];
    c.r0[2] = A.in.r[3 * i + 2];
    c.u[0] = (R)A.in.dir[3 * i + 0];
    c.u[1] = (R)A.in.dir[3 * i + 1];
    c.u[2] = (R)A.in.dir[3 * i + 2];
    w = (R)A.in.wgt[i];
    w0 = w;
    G = CE ? 0 : A.in.G[i];
    if constexpr (CE) set_energy(A.in.E[i]);
    time = (R)A.in.time[i];
    rng.s = s0;
    collN = 0;
    nsites = 0;
    segs = 0;
    splitCount = 0;
    nbuf = 0;
    cache.lvl = 0;
    onSurf = false;
    if (!geom.place(c, false)) raise_error(A.ctr, SG_ERR_UNDEF_MAT, h);
    select_ht();
  }

  __device__ __forceinline__ void finish() {
    if (A.hist_nsites) A.hist_nsites[hist - 1] = nsites;
    if (A.rec_coll) A.rec_coll[hist - 1] = collN;
    if (A.rec_rng) A.rec_rng[hist - 1] = rng.s;
  }

  // One flight segment of surfaceTracking / deltaTracking.  Returns SEG_MORE (keep tracking),
  // SEG_END (the history ended: leak or error) or SEG_COLLIDE (a real collision; trackXS holds the
  // tracking cross section the collision estimators use).
  __device__ __forceinline__ int segment() {
    if (++segs > A.max_segments) { raise_error(A.ctr, SG_ERR_LOST, hist); return SEG_END; }
    if constexpr (OP == OP_DT) return seg_dt();
    else if constexpr (OP == OP_ST) return seg_st();
    else return htDT ? seg_dt() : seg_st();
  }

  // transportOperatorHT%tracking_selection (transportOperatorHT_class.f90:49-81), made at the start
  // of every transit: delta tracking when Sigma_t / Sigma_majorant > 1 - cutoff (surface tracking
  // in void).  No random number is drawn.
  __device__ __forceinline__ void select_ht() {
    if constexpr (OP == OP_HT) {
      R sigT, majInv;
      if constexpr (CE) majInv = R(1) / fmax(ce_major(), ce.collisionXS);
      else majInv = mg.majInv[G - 1];
      if (c.mat == SG_VOID_MAT) sigT = R(0);
      else if constexpr (CE) sigT = ce_total(c.mat);
      else sigT = xs(mg.total, c.mat, G);
      htDT = sigT * majInv > R(1) - A.ht_cutoff;
    }
  }

  __device__ __forceinline__ int seg_st() {
    const R INF_R = R(D_INF);
    int mat = c.mat;
    {
      // surfaceTracking (transportOperatorST_class.f90:48-166)
      const bool isVoid = (mat == SG_VOID_MAT);
      R sigTot, sigmaTrack;
      if constexpr (CE) {
        sigTot = isVoid ? R(0) : ce_total(mat);
        sigmaTrack = isVoid ? fmax(R(0), ce.collisionXS) : fmax(sigTot, ce.collisionXS);
      } else {
        sigTot = isVoid ? R(0) : xs(mg.total, mat, G);
        sigmaTrack = isVoid ? mg.collisionXS : fmax(sigTot, mg.collisionXS);
      }
      R dist, invSig, sigT;
      if (sigmaTrack < Tol<R>::st_void()) { dist = INF_R; invSig = INF_R; sigT = R(0); }
      else { invSig = R(1) / sigmaTrack; dist = -dlog<R>(rng.get()) * invSig; sigT = sigTot; }
      const double rpre[3] = {c.r0[0], c.r0[1], c.r0[2]};
      const R u0[3] = {c.u[0], c.u[1], c.u[2]};
      const int matPre = mat;
      const int cellPre = cellmap() ? lowest_cell() : 0;
      const int ev = geom.move(c, dist, cdist, csurf, cache, A.use_cache != 0, onSurf);
      onSurf = (ev != 1);                                // a crossing or boundary hit leaves it on a surface
      if constexpr (CE) time = time + dist * invSpeed;
      else time = time + dist;
      nEv += 1;
      report_path(rpre, matPre, cellPre, dist);
      mat = c.mat;
      if (current()) report_current(rpre, matPre, cellPre, u0, mat == 0);
      if (mat == 0) { leak(); return SEG_END; }
      if (mat == SG_UNDEF_MAT || mat == SG_OVERLAP_MAT) {
        raise_error(A.ctr, mat == SG_UNDEF_MAT ? SG_ERR_UNDEF_MAT : SG_ERR_OVERLAP, hist);
        return SEG_END;
      }
      if (ev == 1) {
        if (rng.get() < sigT * invSig) {
          cache.lvl = 0;
          trackXS = sigmaTrack;
          return SEG_COLLIDE;
        }
        report_in_coll(true, sigmaTrack, invSig);
      }
      return SEG_MORE;
    }
  }

  __device__ __forceinline__ int seg_dt() {
    int mat = c.mat;
    {
      // deltaTracking (transportOperatorDT_class.f90:47-131)
      R maj, majInv;
      if constexpr (CE) { maj = fmax(ce_major(), ce.collisionXS); majInv = R(1) / maj; }
      else { maj = fmax(mg.majorant[G - 1], mg.collisionXS); majInv = mg.majInv[G - 1]; }
      const R dist = -dlog<R>(rng.get()) * majInv;
      double rpre[3];
      R u0[3];
      if (current()) {
#pragma unroll
        for (int i = 0; i < 3; ++i) { rpre[i] = c.r0[i]; u0[i] = c.u[i]; }
      }
      const int matPre = mat;
      const int cellPre = (cellmap() && current()) ? lowest_cell() : 0;
      onSurf = false;
      if (!geom.teleport(c, dist)) { raise_error(A.ctr, SG_ERR_UNDEF_MAT, hist); return SEG_END; }
      if constexpr (CE) time = time + dist * invSpeed;
      else time = time + dist;
      nEv += 1;
      mat = c.mat;
      if (current()) report_current(rpre, matPre, cellPre, u0, mat == 0);
      if (mat == 0) { leak(); return SEG_END; }
      if (mat == SG_VOID_MAT) { report_in_coll(true, maj, majInv); return SEG_MORE; }
      if (mat == SG_UNDEF_MAT || mat == SG_OVERLAP_MAT) {
        raise_error(A.ctr, mat == SG_UNDEF_MAT ? SG_ERR_UNDEF_MAT : SG_ERR_OVERLAP, hist);
        return SEG_END;
      }
      R sigT;
      if constexpr (CE) sigT = ce_total(mat);
      else sigT = xs(mg.total, mat, G);
      if (rng.get() < sigT * majInv) { trackXS = maj; return SEG_COLLIDE; }
      report_in_coll(true, maj, majInv);
      return SEG_MORE;
    }
  }

  // One segment and, when it ends in a real collision, the collision.  True when the history ended.
  __device__ __forceinline__ bool step() {
    const int e = segment();
    if (e == SEG_COLLIDE) {
      const bool dead = collide(trackXS);
      if (!dead) select_ht();
      return dead;
    }
    return e == SEG_END;
  }

  // ---- particle state held in device memory between the event kernels (component-major SoA)
  __device__ __forceinline__ void store(const DPart<R>& P, int i) const {
    const long long cap = P.cap;
#pragma unroll
    for (int k = 0; k < 3; ++k) { P.r0[k * cap + i] = c.r0[k]; P.u[k * cap + i] = c.u[k]; }
#pragma unroll
    for (int l = 0; l < MAXL - 1; ++l)
#pragma unroll
      for (int k = 0; k < 3; ++k) P.rl[(l * 3 + k) * cap + i] = c.rl[l][k];
#pragma unroll
    for (int l = 0; l < MAXL; ++l) {
      P.geo[(3 * l + 0) * cap + i] = c.uni[l];
      P.geo[(3 * l + 1) * cap + i] = c.base[l];
      P.geo[(3 * l + 2) * cap + i] = c.local[l];
    }
    P.geo[(3 * MAXL + 0) * cap + i] = c.nest;
    P.geo[(3 * MAXL + 1) * cap + i] = c.mat;
    P.geo[(3 * MAXL + 2) * cap + i] = c.uid;
    P.rng[i] = rng.s;
    P.w[i] = w;
    P.w0[i] = w0;
    P.time[i] = time;
    P.trackXS[i] = trackXS;
    P.ints[0 * cap + i] = G;
    P.ints[1 * cap + i] = collN;
    P.ints[2 * cap + i] = hist;
    P.ints[3 * cap + i] = nsites;
    P.ints[4 * cap + i] = segs;
    if constexpr (CE) P.E[i] = E;
  }
  __device__ __forceinline__ void load(const DPart<R>& P, int i) {
    const long long cap = P.cap;
#pragma unroll
    for (int k = 0; k < 3; ++k) { c.r0[k] = P.r0[k * cap + i]; c.u[k] = P.u[k * cap + i]; }
#pragma unroll
    for (int l = 0; l < MAXL - 1; ++l)
#pragma unroll
      for (int k = 0; k < 3; ++k) c.rl[l][k] = P.rl[(l * 3 + k) * cap + i];
#pragma unroll
    for (int l = 0; l < MAXL; ++l) {
      c.uni[l] = P.geo[(3 * l + 0) * cap + i];
      c.base[l] = P.geo[(3 * l + 1) * cap + i];
      c.local[l] = P.geo[(3 * l + 2) * cap + i];
    }
    c.nest = P.geo[(3 * MAXL + 0) * cap + i];
    c.mat = P.geo[(3 * MAXL + 1) * cap + i];
    c.uid = P.geo[(3 * MAXL + 2) * cap + i];
    rng.s = P.rng[i];
    w = P.w[i];
    w0 = P.w0[i];
    time = P.time[i];
    trackXS = P.trackXS[i];
    G = P.ints[0 * cap + i];
    collN = P.ints[1 * cap + i];
    hist = P.ints[2 * cap + i];
    nsites = P.ints[3 * cap + i];
    segs = P.ints[4 * cap + i];
    cache.lvl = 0;
    onSurf = false;                                    // stored particles sit at a collision point or a start
    if constexpr (CE) set_energy(P.E[i]);
    select_ht();
  }

  // reportHist for a leaked particle (keffImplicitClerk ANA_LEAK, :276-290)
  __device__ __forceinline__ void leak() { if (A.keff_clerk >= 0) kleak += w; }
  __device__ __forceinline__ void absorbed() {}
};


// k-implicit partial sums and event counters of a warp, reduced and added to global memory
template <class R, int MAXL, int OP, bool CE, bool LEAN>
__device__ __forceinline__ void flush_counters(Tracker<R, MAXL, OP, CE, LEAN>& T, const TransportArgs<R>& A, int lane) {
  if (A.keff_clerk >= 0) {
    double v[4] = {(double)T.kprod, (double)T.kscat, (double)T.kabs, (double)T.kleak};
#pragma unroll
    for (int q = 0; q < 4; ++q)
      for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(FULL, v[q], o);
    if (lane == 0) {
      long long off = A.clerks[A.keff_clerk].acc_off;
#pragma unroll
      for (int q = 0; q < 4; ++q) if (v[q] != 0.0) atomicAdd(A.acc + off + q, v[q]);
    }
  }
  unsigned long long ev = T.nEv, co = T.nColl;
  for (int o = 16; o > 0; o >>= 1) {
    ev += __shfl_down_sync(FULL, ev, o);
    co += __shfl_down_sync(FULL, co, o);
  }
  if (lane == 0) {
    atomicAdd(&A.ctr->events, ev);
    atomicAdd(&A.ctr->collisions, co);
  }
}

// warp-aggregated append to a queue counter: one atomic per warp for the lanes that are active
__device__ __forceinline__ int warp_append(int* counter) {
  const unsigned m = __activemask();
  const int leader = __ffs(m) - 1;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(m, base, leader);
  return base + __popc(m & ((1u << lane) - 1u));
}

// Blocks per SM the history loop is compiled for (0: ptxas' choice).  The multigroup delta-tracking
// kernels are held to 72 registers (7 blocks of 128 threads) in the mixed form and 80 (6 blocks) in
// the FP64 form: left alone, ptxas picks 64 registers and spills more, which measured slower on the
// lattice.
template <class R, bool CE, int OP>
constexpr int history_min_blocks() { return (CE || OP != OP_DT) ? 0 : (sizeof(R) == 4 ? 7 : 6); }
// The batched kernel in the mixed form with delta tracking is held to 64 registers (8 blocks): on
// the uneven batch +2.3 % over 72 registers, where the same pin on the single-problem kernels
// measured -2 % on the lattice and -4 % on the CE slab (same GB300).
template <class R, int OP>
constexpr int batch_min_blocks() { return (OP == OP_DT && sizeof(R) == 4) ? 8 : history_min_blocks<R, false, OP>(); }

template <class R, int MAXL, int OP, bool CE, bool LEAN = false>
__global__ void __launch_bounds__(128, (history_min_blocks<R, CE, OP>())) k_transport(const __grid_constant__ TransportArgs<R> A) {
  extern __shared__ double s_acc[];
  __shared__ RngJump s_jump;
  const bool smem = A.use_smem != 0;
  if (smem)
    for (int i = threadIdx.x; i < A.acc_n; i += blockDim.x) s_acc[i] = 0.0;
  rng_jump_table(s_jump);
  __syncthreads();
  Tracker<R, MAXL, OP, CE, LEAN> T(A, smem ? s_acc : A.acc);
  const int lane = threadIdx.x & 31;
  bool alive = false, done = false;
  int q_next = 0, q_end = 0;   // warp-uniform range of histories taken from the global counter
  int q_base = 0;              // first history (0-based) of the warp's chunk
  unsigned long long s_base = 0;   // master + stride(q_base + 1), warp-uniform

  while (true) {
    unsigned need = __ballot_sync(FULL, !alive && !done);
    while (need) {
      if (q_next >= q_end) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&A.ctr->work, 32);
        base = __shfl_sync(FULL, base, 0);
        if (base >= A.n) {
          if (!alive) done = true;
          break;
        }
        q_next = base;
        q_end = min(base + 32, A.n);
        q_base = base;
        s_base = lcg_skip(A.master, RNG_STRIDE * (long long)(base + 1));
      }
      const int avail = q_end - q_next;
      const int rank = __popc(need & ((1u << lane) - 1u));
      const bool mine = ((need >> lane) & 1u) && rank < avail;
      if (mine) {
        const int h0 = q_next + rank;
        T.start_from(h0 + 1, rng_jump(s_jump, h0 - q_base, s_base));
        alive = true;
      }
      q_next += min(__popc(need), avail);
      need &= ~__ballot_sync(FULL, mine);
    }
    if (__all_sync(FULL, !alive)) break;
    // One flight per live lane, then the warp meets again (the vote) before the lanes whose flight
    // ended in a real collision process it: the collision code then starts with every colliding lane
    // together (7 % faster on the 17x17 lattice than flight and collision in one branch).  Making
    // lanes wait until half the warp has a collision was no faster with delta tracking and 8 %
    // slower with surface tracking.
    bool ended = false, coll = false;
    if (alive) {
      const int e = T.segment();
      coll = (e == SEG_COLLIDE);
      ended = (e == SEG_END);
    }
    if (__any_sync(FULL, coll) && coll) {
      ended = T.collide(T.trackXS);
      if (!ended) T.select_ht();
    }
    if (ended) {
      if (!LEAN && T.nbuf > 0) T.release();             // the history's split particles, LIFO
      else { T.finish(); alive = false; }
    }
  }

  flush_counters(T, A, lane);
  if (smem) {
    __syncthreads();
    for (int i = threadIdx.x; i < A.acc_n; i += blockDim.x) {
      double v = s_acc[i];
      if (v != 0.0) atomicAdd(A.acc + i, v);
    }
  }
}


// ================================================================== event form
// Histories are started once (k_ev_start), then alternate between the transit kernel (flight
// segments until a real collision, surface crossings and path/virtual-collision tallies included)
// and the collision kernel (neutronMGstd physics), each over a compacted queue of particle slots.
// Every warp in a launch therefore runs one kind of event.  The last few percent of histories are
// finished by the tail kernel (the history loop over the remaining queue).  Per-history RNG streams
// make the results independent of this scheduling.

template <class R, int MAXL, int OP, bool CE>
__global__ void __launch_bounds__(128) k_ev_start(const __grid_constant__ TransportArgs<R> A) {
  Tracker<R, MAXL, OP, CE> T(A, A.acc);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
    T.start(i + 1);
    T.store(A.part, i);
    A.q.out[i] = i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *A.q.n_out = A.n;
}

// TAIL = false: stop at a real collision and queue the particle for k_ev_collide.
// TAIL = true : run each particle to the end of its history (collisions included).
template <class R, int MAXL, int OP, bool CE, bool TAIL>
__global__ void __launch_bounds__(128) k_ev_transit(const __grid_constant__ TransportArgs<R> A) {
  Tracker<R, MAXL, OP, CE> T(A, A.acc);
  const int lane = threadIdx.x & 31;
  const int nIn = *A.q.n_in;
  bool alive = false, done = false;
  int slot = -1;
  int q_next = 0, q_end = 0;
  while (true) {
    unsigned need = __ballot_sync(FULL, !alive && !done);
    while (need) {
      if (q_next >= q_end) {
        int base = 0;
        if (lane == 0) base = atomicAdd(A.q.work, 32);
        base = __shfl_sync(FULL, base, 0);
        if (base >= nIn) {
          if (!alive) done = true;
          break;
        }
        q_next = base;
        q_end = min(base + 32, nIn);
      }
      const int avail = q_end - q_next;
      const int rank = __popc(need & ((1u << lane) - 1u));
      const bool mine = ((need >> lane) & 1u) && rank < avail;
      if (mine) {
        slot = A.q.in[q_next + rank];
        T.load(A.part, slot);
        alive = true;
      }
      q_next += min(__popc(need), avail);
      need &= ~__ballot_sync(FULL, mine);
    }
    if (__all_sync(FULL, !alive)) break;
    if (alive) {
      if constexpr (TAIL) {
        if (T.step()) { T.finish(); alive = false; }
      } else {
        const int e = T.segment();
        if (e == SEG_END) { T.finish(); alive = false; }
        else if (e == SEG_COLLIDE) {
          T.store(A.part, slot);
          A.q.out[warp_append(A.q.n_out)] = slot;
          alive = false;
        }
      }
    }
  }
  flush_counters(T, A, lane);
}

// Block-level stream compaction of one round's flags: a ballot per warp, the warps' counts scanned in
// shared memory, one atomic per block for the block's base in the queue; returns this thread's
// position (meaningful where flag is set).  Every thread of the block calls it.
__device__ __forceinline__ int block_append(bool flag, int* counter, int* s_cnt) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned m = __ballot_sync(FULL, flag);
  if (lane == 0) s_cnt[warp] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < nw; ++w) { const int c = s_cnt[w]; s_cnt[w] = tot; tot += c; }
    s_cnt[nw] = tot ? atomicAdd(counter, tot) : 0;
  }
  __syncthreads();
  const int pos = s_cnt[nw] + s_cnt[warp] + __popc(m & ((1u << lane) - 1u));
  __syncthreads();                                      // the counts are rewritten next round
  return pos;
}

template <class R, int MAXL, int OP, bool CE>
__global__ void __launch_bounds__(128) k_ev_collide(const __grid_constant__ TransportArgs<R> A) {
  __shared__ int s_cnt[4 + 1];
  Tracker<R, MAXL, OP, CE> T(A, A.acc);
  const int nIn = *A.q.n_in;
  const int stride = gridDim.x * blockDim.x;
  const int first = blockIdx.x * blockDim.x + threadIdx.x;
  const int rounds = (nIn + stride - 1) / stride;      // uniform trip count keeps warps convergent
  for (int r = 0; r < rounds; ++r) {
    const int idx = first + r * stride;
    int slot = -1;
    bool survivor = false;
    if (idx < nIn) {
      slot = A.q.in[idx];
      T.load(A.part, slot);
      if (T.collide(T.trackXS)) T.finish();
      else {
        T.store(A.part, slot);
        survivor = true;
      }
    }
    // the survivors go back to the transit queue, compacted per block (contiguous writes)
    const int pos = block_append(survivor, A.q.n_out, s_cnt);
    if (survivor) A.q.out[pos] = slot;
  }
  flush_counters(T, A, threadIdx.x & 31);
}

}  // namespace sg
