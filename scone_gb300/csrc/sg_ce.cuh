// sg_ce.cuh -- continuous-energy cross-section lookup and neutronCEstd scattering kinematics on the
// device (aceNeutronNuclide, ceNeutronMaterial, aceNeutronDatabase, scatteringKernels_func).
//
// Energies are FP64 in both precision forms; cross sections, densities and the kinematics of the
// scattered direction are in R.  A grid search returns the reference's floor index exactly
// (binaryFloorIdxClosed_Real, genericProcedures.f90:132-166: the largest i with e(i) <= E, and
// N-1 for E = e(N)); it starts from a log-energy hash bracket and finishes with a binary search.
#pragma once
#include "sg_device.cuh"

namespace sg {

// Floor index (0-based lower point) of E in e[0..n-1], or -1 when E lies outside [e[0], e[n-1]].
// `b` is the hash bin of E; h[b] brackets it (e[lo] <= E < e[hi] for every E of the bin).  A
// bracket that does not hold (E outside the hashed range) falls back to the whole grid.
// Grid energies are positive, and for non-negative IEEE doubles the order of the values is the order
// of their bit patterns read as signed 64-bit integers; so every comparison here is an integer one
// (the integer pipe instead of the FP64 pipe, which this GPU issues at a small fraction of its
// FP32 rate) with the same outcome.  A negative or NaN E compares outside the grid, as before.
__device__ __forceinline__ int ce_search(const double* __restrict__ e, int n, const int2* __restrict__ h, int b,
                                         double E) {
  const long long* __restrict__ k = reinterpret_cast<const long long*>(e);
  const long long x = __double_as_longlong(E);
  if (!(x >= k[0] && x <= k[n - 1])) return -1;
  if (x == k[n - 1]) return n - 2;
  int lo = 0, hi = n - 1;
  if (h) {
    const int2 br = h[b];
    if (k[br.x] <= x && x < k[br.y]) { lo = br.x; hi = br.y; }
  }
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (k[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int ce_hash_bin(float logE, float logMin, float invStep, int nBins) {
  int b = __float2int_rd((logE - logMin) * invStep);
  return min(max(b, 0), nBins - 1);
}

// interpolation factor f = (E - E_low) / (E_top - E_low) (aceNeutronNuclide_class.f90:342-359)
template <class R>
__device__ __forceinline__ R ce_factor(const double* e, int i, double E) {
  if constexpr (sizeof(R) == 8) return (E - e[i]) / (e[i + 1] - e[i]);
  else return (float)(E - e[i]) / (float)(e[i + 1] - e[i]);
}
// xs(idx+1)*f + (1-f)*xs(idx) of column k (totalXS / microXSs, :374-453)
template <class R>
__device__ __forceinline__ R ce_interp(const R* __restrict__ x, long long i, R f, int k) {
  return x[(i + 1) * 4 + k] * f + (R(1) - f) * x[i * 4 + k];
}

// One energy's lookup context: E, its hash bin in the nuclide table and, with the union table, its
// floor index u in the union grid (-1 outside it).
struct CEPoint {
  double E;
  int b;
  int u;
};

template <class R>
__device__ __forceinline__ CEPoint ce_point(const DCE<R>& d, double E) {
  CEPoint p;
  p.E = E;
  const float lg = __logf((float)E);
  p.b = ce_hash_bin(lg, d.hLogMin, d.hInvStep, d.nHash);
  p.u = -1;
  if (d.lidx) {
    p.u = ce_search(d.lu, d.nLU, d.luhash, ce_hash_bin(lg, d.luLogMin, d.luInvStep, d.nLUHash), E);
    // E on the last union point: its own row (ce_search gives the last interval), so that a nuclide
    // grid ending in a repeated point finds its last index and the closed rule below
    if (p.u == d.nLU - 2 && __double_as_longlong(E) == __double_as_longlong(d.lu[d.nLU - 1])) p.u = d.nLU - 1;
  }
  return p;
}

// nuclide search: returns the global index of the lower grid point (or -1) and f.
// With the union table one search per energy (in ce_point) serves every nuclide: every point of a
// nuclide's grid is a union point, so no nuclide point lies strictly between union points u and
// u + 1, and the nuclide's floor index at E equals its floor index at union point u, which the
// table holds.  At the top of a nuclide's grid the closed rule of binaryFloorIdxClosed applies: E
// equal to its last point takes the last interval, anything above is outside.  The result is the
// index ce_search would find, so both forms keep their results bit for bit.
template <class R>
__device__ __forceinline__ long long ce_nuc_search(const DCE<R>& d, int nuc, const CEPoint& p, R& f) {
  const long long o = d.off[nuc];
  const int n = (int)(d.off[nuc + 1] - o);
  int i;
  if (d.lidx) {
    if (p.u < 0) return -1;
    i = d.lidx[(long long)p.u * d.nNuc + nuc];
    if (i < 0) return -1;
    if (i == n - 1) {
      if (__double_as_longlong(p.E) != __double_as_longlong(d.e[o + n - 1])) return -1;
      i = n - 2;
    }
  } else {
    i = ce_search(d.e + o, n, d.hash + (long long)nuc * d.nHash, p.b, p.E);
    if (i < 0) return -1;
  }
  f = ce_factor<R>(d.e + o, i, p.E);
  return o + i;
}

// updateTotalMatXS (aceNeutronDatabase_class.f90:517-570): sum of dens * sigma_t over the
// composition, in order.  Returns false when E lies outside a nuclide's grid.
template <class R>
__device__ __forceinline__ bool ce_mat_total(const DCE<R>& d, int mat, const CEPoint& p, R& total) {
  total = R(0);
  for (int k = d.matPtr[mat - 1]; k < d.matPtr[mat]; ++k) {
    R f;
    const long long i = ce_nuc_search<R>(d, d.matNuc[k], p, f);
    if (i < 0) return false;
    total = total + d.matDens[k] * ce_interp<R>(d.xs, i, f, 0);
  }
  return true;
}

// updateMacroXSs (:577-640) for a non-fissile material: x = [total, elastic, inelastic, capture]
template <class R>
__device__ __forceinline__ bool ce_mat_macro(const DCE<R>& d, int mat, const CEPoint& p, R x[4]) {
  x[0] = x[1] = x[2] = x[3] = R(0);
  for (int k = d.matPtr[mat - 1]; k < d.matPtr[mat]; ++k) {
    R f;
    const long long i = ce_nuc_search<R>(d, d.matNuc[k], p, f);
    if (i < 0) return false;
    const R dens = d.matDens[k];
#pragma unroll
    for (int c = 0; c < 4; ++c) x[c] = x[c] + dens * ce_interp<R>(d.xs, i, f, c);
  }
  return true;
}

// updateMajorantXS (:346-394): the unionised majorant interpolated at E, or the maximum of the
// active materials' totals
template <class R>
__device__ __forceinline__ bool ce_majorant(const DCE<R>& d, const CEPoint& p, R& xs) {
  if (d.hasMajorant) {
    int i;
    if (d.lmaj) {                      // every majorant grid point is a union point: a table read
      if (p.u < 0) return false;
      i = d.lmaj[p.u];
      if (i < 0) return false;
      if (i == d.nU - 1) {
        if (__double_as_longlong(p.E) != __double_as_longlong(d.ue[d.nU - 1])) return false;
        i = d.nU - 2;
      }
    } else {
      const int b = ce_hash_bin(__logf((float)p.E), d.uLogMin, d.uInvStep, d.nUHash);
      i = ce_search(d.ue, d.nU, d.uhash, b, p.E);
    }
    if (i < 0) return false;
    const R f = ce_factor<R>(d.ue, i, p.E);
    xs = d.umaj[i + 1] * f + (R(1) - f) * d.umaj[i];
    return true;
  }
  xs = R(0);
  for (int a = 0; a < d.nAct; ++a) {
    R t;
    if (!ce_mat_total<R>(d, d.act[a], p, t)) return false;
    xs = fmax(xs, t);
  }
  return true;
}

// Euclidean norm: gfortran's scaled NORM2 in FP64 (as SCONE's norm2 calls), plain in FP32
template <class R> __device__ __forceinline__ R norm3(R a, R b, R c);
template <> __device__ __forceinline__ double norm3<double>(double a, double b, double c) { return norm2_scaled(a, b, c); }
template <> __device__ __forceinline__ float norm3<float>(float a, float b, float c) { return sqrtf(a * a + b * b + c * c); }

// ------------------------------------------------------------------ scatteringKernels_func.f90
// cos(0.5*pi*r1)
template <class R> __device__ __forceinline__ R cos_half_pi(R r);
template <> __device__ __forceinline__ double cos_half_pi<double>(double r) {
  return cos((0.5 * 3.14159265358979323846264338327950288) * r);
}
template <> __device__ __forceinline__ float cos_half_pi<float>(float r) { return cospif(0.5f * r); }

// sample_x2expx2 (:281-311) and sample_x3expx2 (:319-334)
template <class R>
__device__ __forceinline__ R sample_x2expx2(Rng<R>& rng) {
  const R r1 = rng.get(), r2 = rng.get(), r3 = rng.get();
  const R cosine = cos_half_pi<R>(r1);
  const R beta = cosine * cosine;
  const R gamma05 = -dlog<R>(r2) * beta;
  const R sample = -dlog<R>(r3) + gamma05;
  return dsqrt<R>(sample);
}
template <class R>
__device__ __forceinline__ R sample_x3expx2(Rng<R>& rng) {
  const R r1 = rng.get(), r2 = rng.get();
  const R sample = -dlog<R>(r1) - dlog<R>(r2);
  return dsqrt<R>(sample);
}

// targetVelocity_constXS (:101-139) with sample_targetVelocity (:340-380).  The rejection loop is
// bounded (each pass accepts with probability >= 1/2 for the constant-XS kernel); on exhaustion the
// last sample is kept and *bad is set.
template <class R>
__device__ __forceinline__ void target_velocity(R E, R dx, R dy, R dz, R A, R kT, Rng<R>& rng, R V[3], bool* bad) {
  const R SQRT_PI = dsqrt<R>(R(3.14159265358979323846264338327950288));   // numPrecision.f90:24
  const R Y = dsqrt<R>(A * E / kT);
  const R alpha = R(2) / (Y * SQRT_PI + R(2));
  R X = R(0), mu = R(0);
  int it = 0;
  for (;; ++it) {
    const R r1 = rng.get(), r2 = rng.get(), r3 = rng.get();
    if (r1 > alpha) X = sample_x2expx2<R>(rng);
    else X = sample_x3expx2<R>(rng);
    mu = R(2) * r2 - R(1);
    const R rel_v = dsqrt<R>(Y * Y + X * X - R(2) * X * Y * mu);
    const R P_acc = rel_v / (Y + X);
    if (P_acc > r3) break;
    if (it >= 100000) { *bad = true; break; }
  }
  R sp, cp;
  sincos_phi<R>(rng.get(), sp, cp);
  R u = dx, v = dy, w = dz;
  rotate_vector<R>(u, v, w, mu, sp, cp);
  const R s = X * dsqrt<R>(kT / A);
  V[0] = u * s; V[1] = v * s; V[2] = w * s;
}

}  // namespace sg
