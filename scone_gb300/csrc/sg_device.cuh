// sg_device.cuh -- device-side data layout and the particle-tracking hot path of libsconegpu.
//
// Everything in this header is templated on the working precision R:
//   R = double : all-FP64 verification form.  Compiled with -fmad=false so every multiply and add is
//                rounded separately, in SCONE's operation order; per-history results then match the
//                CPU restatement exactly (collision counts, end-of-history RNG states, bin indices).
//   R = float  : mixed form.  Cross sections, distances, sampling, directions and the coordinates
//                below the root (local to their universe) in FP32; the global position, the tests
//                against root-level surfaces, tally sums and k in FP64.  Geometric tolerances are
//                widened to the FP32 distance accuracy (see Tol<float> and the host's surface records).
//
// Data layout in HBM (all flat, read-only during a launch, resident across cycles):
//   surfaces  DSurf[n]           136 B records (type, axes, bc, FP64 params and tolerance, FP32 copies)
//   universes DUni[n]            208 B records; pin radii, cell lists and the geometry graph are
//                                separate int/double arrays indexed from the record
//   MG data   [mat][G] SoA arrays of R, P0/prod as [mat][Gin][Gout]
//   banks     SoA: r (3 x FP64), dir (3 x FP64), wgt, G, brood -- see sg_internal.h
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "sg_internal.h"

// How the cell-universe search and distance are compiled: inlined (default) or as one out-of-line
// copy (-DSG_CELL_SEARCH=__noinline__), which keeps their surface loops out of the code of the
// geometries that have no cell universes.  Out of line measured slower on the same GB300 (lattice
// cycle -3.6 %, uneven batch -13 %): the call costs more than the smaller code saves.
#ifndef SG_CELL_SEARCH
#define SG_CELL_SEARCH __forceinline__
#endif

namespace sg {

// ------------------------------------------------------------------ constants
__device__ __constant__ static const double D_INF = 9223372036854775808.0;   // 2**63 (universalVariables.f90:21)

template <class R> struct Tol;
// SCONE's values (universalVariables.f90:21-25, numPrecision.f90:25, transportOperatorST_class.f90:59,
// genericProcedures.f90:1067 -- the last two are default-real literals).
template <> struct Tol<double> {
  static __device__ __forceinline__ double fp_rel() { return 1.0e-7; }
  static __device__ __forceinline__ double st_void() { return (double)1.0E-12f; }
  static __device__ __forceinline__ double rot() { return (double)1.0E-8f; }
};
// FP32 distances land a crossing within ~1e-6 relative of the surface, so the tie rule between
// nesting levels is widened to 1e-5; surface tolerances and the cell-crossing nudge are scaled on
// the host (surface records carry the tolerance of the form they were uploaded for).
template <> struct Tol<float> {
  static __device__ __forceinline__ float fp_rel() { return 1.0e-5f; }
  static __device__ __forceinline__ float st_void() { return 1.0E-12f; }
  static __device__ __forceinline__ float rot() { return 1.0E-4f; }
};

// ------------------------------------------------------------------ RNG (RandomNumbers/RNG_class.f90)
static constexpr uint64_t RNG_G = 2806196910506780709ULL;
static constexpr uint64_t RNG_MASK = 0x7FFFFFFFFFFFFFFFULL;
static constexpr int64_t RNG_STRIDE = 152917;

__device__ __forceinline__ uint64_t lcg_next(uint64_t s) {
  s = (RNG_G * s) & RNG_MASK;
  return (s + 1ULL) & RNG_MASK;
}
template <class R> __device__ __forceinline__ R rng_to_real(uint64_t s);
// get: real(seed) * 2^-63 (RNG_class.f90:161)
template <> __device__ __forceinline__ double rng_to_real<double>(uint64_t s) {
  return __ll2double_rn((long long)s) * 0x1p-63;
}
// mixed form: the top 24 bits of the 63-bit state, made odd so that xi lies in (0,1) and -log(xi)
// is finite; the LCG stream (and so every draw's position in it) is the same as in FP64.
template <> __device__ __forceinline__ float rng_to_real<float>(uint64_t s) {
  return (float)((uint32_t)(s >> 39) | 1u) * 0x1p-24f;
}
// skip (RNG_class.f90:251-304)
__host__ __device__ inline uint64_t lcg_skip(uint64_t s, int64_t k_in) {
  uint64_t k = (k_in >= 0) ? (uint64_t)k_in : (uint64_t)INT64_MAX - (uint64_t)(-k_in) + 1ULL;
  k &= RNG_MASK;
  uint64_t Gk = 1, Ck = 0, gsq = RNG_G, L = 1;
  while (k > 0) {
    if (k & 1ULL) {
      Gk = (Gk * gsq) & RNG_MASK;
      Ck = (Ck * gsq) & RNG_MASK;
      Ck = (Ck + L) & RNG_MASK;
    }
    L = (L * (gsq + 1ULL)) & RNG_MASK;
    gsq = (gsq * gsq) & RNG_MASK;
    k >>= 1;
  }
  return (Gk * s + Ck) & RNG_MASK;
}

template <class R> struct Rng {
  uint64_t s;
  __device__ __forceinline__ R get() { s = lcg_next(s); return rng_to_real<R>(s); }
};

// ------------------------------------------------------------------ math helpers
template <class R> __device__ __forceinline__ R dlog(R x);
template <> __device__ __forceinline__ double dlog<double>(double x) { return log(x); }
template <> __device__ __forceinline__ float dlog<float>(float x) { return logf(x); }
template <class R> __device__ __forceinline__ R dsqrt(R x);
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
__device__ __forceinline__ double sgn(double a, double b) { return copysign(fabs(a), b); }
__device__ __forceinline__ float sgn(float a, float b) { return copysignf(fabsf(a), b); }
// Component i of a 3-vector held in registers, by selects (a runtime index into a register array
// would force the array into local memory).
template <class T> __device__ __forceinline__ T at3(const T* a, int i) { return i == 0 ? a[0] : (i == 1 ? a[1] : a[2]); }

// sin/cos of phi = 2*pi*xi (multiScatterMG_class.f90:208, pointSource_class.f90:221)
template <class R> __device__ __forceinline__ void sincos_phi(R xi, R& s, R& c);
template <> __device__ __forceinline__ void sincos_phi<double>(double xi, double& s, double& c) {
  const double TWO_PI = 2.0 * 3.14159265358979323846264338327950288;
  double phi = TWO_PI * xi;
  sincos(phi, &s, &c);
}
template <> __device__ __forceinline__ void sincos_phi<float>(float xi, float& s, float& c) {
  sincospif(2.0f * xi, &s, &c);
}

// gfortran NORM2 (scaled sum of squares) used by rotateVector's final normalisation
__device__ __forceinline__ double norm2_scaled(double a0, double a1, double a2) {
  double scale = 1.0, ssq = 0.0;
  double v[3] = {a0, a1, a2};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (v[i] != 0.0) {
      double a = fabs(v[i]);
      if (scale < a) { double t = scale / a; ssq = 1.0 + ssq * t * t; scale = a; }
      else { double t = a / scale; ssq = ssq + t * t; }
    }
  }
  return scale * sqrt(ssq);
}

// rotateVector (SharedModules/genericProcedures.f90:1047-1084)
// sampleLegendre_P1 (SharedModules/legendrePoly_func.f90:35-99): the mixing method of Lux and
// Koblinger for the linearly anisotropic density 1/2 (1 + a mu), a = 3 P1/P0: with |a| < 1 the
// linear density (1 + mu)/2 with probability |a|, else uniform; with 1 <= |a| <= 3 a delta at
// mu = 1 with probability (|a| - 1)/2, else the linear density; mirrored for a < 0.
template <class R, class G>
__device__ __forceinline__ R sample_legendre_p1(R a, G& rng) {
  const R al = fabs(a);
  R thr;
  int top, low;                            // 1 uniform, 2 linear, 3 delta
  if (al < R(1)) { thr = al; top = 2; low = 1; }
  else { thr = R(0.5) * (al - R(1)); top = 3; low = 2; }
  const int ex = (rng.get() < thr) ? top : low;
  R x;
  if (ex == 1) x = R(2) * rng.get() - R(1);
  else if (ex == 2) x = R(2) * dsqrt<R>(rng.get()) - R(1);
  else x = R(1);
  return a < R(0) ? -x : x;
}

template <class R>
__device__ __forceinline__ void rotate_vector(R& u, R& v, R& w, R mu, R sinPol, R cosPol) {
  R A = dsqrt<R>(fmax(R(0), R(1) - mu * mu));
  R B = dsqrt<R>(fmax(R(0), R(1) - w * w));
  R n0, n1, n2;
  if (B > Tol<R>::rot()) {
    n0 = mu * u + A * (u * w * cosPol - v * sinPol) / B;
    n1 = mu * v + A * (v * w * cosPol + u * sinPol) / B;
    n2 = mu * w - A * B * cosPol;
  } else {
    B = dsqrt<R>(fmax(R(0), R(1) - v * v));
    n0 = mu * u + A * (u * v * cosPol + w * sinPol) / B;
    n1 = mu * v - A * B * cosPol;
    n2 = mu * w + A * (v * w * cosPol - u * sinPol) / B;
  }
  if constexpr (sizeof(R) == 8) {
    double n = norm2_scaled(n0, n1, n2);
    u = n0 / n; v = n1 / n; w = n2 / n;
  } else {
    float inv = rsqrtf(n0 * n0 + n1 * n1 + n2 * n2);
    u = n0 * inv; v = n1 * inv; w = n2 * inv;
  }
}

// ------------------------------------------------------------------ surfaces (Geometry/Surfaces)
// Position type T: double for the root level (global coordinates) and for every level in the FP64
// form; R (float) for levels below the root in the mixed form, where parameters come from the FP32
// copies.  The coincidence test `abs(c) < tol` is evaluated in T.
template <class T> __device__ __forceinline__ T SP(const DSurf& s, int i);
template <> __device__ __forceinline__ double SP<double>(const DSurf& s, int i) { return s.p[i]; }
template <> __device__ __forceinline__ float SP<float>(const DSurf& s, int i) { return s.pf[i]; }
template <class T> __device__ __forceinline__ T STOL(const DSurf& s);
template <> __device__ __forceinline__ double STOL<double>(const DSurf& s) { return s.tol; }
template <> __device__ __forceinline__ float STOL<float>(const DSurf& s) { return s.tolf; }
template <class T> __device__ __forceinline__ T UD(const DUni& u, int i);
template <> __device__ __forceinline__ double UD<double>(const DUni& u, int i) { return u.d[i]; }
template <> __device__ __forceinline__ float UD<float>(const DUni& u, int i) { return u.f[i]; }
template <class T> __device__ __forceinline__ T UO(const DUni& u, int i);
template <> __device__ __forceinline__ double UO<double>(const DUni& u, int i) { return u.origin[i]; }
template <> __device__ __forceinline__ float UO<float>(const DUni& u, int i) { return u.originf[i]; }
template <class T> __device__ __forceinline__ T PIN_RSQ(const DGeom& g, int k);
template <> __device__ __forceinline__ double PIN_RSQ<double>(const DGeom& g, int k) { return g.pin_rsq[k]; }
template <> __device__ __forceinline__ float PIN_RSQ<float>(const DGeom& g, int k) { return g.pin_rsqf[k]; }
template <class T> __device__ __forceinline__ T PIN_TOL(const DGeom& g, int k);
template <> __device__ __forceinline__ double PIN_TOL<double>(const DGeom& g, int k) { return g.pin_tol[k]; }
template <> __device__ __forceinline__ float PIN_TOL<float>(const DGeom& g, int k) { return g.pin_tolf[k]; }

template <class T>
__device__ __forceinline__ T surf_evaluate(const DSurf& s, const T r[3]) {
  switch (s.type) {
    case SG_SURF_XPLANE: case SG_SURF_YPLANE: case SG_SURF_ZPLANE:
      return at3(r, s.axis) - SP<T>(s, 0);                                       // aPlane_class.f90:139
    case SG_SURF_PLANE:
      return (r[0] * SP<T>(s, 0) + r[1] * SP<T>(s, 1) + r[2] * SP<T>(s, 2)) - SP<T>(s, 3);   // plane :125
    case SG_SURF_XCYL: case SG_SURF_YCYL: case SG_SURF_ZCYL: {                   // cylinder_class.f90:222
      T d0 = at3(r, s.pl0) - SP<T>(s, s.pl0), d1 = at3(r, s.pl1) - SP<T>(s, s.pl1);
      return (d0 * d0 + d1 * d1) - SP<T>(s, 3) * SP<T>(s, 3);
    }
    case SG_SURF_SPHERE: {                                                        // sphere_class.f90:143
      T d0 = r[0] - SP<T>(s, 0), d1 = r[1] - SP<T>(s, 1), d2 = r[2] - SP<T>(s, 2);
      return (d0 * d0 + d1 * d1 + d2 * d2) - SP<T>(s, 3) * SP<T>(s, 3);
    }
    case SG_SURF_BOX: {                                                           // box_class.f90:134-143
      T m = fmax(fabs(r[0] - SP<T>(s, 0)) - SP<T>(s, 3), fabs(r[1] - SP<T>(s, 1)) - SP<T>(s, 4));
      return fmax(m, fabs(r[2] - SP<T>(s, 2)) - SP<T>(s, 5));
    }
    default: {                                                                    // squareCylinder evaluate
      T a = fabs(at3(r, s.pl0) - SP<T>(s, s.pl0)) - SP<T>(s, 3 + s.pl0);
      T b = fabs(at3(r, s.pl1) - SP<T>(s, s.pl1)) - SP<T>(s, 3 + s.pl1);
      return fmax(a, b);
    }
  }
}

// box/squareCylinder slab intersection (box_class.f90:168-237, squareCylinder_class.f90:212-270)
// onSurf: the particle may sit on a surface (it has just crossed or hit one), so a point within the
// surface tolerance takes SCONE's on-surface branches; false: the plain intersection (mixed form,
// after a collision or a placement; see Geom::place)
template <class R, class T>
__device__ __forceinline__ R slab_distance(const DSurf& s, const T r[3], const R u[3], int nax,
                                           int ax0, int ax1, int ax2, bool onSurf = true) {
  const R FP_MISS_TOL = (sizeof(R) == 8) ? R(1.0 + 10.0 * 2.220446049250313e-16) : R(1.0f + 10.0f * 1.1920929e-7f);
  const R HUGE_R = (sizeof(R) == 8) ? R(1.7976931348623157e308) : R(3.4028234663852886e38f);
  const R INF_R = R(D_INF);
  R far = HUGE_R, near = -HUGE_R;
  int axes[3] = {ax0, ax1, ax2};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (i < nax) {
      int ax = axes[i];
      R rb = R(at3(r, ax) - SP<T>(s, ax));
      R ua = at3(u, ax);
      R a_far = sgn(R(SP<T>(s, 3 + ax)), ua);
      R a_near = -a_far;
      R tn, tf;
      if (ua != R(0)) { tn = (a_near - rb) / ua; tf = (a_far - rb) / ua; }
      else {
        tn = sgn(INF_R, a_near - rb); tf = sgn(INF_R, a_far - rb);
        if (tn > tf) { R t = tn; tn = tf; tf = t; }
      }
      far = fmin(far, tf);
      near = fmax(near, tn);
    }
  }
  R d;
  if (far <= near * FP_MISS_TOL) d = INF_R;
  else if (onSurf && fabs(surf_evaluate<T>(s, r)) < STOL<T>(s)) d = (fabs(far) >= fabs(near)) ? far : near;
  else d = (near <= R(0)) ? far : near;
  if (d <= R(0) || d > INF_R) d = INF_R;
  return d;
}

template <class R, class T>
__device__ __forceinline__ R surf_distance(const DSurf& s, const T r[3], const R u[3], bool onSurf = true) {
  const R INF_R = R(D_INF);
  switch (s.type) {
    case SG_SURF_XPLANE: case SG_SURF_YPLANE: case SG_SURF_ZPLANE: {   // aPlane_class.f90:157-181
      T ra = SP<T>(s, 0) - at3(r, s.axis);
      R ua = at3(u, s.axis), d;
      if (onSurf && fabs(ra) < STOL<T>(s)) d = INF_R;
      else if (ua != R(0)) d = R(ra) / ua;
      else d = INF_R;
      if (d <= R(0) || d > INF_R) d = INF_R;
      return d;
    }
    case SG_SURF_PLANE: {                                                // plane_class.f90:144-163
      R k = u[0] * R(SP<T>(s, 0)) + u[1] * R(SP<T>(s, 1)) + u[2] * R(SP<T>(s, 2));
      T c = surf_evaluate<T>(s, r);
      R d;
      if (k == R(0) || (onSurf && fabs(c) < STOL<T>(s))) d = INF_R;
      else { d = -R(c) / k; if (d <= R(0) || d > INF_R) d = INF_R; }
      return d;
    }
    case SG_SURF_XCYL: case SG_SURF_YCYL: case SG_SURF_ZCYL: {           // cylinder_class.f90:231-270
      T c = surf_evaluate<T>(s, r);
      R k = R(at3(r, s.pl0) - SP<T>(s, s.pl0)) * at3(u, s.pl0) + R(at3(r, s.pl1) - SP<T>(s, s.pl1)) * at3(u, s.pl1);
      R a = R(1) - at3(u, s.axis) * at3(u, s.axis);
      R delta = k * k - a * R(c), d;
      if (delta < R(0) || a == R(0)) d = INF_R;
      else if (onSurf && fabs(c) < STOL<T>(s)) {
        if (k >= R(0)) d = INF_R;
        else { d = -k + dsqrt<R>(delta); d = d / a; }
      } else if (c < T(0)) { d = -k + dsqrt<R>(delta); d = d / a; }
      else { d = -k - dsqrt<R>(delta); d = d / a; if (d <= R(0)) d = INF_R; }
      return fmin(d, INF_R);
    }
    case SG_SURF_SPHERE: {                                               // sphere_class.f90:152-183
      T c = surf_evaluate<T>(s, r);
      R k = R(r[0] - SP<T>(s, 0)) * u[0] + R(r[1] - SP<T>(s, 1)) * u[1] + R(r[2] - SP<T>(s, 2)) * u[2];
      R delta = k * k - R(c), d;
      if (delta < R(0)) d = INF_R;
      else if (onSurf && fabs(c) < STOL<T>(s)) { if (k >= R(0)) d = INF_R; else d = -k + dsqrt<R>(delta); }
      else if (c < T(0)) d = -k + dsqrt<R>(delta);
      else { d = -k - dsqrt<R>(delta); if (d <= R(0)) d = INF_R; }
      return d;
    }
    case SG_SURF_BOX:
      return slab_distance<R, T>(s, r, u, 3, 0, 1, 2, onSurf);
    default:
      return slab_distance<R, T>(s, r, u, 2, s.pl0, s.pl1, 0, onSurf);
  }
}

template <class R, class T>
__device__ __forceinline__ bool surf_going(const DSurf& s, const T r[3], const R u[3]) {
  switch (s.type) {
    case SG_SURF_XPLANE: case SG_SURF_YPLANE: case SG_SURF_ZPLANE:
      return at3(u, s.axis) > R(0);
    case SG_SURF_PLANE: {
      R proj = u[0] * R(SP<T>(s, 0)) + u[1] * R(SP<T>(s, 1)) + u[2] * R(SP<T>(s, 2));
      if (proj == R(0)) return surf_evaluate<T>(s, r) >= T(0);
      return proj > R(0);
    }
    case SG_SURF_XCYL: case SG_SURF_YCYL: case SG_SURF_ZCYL:
      return (R(at3(r, s.pl0) - SP<T>(s, s.pl0)) * at3(u, s.pl0) + R(at3(r, s.pl1) - SP<T>(s, s.pl1)) * at3(u, s.pl1)) >= R(0);
    case SG_SURF_SPHERE:
      return (R(r[0] - SP<T>(s, 0)) * u[0] + R(r[1] - SP<T>(s, 1)) * u[1] + R(r[2] - SP<T>(s, 2)) * u[2]) >= R(0);
    default: {   // box (box_class.f90:253-281) and squareCylinder (:272-300)
      int axes[3] = {0, 1, 2};
      int nax = 3;
      if (s.type != SG_SURF_BOX) { axes[0] = s.pl0; axes[1] = s.pl1; nax = 2; }
      int maxCom = axes[0];
      T best = T(-1.0e30);
      T rlm = T(0);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        if (i < nax) {
          T rl = at3(r, axes[i]) - SP<T>(s, axes[i]);
          T v = fabs(rl) - SP<T>(s, 3 + axes[i]);
          if (i == 0 || v > best) { best = v; maxCom = axes[i]; rlm = rl; }
        }
      }
      R proj = at3(u, maxCom) * (R)sgn(T(1), rlm);
      if (proj == R(0)) return surf_evaluate<T>(s, r) >= T(0);
      return proj > R(0);
    }
  }
}

// dirTol: SCONE's rule for a point within the surface tolerance -- the side the direction points
// to (surface_inter.f90:363-378).  Without it the sign of the surface function decides (mixed form,
// points not on a surface; see Geom::place).
template <class R, class T>
__device__ __forceinline__ bool surf_halfspace(const DSurf& s, const T r[3], const R u[3], bool dirTol = true) {
  T c = surf_evaluate<T>(s, r);
  bool hs = c > T(0);
  if (dirTol && fabs(c) < STOL<T>(s)) hs = surf_going<R, T>(s, r, u);
  return hs;
}

// The reduced half-width below which a coordinate is "well inside" for the boundary transforms.
// FP64 form: SCONE's halfwidth * (1 - surfTol) with the relative SURF_TOL (box_class.f90:393,440).
// Mixed form, whose tolerance is an absolute length of a few FP32 ulps of the geometry: the explicit
// BC (applied on a boundary hit, where the hit coordinates sit on their faces only to FP32 accuracy)
// takes the half-width less that length; the transform BC after a delta-tracking flight takes the
// half-width itself, so that it transforms exactly the coordinates that the sign classification of
// the flight's end point put outside.  (A wider band reflects a coordinate that was inside next to
// another face and leaves the point outside: the history would end as a leak.)
template <class R>
__device__ __forceinline__ double bc_inner(const DSurf& s, int ax, bool transform) {
  if constexpr (sizeof(R) == 8) return s.p[3 + ax] * (1.0 - s.tol);
  else return transform ? s.p[3 + ax] : s.p[3 + ax] - s.tol;
}

// explicitBC (box_class.f90:380-420, squareCylinder_class.f90:430-472); root level, FP64 positions
template <class R>
__device__ __forceinline__ void surf_explicit_bc(const DSurf& s, double r[3], R u[3]) {
  if (s.type != SG_SURF_BOX && !(s.type >= SG_SURF_XSQCYL && s.type <= SG_SURF_ZSQCYL)) return;
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    bool active = (s.type == SG_SURF_BOX) || ax == s.pl0 || ax == s.pl1;
    if (!active) continue;
    double r0 = r[ax] - s.p[ax];
    if (fabs(r0) <= bc_inner<R>(s, ax, false)) continue;
    // mixed form: of the coordinates within that band of their faces only those heading out (the
    // hit one, and a second one at a corner hit); one heading in keeps its direction, where a
    // reflection would turn it outward on its face and the placement would put it outside
    if constexpr (sizeof(R) == 4) { if ((double)u[ax] * r0 <= 0.0) continue; }
    int b = (r0 < 0.0) ? s.bc[2 * ax] : s.bc[2 * ax + 1];
    if (b == SG_BC_REFLECTIVE) u[ax] = -u[ax];
    else if (b == SG_BC_PERIODIC) r[ax] = r[ax] - 2.0 * sgn(s.p[3 + ax], r0);
  }
}

// transformBC (box_class.f90:430-487, squareCylinder_class.f90:482-544); root level, FP64 positions
template <class R>
__device__ __forceinline__ void surf_transform_bc(const DSurf& s, double r[3], R u[3]) {
  if (s.type != SG_SURF_BOX && !(s.type >= SG_SURF_XSQCYL && s.type <= SG_SURF_ZSQCYL)) return;
  int Ri[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    bool active = (s.type == SG_SURF_BOX) || ax == s.pl0 || ax == s.pl1;
    double a_bar = bc_inner<R>(s, ax, true);
    Ri[ax] = active ? ((int)ceil(fabs(r[ax] - s.p[ax]) / a_bar)) / 2 : 0;
  }
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    bool active = (s.type == SG_SURF_BOX) || ax == s.pl0 || ax == s.pl1;
    if (!active) continue;
    for (int t = 1; t <= Ri[ax] && t <= 64; ++t) {
      double r0 = r[ax] - s.p[ax];
      int b = (r0 < 0.0) ? s.bc[2 * ax] : s.bc[2 * ax + 1];
      if (b == SG_BC_REFLECTIVE) {
        double a0 = sgn(s.p[3 + ax], r0) + s.p[ax];
        double d = r[ax] - a0;
        r[ax] = r[ax] - 2.0 * d;
        u[ax] = -u[ax];
      } else if (b == SG_BC_PERIODIC) {
        double d = sgn(s.p[3 + ax], r0);
        r[ax] = r[ax] - 2.0 * d;
      }
    }
  }
}

// ------------------------------------------------------------------ geometry state of one particle
// Level 1 (the root universe, global coordinates) is held in FP64; the levels below in R: FP64 in the
// verification form, FP32 local coordinates in the mixed form.  Levels live in registers (MAXL is a
// compile-time bound >= the geometry's nesting).  One direction is kept, the global one: the
// direction at a level below a rotated universe is the rotation matrix times the direction of the
// level above, recomputed where it is needed, which is what SCONE stores per level and recomputes
// after every change of the global direction (coord_class.f90:385-408,453-472).
template <class R, int MAXL>
struct Coords {
  double r0[3];
  R rl[MAXL > 1 ? MAXL - 1 : 1][3];
  R u[3];
  int uni[MAXL];
  int base[MAXL];    // graph location (0-based) of local cell 1 of the level's universe (uniRootID-1)
  int local[MAXL];   // localID, 1-based
  int nest;
  int mat;
  int uid;
};

struct DistCache {   // geometry_inter.f90:21-25
  int lvl;
};

template <class T> struct Vec3 { T x, y, z; };

// matmul(rotMat, v) of a 3x3 row-major matrix (universe%enter, universe_inter.f90:400-424), each
// component summed left to right as gfortran's matmul does
template <class T>
__device__ __noinline__ Vec3<T> rot_vec(const T* m, T x, T y, T z) {
  return Vec3<T>{m[0] * x + m[1] * y + m[2] * z, m[3] * x + m[4] * y + m[5] * z, m[6] * x + m[7] * y + m[8] * z};
}

// LEAN: compiled for geometries without rotated universes (the rotation code is left out).
template <class R, int MAXL, bool LEAN = false>
struct Geom {
  const DGeom& g;
  __device__ __forceinline__ explicit Geom(const DGeom& gg) : g(gg) {}
  __device__ __forceinline__ bool rotated() const { return !LEAN && g.rot != nullptr; }

  template <class T> __device__ __forceinline__ const T* rotm(int u) const {
    if constexpr (sizeof(T) == 8) return g.rot + 9 * u;
    else return g.rotf + 9 * u;
  }
  // direction at level l (1..MAXL-1; level 0 is the root): the global direction turned by every
  // rotated universe entered on levels 1..l
  __device__ __forceinline__ void level_dir(const Coords<R, MAXL>& c, int l, R d[3]) const {
    d[0] = c.u[0]; d[1] = c.u[1]; d[2] = c.u[2];
    if (!rotated()) return;
#pragma unroll
    for (int j = 1; j < MAXL; ++j) {
      if (j > l) break;
      const int u = c.uni[j];
      if (g.unis[u].rot) {
        const Vec3<R> v = rot_vec<R>(rotm<R>(u), d[0], d[1], d[2]);
        d[0] = v.x; d[1] = v.y; d[2] = v.z;
      }
    }
  }

  // unionCell%insideComplex (unionCell_class.f90:365-401): left to right over the evaluation array;
  // a union that is already true or an intersection that is already false ends the current bracket
  // (shortCircuit, :406-422) or, at depth 0, the whole cell
  template <class T>
  __device__ __forceinline__ bool inside_complex(int cell, const T r[3], const R dir[3], bool dirTol = true) const {
    bool isIt = true;
    int depth = 0;
    const int end = g.cell_ptr[cell + 1];
    for (int i = g.cell_ptr[cell]; i < end; ++i) {
      const int el = g.cell_surf[i];
      if (!cell_is_op(el)) {
        const bool hs = surf_halfspace<R, T>(g.surfs[abs(el) - 1], r, dir, dirTol);
        isIt = (hs == (el > 0));
      } else if ((el == CELL_UNION && isIt) || (el == CELL_INTERSECT && !isIt)) {
        if (depth == 0) return isIt;
        depth -= 1;
        for (int d = 1; d > 0 && i + 1 < end;) {
          const int e2 = g.cell_surf[++i];
          if (e2 == CELL_OPEN) d += 1;
          else if (e2 == CELL_CLOSE) d -= 1;
        }
      } else if (el == CELL_OPEN) depth += 1;
      else if (el == CELL_CLOSE) depth -= 1;
    }
    return isIt;
  }

  // cellUniverse%findCell (cellUniverse_class.f90:203-246): the first cell of the universe whose
  // simpleCell / unionCell test holds, n + 1 if none.  SG_CELL_SEARCH sets how it is compiled
  // (inlined into every level's search, or one out-of-line copy).
  template <class T>
  __device__ SG_CELL_SEARCH int find_cell_cells(const DUni& U, const T r[3], const R dir[3], bool dirTol) const {
    const int nc = U.i[1];
    for (int c = 0; c < nc; ++c) {
      const int cell = g.uni_cells[U.i[0] + c];
      bool isIt = false;
      if (g.cell_complex && g.cell_complex[cell]) isIt = inside_complex<T>(cell, r, dir, dirTol);
      else
        for (int k = g.cell_ptr[cell]; k < g.cell_ptr[cell + 1]; ++k) {   // simpleCell :90-111
          const int ss = g.cell_surf[k];
          if (cell_is_op(ss)) continue;                        // brackets of an all-intersection cell
          const bool hs = surf_halfspace<R, T>(g.surfs[abs(ss) - 1], r, dir, dirTol);
          isIt = (hs == (ss > 0));
          if (!isIt) break;
        }
      if (isIt) return c + 1;
    }
    return nc + 1;
  }

  // universe%findCell for the universe `u` at local position r; dirTol as in surf_halfspace (the
  // pin and lattice searches' direction-dependent tolerances follow it too)
  template <class T>
  __device__ __forceinline__ int find_cell(int u, const T r[3], const R dir[3], bool dirTol = true) const {
    const DUni& U = g.unis[u];
    switch (U.type) {
      case SG_UNI_ROOT:                                          // rootUniverse_class.f90:127-145
        return surf_halfspace<R, T>(g.surfs[U.i[0]], r, dir, dirTol) ? 2 : 1;
      case SG_UNI_CELL:
        return find_cell_cells<T>(U, r, dir, dirTol);
      case SG_UNI_PIN: {                                         // pinUniverse_class.f90:150-173
        T rsq = r[0] * r[0] + r[1] * r[1];
        T mul = !dirTol ? T(0) : (((T)(r[0] * (T)dir[0] + r[1] * (T)dir[1]) >= T(0)) ? T(-1) : T(1));
        int N = U.i[1];
        for (int l = 1; l <= N; ++l)
          if (rsq < PIN_RSQ<T>(g, U.i[0] + l - 1) + mul * PIN_TOL<T>(g, U.i[0] + l - 1)) return l;
        return N + 1;
      }
      default: {                                                 // latUniverse_class.f90:270-312
        int ijk[3];
        bool out = false;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const T pitch = UD<T>(U, i), corner = UD<T>(U, 3 + i);
          // FP64 form: SCONE's division; mixed form: the reciprocal pitch (a cell boundary within an
          // ulp is then settled by the tolerance test below, as any FP32 rounding is)
          if constexpr (sizeof(T) == 8) ijk[i] = (int)floor((r[i] - corner) / pitch) + 1;
          else ijk[i] = (int)floorf((r[i] - corner) * U.invf[i]) + 1;
          T r_bar = r[i] - corner - ijk[i] * pitch + T(0.5) * pitch;
          if (dirTol && fabs(r_bar) > UD<T>(U, 6 + i) && r_bar * (T)dir[i] > T(0)) ijk[i] += (dir[i] < R(0)) ? -1 : 1;
          if (ijk[i] <= 0 || ijk[i] > U.i[i]) out = true;
        }
        return out ? U.i[3] : ijk[0] + U.i[0] * (ijk[1] - 1 + U.i[1] * (ijk[2] - 1));
      }
    }
  }

  // floor(t / n) for 0 <= t < 2^24 and n >= 1 from the FP32 reciprocal inv ~ 1/n: the estimate is
  // off by at most one and corrected exactly, so the quotient equals the integer division's
  __device__ __forceinline__ static int quot(int t, int n, float inv) {
    int q = __float2int_rz(__int2float_rn(t) * inv);
    const int r = t - q * n;
    if (r < 0) q -= 1;
    else if (r >= n) q += 1;
    return q;
  }
  __device__ __forceinline__ static void get_ijk(int localID, const DUni& U, int ijk[3]) {
    int temp = localID - 1;                                      // latUniverse_class.f90:489-506
    int base = quot(temp, U.i[0], U.invn[0]);
    ijk[0] = temp - U.i[0] * base + 1;
    temp = base;
    base = quot(temp, U.i[1], U.invn[1]);
    ijk[1] = temp - U.i[1] * base + 1;
    ijk[2] = base + 1;
  }

  // pin annulus k: zCylinder at the origin (pinUniverse_class.f90:114-118)
  template <class T>
  __device__ __forceinline__ R pin_cyl(const DUni& U, int k, const T r[3], const R u[3], bool onSurf) const {
    const R INF_R = R(D_INF);
    T c = (r[0] * r[0] + r[1] * r[1]) - PIN_RSQ<T>(g, U.i[0] + k);
    R kk = R(r[0]) * u[0] + R(r[1]) * u[1];
    R a = R(1) - u[2] * u[2];
    R delta = kk * kk - a * R(c), d;
    if (delta < R(0) || a == R(0)) d = INF_R;
    else if (onSurf && fabs(c) < PIN_TOL<T>(g, U.i[0] + k)) {
      if (kk >= R(0)) d = INF_R;
      else { d = -kk + dsqrt<R>(delta); d = d / a; }
    } else if (c < T(0)) { d = -kk + dsqrt<R>(delta); d = d / a; }
    else { d = -kk - dsqrt<R>(delta); d = d / a; if (d <= R(0)) d = INF_R; }
    return fmin(d, INF_R);
  }

  // simpleCell%distance (simpleCell_class.f90:120-141; unionCell :426-443 alike): the nearest of the
  // cell's surfaces; compiled as SG_CELL_SEARCH says
  template <class T>
  __device__ SG_CELL_SEARCH void cell_distance(const DUni& U, int localID, const T r[3], const R dir[3], R& d,
                                               int& surfIdx, bool onSurf) const {
    const int cell = g.uni_cells[U.i[0] + localID - 1];
    d = R(D_INF);
    surfIdx = 0;
    for (int k = g.cell_ptr[cell]; k < g.cell_ptr[cell + 1]; ++k) {
      const int ss = g.cell_surf[k];
      if (cell_is_op(ss)) continue;
      const R td = surf_distance<R, T>(g.surfs[abs(ss) - 1], r, dir, onSurf);
      if (td < d) { d = td; surfIdx = abs(ss); }
    }
  }

  // universe%distance; onSurf as in surf_distance
  template <class T>
  __device__ __forceinline__ void uni_distance(int u, int localID, const T r[3], const R dir[3],
                                               R& d, int& surfIdx, bool onSurf = true) const {
    const R INF_R = R(D_INF);
    const DUni& U = g.unis[u];
    switch (U.type) {
      case SG_UNI_ROOT:                                          // rootUniverse_class.f90:152-162
        surfIdx = U.i[0] + 1;
        d = surf_distance<R, T>(g.surfs[U.i[0]], r, dir, onSurf);
        return;
      case SG_UNI_CELL:
        cell_distance<T>(U, localID, r, dir, d, surfIdx, onSurf);
        return;
      case SG_UNI_PIN: {                                         // pinUniverse_class.f90:185-226
        int N = U.i[1];
        R d_out = (localID > N) ? INF_R : pin_cyl<T>(U, localID - 1, r, dir, onSurf);
        R d_in = (localID == 1) ? INF_R : pin_cyl<T>(U, localID - 2, r, dir, onSurf);
        if (d_in < d_out) { surfIdx = -1; d = d_in; } else { surfIdx = -2; d = d_out; }
        return;
      }
      default: {                                                 // latUniverse_class.f90:319-373
        if (localID == U.i[3]) {
          surfIdx = -7;
          d = surf_distance<R, T>(g.surfs[U.i[4]], r, dir, onSurf);     // outline box
          return;
        }
        int ijk[3];
        get_ijk(localID, U, ijk);
        d = INF_R;
        int ax = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const T pitch = UD<T>(U, i);
          T r_bar = r[i] - UD<T>(U, 3 + i);
          r_bar = r_bar - (ijk[i] - T(0.5)) * pitch;
          R bound = sgn(R(pitch * T(0.5)), dir[i]);
          R td = (bound - R(r_bar)) / dir[i];
          if (td < d) { d = td; ax = i; }
        }
        d = fmax(R(0), d);
        d = fmin(INF_R, d);
        R uax = (ax == 0) ? dir[0] : (ax == 1) ? dir[1] : dir[2];
        int s = (ax + 1) * 2;
        if (uax < R(0)) s -= 1;
        surfIdx = -s;
        return;
      }
    }
  }

  // universe%cellOffset (latUniverse_class.f90:394-414; zero for the others)
  template <class T>
  __device__ __forceinline__ void cell_offset(int u, int localID, T off[3]) const {
    const DUni& U = g.unis[u];
    off[0] = off[1] = off[2] = T(0);
    if (U.type == SG_UNI_LAT && U.i[5] != 0 && localID != U.i[3]) {
      int ijk[3];
      get_ijk(localID, U, ijk);
#pragma unroll
      for (int i = 0; i < 3; ++i) off[i] = (ijk[i] - T(0.5)) * UD<T>(U, i) + UD<T>(U, 3 + i);
    }
  }

  // Mixed form: the level-2 coordinates are re-derived from the FP64 level-1 position instead of
  // being accumulated separately in FP32, so both levels see one position wherever their surfaces
  // coincide (a lattice filling the root box).  The FP64 form accumulates every level as SCONE does.
  // The root universe carries no cell offset, so a level-2 universe without an origin offset takes
  // float(r0) directly (the same value, without two FP64 subtractions of zero).
  __device__ __forceinline__ void sync_level2(Coords<R, MAXL>& c) const {
    if constexpr (sizeof(R) == 4 && MAXL > 1) {
      if (c.nest > 1) {
        const DUni& N = g.unis[c.uni[1]];
        if (N.i[6]) {
#pragma unroll
          for (int k = 0; k < 3; ++k) c.rl[0][k] = R(c.r0[k]);
          return;
        }
        enter_level1(c, c.uni[1]);
      }
    }
  }

  // level-1 coordinates in universe nu entered from the root (cell offset, rotation, origin), from
  // the FP64 global position
  __device__ __forceinline__ void enter_level1(Coords<R, MAXL>& c, int nu) const {
    const DUni& N = g.unis[nu];
    double off[3];
    cell_offset<double>(c.uni[0], c.local[0], off);
    double t[3] = {c.r0[0] - off[0], c.r0[1] - off[1], c.r0[2] - off[2]};
    if (rotated() && N.rot) {
      const Vec3<double> v = rot_vec<double>(rotm<double>(nu), t[0], t[1], t[2]);
      t[0] = v.x; t[1] = v.y; t[2] = v.z;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) c.rl[0][k] = R(t[k] - N.origin[k]);
  }

  // level-l distance (root level in FP64 positions, lower levels in R)
  __device__ __forceinline__ void level_distance(Coords<R, MAXL>& c, int l, R& d, int& s, bool onSurf = true) const {
    if (l == 0) uni_distance<double>(c.uni[0], c.local[0], c.r0, c.u, d, s, onSurf);
    else {
      if (l == 1) sync_level2(c);
      R dl[3];
      level_dir(c, l, dl);
      uni_distance<R>(c.uni[l], c.local[l], c.rl[l > 0 ? l - 1 : 0], dl, d, s, onSurf);
    }
  }

  // geometryStd%diveToMat (geometryStd_class.f90:565-619); returns false on nesting overflow.
  // rf: float(r0) when the caller has it (mixed form), so an origin-free level 2 reuses it
  __device__ __forceinline__ bool dive(Coords<R, MAXL>& c, int start, const float* rf = nullptr,
                                       bool dirTol = true) const {
#pragma unroll
    for (int i = 0; i < MAXL; ++i) {
      if (i < start) continue;
      int loc = c.base[i] + c.local[i] - 1;
      int2 gf = g.graph[loc];
      if (gf.x >= 0) { c.mat = gf.x; c.uid = gf.y; c.nest = i + 1; return true; }
      if (i + 1 >= MAXL) break;
      int nu = -gf.x - 1;
      const DUni& N = g.unis[nu];
      if (i == 0) {
        if (sizeof(R) == 4 && N.i[6]) {
          if (rf) {
#pragma unroll
            for (int k = 0; k < 3; ++k) c.rl[0][k] = R(rf[k]);
          } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) c.rl[0][k] = R(c.r0[k]);
          }
        } else {
          enter_level1(c, nu);
        }
      } else {
        R off[3];
        cell_offset<R>(c.uni[i], c.local[i], off);
        R t[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) t[k] = c.rl[i > 0 ? i - 1 : 0][k] - off[k];
        if (rotated() && N.rot) {
          const Vec3<R> v = rot_vec<R>(rotm<R>(nu), t[0], t[1], t[2]);
          t[0] = v.x; t[1] = v.y; t[2] = v.z;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) c.rl[i][k] = t[k] - UO<R>(N, k);
      }
      c.uni[i + 1] = nu;
      c.base[i + 1] = gf.y - 1;
      R dl[3];
      level_dir(c, i + 1, dl);
      c.local[i + 1] = find_cell<R>(nu, c.rl[i], dl, dirTol);
    }
    c.mat = SG_UNDEF_MAT;
    c.nest = MAXL;
    return false;
  }

  // geometryStd%placeCoord (geometryStd_class.f90:119-147): level-1 position is c.r0 (global;
  // the root universe carries no origin offset)
  // Mixed form: the root border test is first made in FP32 at float(r0); only a value within the
  // surface's filter margin (tolerance plus the FP32 error bound) goes to the FP64 test, so the side
  // found is always the FP64 one.
  // onSurface: the point may lie on a surface (a boundary hit), so SCONE's direction-dependent
  // tolerance rule decides it.  Points reached by a flight, a history start or a split release are
  // not on a surface; in the mixed form they are classified by the sign of each surface function.
  // There the tolerances are sized to FP32 crossing accuracy (~4e-6 cm), and the rule would assign
  // a shell of that thickness around every surface by flight direction instead of by position.
  // The FP64 form applies the rule everywhere, as SCONE does (its 1e-12 tolerance leaves no shell).
  // (The global position stays FP64 in the mixed form too: keeping it as a pair of floats added
  // with error-free two-sums removed the FP64 adds and conversions per flight but measured slower,
  // -8 % on the lattice with delta tracking and -12 % on the uneven batch, same GB300.)
  __device__ __forceinline__ bool place(Coords<R, MAXL>& c, bool onSurface = true) const {
    c.uni[0] = g.root;
    c.base[0] = 0;
    int loc = 0;
    if constexpr (sizeof(R) == 4) {
      const float rf[3] = {(float)c.r0[0], (float)c.r0[1], (float)c.r0[2]};
      const DSurf& S = g.surfs[g.border];
      if (S.filt > 0.0f) {
        const float v = surf_evaluate<float>(S, rf);
        if (v > S.filt) loc = 2;
        else if (v < -S.filt) loc = 1;
      }
      if (loc == 0) loc = find_cell<double>(g.root, c.r0, c.u, onSurface);
      c.local[0] = loc;
      return dive(c, 0, rf, onSurface);
    }
    (void)onSurface;
    if (loc == 0) loc = find_cell<double>(g.root, c.r0, c.u);
    c.local[0] = loc;
    return dive(c, 0);
  }

  // geometryStd%teleport (geometryStd_class.f90:492-514)
  __device__ __forceinline__ bool teleport(Coords<R, MAXL>& c, R dist) const {
    // the step in the working precision, accumulated in FP64 (in the FP64 form the same products)
#pragma unroll
    for (int k = 0; k < 3; ++k) c.r0[k] = c.r0[k] + (double)(dist * c.u[k]);
    bool ok = place(c, false);
    if (c.mat == 0) {
      surf_transform_bc<R>(g.surfs[g.border], c.r0, c.u);
      ok = place(c, false);
    }
    return ok;
  }

  // moveLocal over levels 1..n (coord_class.f90:346-356)
  __device__ __forceinline__ void move_levels(Coords<R, MAXL>& c, int n, R d) const {
#pragma unroll
    for (int k = 0; k < 3; ++k) c.r0[k] = c.r0[k] + (double)(d * c.u[k]);
    R v[3] = {c.u[0], c.u[1], c.u[2]};
#pragma unroll
    for (int l = 1; l < MAXL; ++l)
      if (l < n) {
        if (rotated() && g.unis[c.uni[l]].rot) {          // this level's direction (rotated universe)
          const Vec3<R> t = rot_vec<R>(rotm<R>(c.uni[l]), v[0], v[1], v[2]);
          v[0] = t.x; v[1] = t.y; v[2] = t.z;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) c.rl[l - 1][k] = c.rl[l - 1][k] + d * v[k];
      }
  }

  // move_withCache / move_noCache (geometryStd_class.f90:214-352); fields absent (fieldDist = INF).
  // Returns the event; maxDist is replaced by the distance moved.
  // onSurf: whether the particle may sit on a surface (it reached this point by a crossing or a
  // boundary hit); the FP64 form always takes SCONE's on-surface branches
  __device__ __forceinline__ int move(Coords<R, MAXL>& c, R& maxDist, R cdist[MAXL], int csurf[MAXL],
                                      DistCache& cache, bool useCache, bool onSurf = true) const {
    if constexpr (sizeof(R) == 8) onSurf = true;
    R dist = R(D_INF);
    int surfIdx = 0, level = 0;
    if (!useCache) cache.lvl = 0;
#pragma unroll
    for (int l = 0; l < MAXL; ++l) {
      if (l < c.nest) {
        if (cache.lvl < l + 1) {
          level_distance(c, l, cdist[l], csurf[l], onSurf);
          cache.lvl += 1;
        }
        R td = cdist[l];
        // geometryStd_class.f90:655,710 tie rule; the mixed form adds an absolute term of a few FP32
        // ulps of the geometry size so coincident surfaces at different levels resolve to the upper one
        if ((dist - td) >= dist * Tol<R>::fp_rel() + R(g.tie_abs)) { dist = td; surfIdx = csurf[l]; level = l + 1; }
      }
    }
    if (maxDist < dist) {                                         // collision inside the cell
      move_levels(c, c.nest, maxDist);
      cache.lvl = 0;
      return 1;   // COLL_EV
    }
    if (surfIdx == g.border + 1 && level == 1) {                  // domain boundary
#pragma unroll
      for (int k = 0; k < 3; ++k) c.r0[k] = c.r0[k] + (double)(dist * c.u[k]);
      maxDist = dist;
      cache.lvl = 0;
      surf_explicit_bc<R>(g.surfs[g.border], c.r0, c.u);
      place(c);
      return 2;   // BOUNDARY_EV
    }
    // crossing at `level`
    move_levels(c, level, dist);
    maxDist = dist;
#pragma unroll
    for (int l = 0; l < MAXL; ++l) if (l < level - 1) cdist[l] = cdist[l] - dist;
    cache.lvl = level - 1;
    c.nest = level;
#pragma unroll
    for (int l = 0; l < MAXL; ++l) {
      if (l == level - 1) {
        const DUni& U = g.unis[c.uni[l]];
        if (U.type == SG_UNI_PIN) {                               // pinUniverse_class.f90:236-253
          c.local[l] += (surfIdx == -1) ? -1 : 1;
        } else if (l == 0) {
          if (U.type == SG_UNI_CELL) {                            // cellUniverse_class.f90:388-431
#pragma unroll
            for (int k = 0; k < 3; ++k) c.r0[k] = c.r0[k] + (double)c.u[k] * g.nudge;
          }
          c.local[0] = find_cell<double>(c.uni[0], c.r0, c.u);
        } else {
          if (l == 1) sync_level2(c);
          R* rr = c.rl[l > 0 ? l - 1 : 0];
          R dl[3];
          level_dir(c, l, dl);
          if (U.type == SG_UNI_CELL) {
#pragma unroll
            for (int k = 0; k < 3; ++k) rr[k] = rr[k] + dl[k] * (R)g.nudge;
          }
          c.local[l] = find_cell<R>(c.uni[l], rr, dl);
        }
      }
    }
    dive(c, level - 1);
    return 3;   // CROSS_EV
  }
};

}  // namespace sg
