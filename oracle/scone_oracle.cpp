// SPDX-License-Identifier: MIT
//
// TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
//
// A scalar CPU restatement of SCONE's particle-tracking cycle (Fortran, CambridgeNuclear/SCONE),
// used as the correctness oracle for libsconegpu.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py may load it.  Every routine cites the SCONE file:line
// it restates.  The arithmetic follows SCONE's operation order; build with -ffp-contract=off so
// no fused multiply-add changes a rounding (gfortran -O3 without -march emits none on x86-64).
//
// Parity pinning: SCONE cannot be compiled in this build environment (no Fortran compiler), so the
// restatement is pinned against the golden values of SCONE's own unit/integration tests
// (RNG, surfaces, universes, geometryStd, MG data, scoreMemory, clerks) in tests/test_oracle_*.py,
// and the RNG against a Python big-integer evaluation of the same recurrence.
//
// It consumes the same description structs as the product ABI (include/scone_gpu.h) and exposes
// an `or_*` C ABI with the same meaning as the `sg_*` entry points.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <string>
#include <algorithm>
#include <map>
#include <memory>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/scone_gpu.h"

namespace orc {

// ---------------------------------------------------------------- constants
// SharedModules/universalVariables.f90:21-25, numPrecision.f90:24-25
static const double INF = 9223372036854775808.0;   // 2**63
static const double SURF_TOL = 1.0e-12;
static const double NUDGE = 1.0e-8;
static const double FP_REL_TOL = 1.0e-7;
static const double ST_TOL = (double)1.0E-12f;     // transportOperatorST_class.f90:59 (default-real literal)
static const double ROT_TOL = (double)1.0E-8f;     // genericProcedures.f90:1067 (default-real literal)
static const double PI = 3.14159265358979323846264338327950288;
static const double TWO_PI = 2.0 * PI;
static const int MAX_NEST = 12;

static const int OUTSIDE_MAT = 0;
static const int VOID_MAT = 2147483647;
static const int UNDEF_MAT = VOID_MAT - 1;
static const int OVERLAP_MAT = VOID_MAT - 2;

// geometry events (universalVariables.f90:28-32)
enum { COLL_EV = 1, BOUNDARY_EV = 2, CROSS_EV = 3 };
// fates (tallyCodes.f90:23-27)
enum { NO_FATE = 5000, ABS_FATE = 5001, LEAK_FATE = 5002 };
// macro MTs (endfConstants.f90:116-130)
enum { macroTotal = -1, macroDisappearance = -2, macroEscatter = -3, macroIEscatter = -4,
       macroFission = -6, macroNuFission = -7, macroKappaFission = -80, macroAllScatter = -20,
       macroAbsorbtion = -21, macroNonElastic = -22 };

// ---------------------------------------------------------------- RNG (RandomNumbers/RNG_class.f90)
static const uint64_t RNG_G = 2806196910506780709ULL;   // :40
static const uint64_t RNG_MASK = 0x7FFFFFFFFFFFFFFFULL; // :43 bitMask = huge(0_int64)
static const int64_t STRIDE = 152917;                   // :128

struct RNG {
  uint64_t s = 0;
  // get (:147-168): seed = iand(g*seed, mask); seed = iand(seed+c, mask); rand = seed*2^-63
  double get() {
    s = (RNG_G * s) & RNG_MASK;
    s = (s + 1ULL) & RNG_MASK;
    return (double)(int64_t)s * 0x1p-63;
  }
  // skip (:251-304), F. Brown's O(log k) jump
  void skip(int64_t k_in) {
    uint64_t k;
    if (k_in >= 0) k = (uint64_t)k_in;
    else k = (uint64_t)INT64_MAX - (uint64_t)(-k_in) + 1ULL;   // huge(M) - abs(k) + 1
    k &= RNG_MASK;
    uint64_t Gk = 1, Ck = 0, gsq = RNG_G, L = 1;
    while (k > 0) {
      if (k & 1ULL) {
        Gk = (Gk * gsq) & RNG_MASK;
        Ck = (Ck * gsq) & RNG_MASK;
        Ck = (Ck + L) & RNG_MASK;
      }
      L = (L * (gsq + 1ULL)) & RNG_MASK;
      gsq = (gsq * gsq) & RNG_MASK;        // pow_of_gsq table (:61-123) = successive squares
      k >>= 1;
    }
    s = (Gk * s + Ck) & RNG_MASK;
  }
  void stride(int32_t n) { skip(STRIDE * (int64_t)n); }   // :310-316
};

// ---------------------------------------------------------------- helpers
static inline double sgn(double a, double b) { return std::copysign(std::fabs(a), b); }  // Fortran SIGN

// gfortran NORM2: scaled sum of squares (avoids overflow), used for norm2() calls in SCONE
static double norm2_3(const double v[3]) {
  double scale = 1.0, ssq = 0.0;
  for (int i = 0; i < 3; ++i) {
    if (v[i] != 0.0) {
      double a = std::fabs(v[i]);
      if (scale < a) { double t = scale / a; ssq = 1.0 + ssq * t * t; scale = a; }
      else { double t = a / scale; ssq = ssq + t * t; }
    }
  }
  return scale * std::sqrt(ssq);
}

// sampleLegendre_P1 (SharedModules/legendrePoly_func.f90:35-99), mixing method (Lux & Koblinger)
static double sampleLegendreP1(double P1, RNG& rng, std::string& err) {
  const double a = std::fabs(P1);
  double threshold;
  int top, low;                                          // 1 uniform, 2 linear, 3 delta
  if (a < 1.0) { threshold = a; top = 2; low = 1; }
  else if (a <= 3.0) { threshold = 0.5 * (a - 1.0); top = 3; low = 2; }
  else { err = "P1 must have absolute value < 3.0"; return 0.0; }
  const int exec = (rng.get() < threshold) ? top : low;
  double x;
  if (exec == 1) x = 2.0 * rng.get() - 1.0;
  else if (exec == 2) x = 2.0 * std::sqrt(rng.get()) - 1.0;
  else x = 1.0;
  if (P1 < 0.0) x = -x;
  return x;
}

// rotateVector (SharedModules/genericProcedures.f90:1047-1084)
static void rotateVector(const double dir[3], double mu, double phi, double out[3]) {
  double sinPol = std::sin(phi);
  double cosPol = std::cos(phi);
  double u = dir[0], v = dir[1], w = dir[2];
  double A = std::sqrt(std::max(0.0, 1.0 - mu * mu));
  double B = std::sqrt(std::max(0.0, 1.0 - w * w));
  if (B > ROT_TOL) {
    out[0] = mu * u + A * (u * w * cosPol - v * sinPol) / B;
    out[1] = mu * v + A * (v * w * cosPol + u * sinPol) / B;
    out[2] = mu * w - A * B * cosPol;
  } else {
    B = std::sqrt(std::max(0.0, 1.0 - v * v));
    out[0] = mu * u + A * (u * v * cosPol + w * sinPol) / B;
    out[1] = mu * v - A * B * cosPol;
    out[2] = mu * w + A * (v * w * cosPol - u * sinPol) / B;
  }
  double n = norm2_3(out);
  out[0] /= n; out[1] /= n; out[2] /= n;
}

// ---------------------------------------------------------------- surfaces (Geometry/Surfaces)
struct Surface {
  int type = 0;
  double p[SG_SURF_NPAR] = {0};
  double tol = SURF_TOL;
  int bc[6] = {0, 0, 0, 0, 0, 0};
  int axis = 2, plane0 = 0, plane1 = 1;   // cylinders / square cylinders

  void build(int t, const double* par) {
    type = t;
    for (int i = 0; i < SG_SURF_NPAR; ++i) p[i] = par[i];
    switch (t) {
      case SG_SURF_XCYL: case SG_SURF_XSQCYL: axis = 0; plane0 = 1; plane1 = 2; break;
      case SG_SURF_YCYL: case SG_SURF_YSQCYL: axis = 1; plane0 = 0; plane1 = 2; break;
      default: axis = 2; plane0 = 0; plane1 = 1; break;
    }
    if (t == SG_SURF_PLANE) {                       // plane_class.f90:78-84 coeffs/norm2(coeffs(1:3))
      double n3[3] = {par[0], par[1], par[2]};
      double n = norm2_3(n3);
      for (int i = 0; i < 4; ++i) p[i] = par[i] / n;
    }
    if (t == SG_SURF_XCYL || t == SG_SURF_YCYL || t == SG_SURF_ZCYL || t == SG_SURF_SPHERE)
      tol = 2.0 * p[3] * SURF_TOL;                  // cylinder_class.f90:181, sphere_class.f90:107
    else
      tol = SURF_TOL;
  }
  int aplaneAxis() const { return type - SG_SURF_XPLANE; }

  double evaluate(const double r[3]) const {
    switch (type) {
      case SG_SURF_XPLANE: case SG_SURF_YPLANE: case SG_SURF_ZPLANE:
        return r[aplaneAxis()] - p[0];                                   // aPlane_class.f90:139
      case SG_SURF_PLANE:
        return (r[0] * p[0] + r[1] * p[1] + r[2] * p[2]) - p[3];        // plane_class.f90:125
      case SG_SURF_XCYL: case SG_SURF_YCYL: case SG_SURF_ZCYL: {        // cylinder_class.f90:222
        double d0 = r[plane0] - p[plane0], d1 = r[plane1] - p[plane1];
        return (d0 * d0 + d1 * d1) - p[3] * p[3];
      }
      case SG_SURF_SPHERE: {                                            // sphere_class.f90:143
        double d0 = r[0] - p[0], d1 = r[1] - p[1], d2 = r[2] - p[2];
        return (d0 * d0 + d1 * d1 + d2 * d2) - p[3] * p[3];
      }
      case SG_SURF_BOX: {                                               // box_class.f90:134-143
        double m = -HUGE_VAL;
        for (int i = 0; i < 3; ++i) m = std::max(m, std::fabs(r[i] - p[i]) - p[3 + i]);
        return m;
      }
      default: {                                                        // squareCylinder evaluate
        double a = std::fabs(r[plane0] - p[plane0]) - p[3 + plane0];
        double b = std::fabs(r[plane1] - p[plane1]) - p[3 + plane1];
        return std::max(a, b);
      }
    }
  }

  double distance(const double r[3], const double u[3]) const {
    switch (type) {
      case SG_SURF_XPLANE: case SG_SURF_YPLANE: case SG_SURF_ZPLANE: {  // aPlane_class.f90:157-181
        int ax = aplaneAxis();
        double ra = p[0] - r[ax], ua = u[ax], d;
        if (std::fabs(ra) < tol) d = INF;
        else if (ua != 0.0) d = ra / ua;
        else d = INF;
        if (d <= 0.0 || d > INF) d = INF;
        return d;
      }
      case SG_SURF_PLANE: {                                             // plane_class.f90:144-163
        double k = u[0] * p[0] + u[1] * p[1] + u[2] * p[2];
        double c = evaluate(r), d;
        if (k == 0.0 || std::fabs(c) < tol) d = INF;
        else { d = -c / k; if (d <= 0.0 || d > INF) d = INF; }
        return d;
      }
      case SG_SURF_XCYL: case SG_SURF_YCYL: case SG_SURF_ZCYL: {        // cylinder_class.f90:231-270
        double c = evaluate(r);
        double k = (r[plane0] - p[plane0]) * u[plane0] + (r[plane1] - p[plane1]) * u[plane1];
        double a = 1.0 - u[axis] * u[axis];
        double delta = k * k - a * c, d;
        if (delta < 0.0 || a == 0.0) d = INF;
        else if (std::fabs(c) < tol) {
          if (k >= 0.0) d = INF;
          else { d = -k + std::sqrt(delta); d = d / a; }
        } else if (c < 0.0) { d = -k + std::sqrt(delta); d = d / a; }
        else { d = -k - std::sqrt(delta); d = d / a; if (d <= 0.0) d = INF; }
        return std::min(d, INF);
      }
      case SG_SURF_SPHERE: {                                            // sphere_class.f90:152-183
        double c = evaluate(r);
        double k = (r[0] - p[0]) * u[0] + (r[1] - p[1]) * u[1] + (r[2] - p[2]) * u[2];
        double delta = k * k - c, d;
        if (delta < 0.0) d = INF;
        else if (std::fabs(c) < tol) { if (k >= 0.0) d = INF; else d = -k + std::sqrt(delta); }
        else if (c < 0.0) d = -k + std::sqrt(delta);
        else { d = -k - std::sqrt(delta); if (d <= 0.0) d = INF; }
        return d;
      }
      case SG_SURF_BOX: {                                               // box_class.f90:168-237
        static const double FP_MISS_TOL = 1.0 + 10.0 * 2.220446049250313e-16;
        double far = 1.7976931348623157e308, near = -1.7976931348623157e308;   // huge(far)
        for (int ax = 0; ax < 3; ++ax) {
          double rb = r[ax] - p[ax];
          double a_far = sgn(p[3 + ax], u[ax]);
          double a_near = -a_far;
          double tn, tf;
          if (u[ax] != 0.0) { tn = (a_near - rb) / u[ax]; tf = (a_far - rb) / u[ax]; }
          else {
            tn = sgn(INF, a_near - rb); tf = sgn(INF, a_far - rb);
            if (tn > tf) std::swap(tn, tf);
          }
          far = std::min(far, tf);
          near = std::max(near, tn);
        }
        double d;
        if (far <= near * FP_MISS_TOL) d = INF;
        else if (std::fabs(evaluate(r)) < tol) d = (std::fabs(far) >= std::fabs(near)) ? far : near;
        else d = (near <= 0.0) ? far : near;
        if (d <= 0.0 || d > INF) d = INF;
        return d;
      }
      default: {                                                        // squareCylinder :212-270
        static const double FP_MISS_TOL = 1.0 + 10.0 * 2.220446049250313e-16;
        double far = 1.7976931348623157e308, near = -1.7976931348623157e308;
        int pl[2] = {plane0, plane1};
        for (int i = 0; i < 2; ++i) {
          int ax = pl[i];
          double rb = r[ax] - p[ax];
          double a_far = sgn(p[3 + ax], u[ax]);
          double a_near = -a_far;
          double tn, tf;
          if (u[ax] != 0.0) { tn = (a_near - rb) / u[ax]; tf = (a_far - rb) / u[ax]; }
          else {
            tn = sgn(INF, a_near - rb); tf = sgn(INF, a_far - rb);
            if (tn > tf) std::swap(tn, tf);
          }
          far = std::min(far, tf);
          near = std::max(near, tn);
        }
        double d;
        if (far <= near * FP_MISS_TOL) d = INF;
        else if (std::fabs(evaluate(r)) < tol) d = (std::fabs(far) >= std::fabs(near)) ? far : near;
        else d = (near <= 0.0) ? far : near;
        if (d <= 0.0 || d > INF) d = INF;
        return d;
      }
    }
  }

  bool going(const double r[3], const double u[3]) const {
    switch (type) {
      case SG_SURF_XPLANE: case SG_SURF_YPLANE: case SG_SURF_ZPLANE:
        return u[aplaneAxis()] > 0.0;                                   // aPlane_class.f90:195
      case SG_SURF_PLANE: {                                             // plane_class.f90:172-186
        double proj = u[0] * p[0] + u[1] * p[1] + u[2] * p[2];
        bool hs = proj > 0.0;
        if (proj == 0.0) hs = evaluate(r) >= 0.0;
        return hs;
      }
      case SG_SURF_XCYL: case SG_SURF_YCYL: case SG_SURF_ZCYL:          // cylinder_class.f90:281
        return ((r[plane0] - p[plane0]) * u[plane0] + (r[plane1] - p[plane1]) * u[plane1]) >= 0.0;
      case SG_SURF_SPHERE:                                              // sphere_class.f90:192
        return ((r[0] - p[0]) * u[0] + (r[1] - p[1]) * u[1] + (r[2] - p[2]) * u[2]) >= 0.0;
      case SG_SURF_BOX: {                                               // box_class.f90:253-281
        double rl[3]; int maxCom = 0; double best = -HUGE_VAL;
        for (int i = 0; i < 3; ++i) {
          rl[i] = r[i] - p[i];
          double v = std::fabs(rl[i]) - p[3 + i];
          if (v > best) { best = v; maxCom = i; }
        }
        double proj = u[maxCom] * sgn(1.0, rl[maxCom]);
        bool hs = proj > 0.0;
        if (proj == 0.0) hs = evaluate(r) >= 0.0;
        return hs;
      }
      default: {                                                        // squareCylinder :272-300
        int pl[2] = {plane0, plane1};
        double rl[2]; int maxCom = 0; double best = -HUGE_VAL;
        for (int i = 0; i < 2; ++i) {
          rl[i] = r[pl[i]] - p[pl[i]];
          double v = std::fabs(rl[i]) - p[3 + pl[i]];
          if (v > best) { best = v; maxCom = i; }
        }
        double proj = u[pl[maxCom]] * sgn(1.0, rl[maxCom]);
        bool hs = proj > 0.0;
        if (proj == 0.0) hs = evaluate(r) >= 0.0;
        return hs;
      }
    }
  }

  // surface_inter.f90:363-378
  bool halfspace(const double r[3], const double u[3]) const {
    double c = evaluate(r);
    bool hs = c > 0.0;
    if (std::fabs(c) < tol) hs = going(r, u);
    return hs;
  }

  // box_class.f90:380-420, squareCylinder_class.f90:430-472 (vacuum for all other surfaces)
  void explicitBC(double r[3], double u[3]) const {
    if (type != SG_SURF_BOX && !(type >= SG_SURF_XSQCYL && type <= SG_SURF_ZSQCYL)) return;
    int axes[3] = {0, 1, 2}; int nax = 3;
    if (type != SG_SURF_BOX) { axes[0] = plane0; axes[1] = plane1; nax = 2; }
    for (int i = 0; i < nax; ++i) {
      int ax = axes[i];
      double r0 = r[ax] - p[ax];
      if (std::fabs(r0) <= p[3 + ax] * (1.0 - tol)) continue;
      int b = (r0 < 0.0) ? bc[2 * ax] : bc[2 * ax + 1];
      if (b == SG_BC_REFLECTIVE) u[ax] = -u[ax];
      else if (b == SG_BC_PERIODIC) r[ax] = r[ax] - 2.0 * sgn(p[3 + ax], r0);
    }
  }

  // box_class.f90:430-487, squareCylinder_class.f90:482-544
  void transformBC(double r[3], double u[3]) const {
    if (type != SG_SURF_BOX && !(type >= SG_SURF_XSQCYL && type <= SG_SURF_ZSQCYL)) return;
    int axes[3] = {0, 1, 2}; int nax = 3;
    if (type != SG_SURF_BOX) { axes[0] = plane0; axes[1] = plane1; nax = 2; }
    int Ri[3];
    for (int i = 0; i < nax; ++i) {
      int ax = axes[i];
      double a_bar = p[3 + ax] * (1.0 - tol);
      Ri[i] = ((int)std::ceil(std::fabs(r[ax] - p[ax]) / a_bar)) / 2;
    }
    for (int i = 0; i < nax; ++i) {
      int ax = axes[i];
      for (int t = 1; t <= Ri[i]; ++t) {
        double r0 = r[ax] - p[ax];
        int b = (r0 < 0.0) ? bc[2 * ax] : bc[2 * ax + 1];
        if (b == SG_BC_REFLECTIVE) {
          double a0 = sgn(p[3 + ax], r0) + p[ax];
          double d = r[ax] - a0;
          r[ax] = r[ax] - 2.0 * d;
          u[ax] = -u[ax];
        } else if (b == SG_BC_PERIODIC) {
          double d = sgn(p[3 + ax], r0);
          r[ax] = r[ax] - 2.0 * d;
        }
      }
    }
  }

  // axis-aligned bounding box (boundingBox of each surface)
  void boundingBox(double bb[6]) const {
    for (int i = 0; i < 3; ++i) { bb[i] = -INF; bb[3 + i] = INF; }
    if (type == SG_SURF_BOX) for (int i = 0; i < 3; ++i) { bb[i] = p[i] - p[3 + i]; bb[3 + i] = p[i] + p[3 + i]; }
    else if (type >= SG_SURF_XSQCYL && type <= SG_SURF_ZSQCYL) {
      int pl[2] = {plane0, plane1};
      for (int i : pl) { bb[i] = p[i] - p[3 + i]; bb[3 + i] = p[i] + p[3 + i]; }
    } else if (type == SG_SURF_SPHERE) for (int i = 0; i < 3; ++i) { bb[i] = p[i] - p[3]; bb[3 + i] = p[i] + p[3]; }
    else if (type >= SG_SURF_XCYL && type <= SG_SURF_ZCYL) {
      int pl[2] = {plane0, plane1};
      for (int i : pl) { bb[i] = p[i] - p[3]; bb[3 + i] = p[i] + p[3]; }
    }
  }
};

// ---------------------------------------------------------------- coordinates (Geometry/coord_class.f90)
struct Coord {
  double r[3] = {0, 0, 0};
  double dir[3] = {0, 0, 0};
  int uniIdx = 0, uniRootID = 0, localID = 0, cellIdx = 0;
  bool isRotated = false;                 // coord_class.f90:33-47
  double rotMat[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
};

// matmul(rotMat, v) with rotMat row-major
static void matVec(const double m[9], const double v[3], double out[3]) {
  for (int i = 0; i < 3; ++i) out[i] = m[3 * i + 0] * v[0] + m[3 * i + 1] * v[1] + m[3 * i + 2] * v[2];
}

// rotationMatrix (genericProcedures.f90:1098-1140): ZXZ Euler angles in degrees, row-major
static void rotationMatrix(double phi, double theta, double psi, double m[9]) {
  const double conv = 2.0 * 3.14159265358979323846264338327950288 / 360.0;
  const double sf = std::sin(phi * conv), cf = std::cos(phi * conv);
  const double st = std::sin(theta * conv), ct = std::cos(theta * conv);
  const double sp = std::sin(psi * conv), cp = std::cos(psi * conv);
  m[0] = cp * cf - ct * sf * sp;  m[1] = cp * sf + ct * cf * sp;   m[2] = sp * sf;
  m[3] = -sp * cf - ct * sf * cp; m[4] = -sp * sf + ct * cf * cp;  m[5] = cp * st;
  m[6] = st * sf;                 m[7] = -st * cf;                 m[8] = ct;
}

struct CoordList {
  int nesting = 0;
  Coord lvl[MAX_NEST];
  int matIdx = UNDEF_MAT;
  int uniqueID = -3;
  void init(const double r[3], const double u[3]) {   // :193-203
    takeAboveGeom();
    for (int i = 0; i < 3; ++i) { lvl[0].r[i] = r[i]; lvl[0].dir[i] = u[i]; }
    nesting = 1;
  }
  void takeAboveGeom() { nesting = 1; matIdx = UNDEF_MAT; uniqueID = -3; }   // :283-290
  int cell() const { return lvl[std::max(nesting, 1) - 1].cellIdx; }          // :419-425
  void moveGlobal(double d) {                                                  // :326-332
    takeAboveGeom();
    for (int i = 0; i < 3; ++i) lvl[0].r[i] = lvl[0].r[i] + d * lvl[0].dir[i];
  }
  void moveLocal(double d, int n) {                                            // :346-356
    nesting = n;
    for (int l = 0; l < n; ++l)
      for (int i = 0; i < 3; ++i) lvl[l].r[i] = lvl[l].r[i] + d * lvl[l].dir[i];
  }
  // the direction of levels 2..nesting from the level above (matmul by rotMat where rotated)
  void propagateDir() {
    for (int l = 1; l < nesting; ++l) {
      if (lvl[l].isRotated) matVec(lvl[l].rotMat, lvl[l - 1].dir, lvl[l].dir);
      else for (int i = 0; i < 3; ++i) lvl[l].dir[i] = lvl[l - 1].dir[i];
    }
  }
  void assignDirection(const double u[3]) {                                     // :453-472
    for (int i = 0; i < 3; ++i) lvl[0].dir[i] = u[i];
    propagateDir();
  }
  void rotate(double mu, double phi) {                                          // :385-408
    double nd[3];
    rotateVector(lvl[0].dir, mu, phi, nd);
    for (int i = 0; i < 3; ++i) lvl[0].dir[i] = nd[i];
    propagateDir();
  }
};

struct distCache {   // geometry_inter.f90:21-25
  int lvl = 0;
  double dist[MAX_NEST] = {0};
  int surf[MAX_NEST] = {0};
};

// ---------------------------------------------------------------- geometry (csg + universes + graph)
struct Universe {
  int type = 0;
  double origin[3] = {0, 0, 0};
  bool rot = false;                       // universe_inter.f90:67-68
  double rotMat[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<int> ip;
  std::vector<double> dp;
  std::vector<int> fill;
  int nLocal = 0;
  // pin
  std::vector<double> r_sq, ptol;
  // lattice
  double pitch[3], corner[3], a_bar[3];
  int sizeN[3], outLocalID = 0;
  bool offset = true;
  Surface outline;
};

struct Geometry {
  std::vector<Surface> surfs;
  std::vector<std::vector<int>> cells;   // signed 1-based surface index per cell (unionCell: its evalArray)
  std::vector<char> cellComplex;         // unionCell with unions: evaluated by insideComplex

  // unionCell operator codes inside an evaluation array (unionCell_class.f90:15-19)
  static constexpr int OP_OPEN = SG_CELL_OPEN, OP_CLOSE = SG_CELL_CLOSE, OP_UNION = SG_CELL_UNION,
                       OP_COMPLEM = SG_CELL_COMPLEMENT, OP_INTERSECT = SG_CELL_COMPLEMENT + 1;
  static bool isOp(int t) { return t >= OP_OPEN && t <= OP_INTERSECT; }

  // unionCell%init (unionCell_class.f90:80-199) with deMorgan (:202-262) and checkPrecedence (:267-305)
  static bool unionCellInit(const std::vector<int>& in, std::vector<int>& ev, bool& cx, std::string& err) {
    bool ops = false;
    for (int t : in) if (isOp(t)) ops = true;
    cx = false;
    if (!ops) { ev = in; return true; }
    std::vector<int> a;
    bool surfacePrev = false, closePrev = false;
    int depth = 0;
    for (int t : in) {
      if (isOp(t)) {
        if (t == OP_OPEN) {
          depth += 1;
          if (surfacePrev || closePrev) a.push_back(OP_INTERSECT);
          a.push_back(OP_OPEN); closePrev = false;
        } else if (t == OP_CLOSE) {
          depth -= 1; a.push_back(OP_CLOSE); closePrev = true;
        } else if (t == OP_UNION) {
          a.push_back(OP_UNION); closePrev = false;
        } else if (t == OP_COMPLEM) {
          if (surfacePrev || closePrev) a.push_back(OP_INTERSECT);
          a.push_back(OP_COMPLEM); closePrev = false;
        } else { err = "unrecognised entry in surfaces"; return false; }
        surfacePrev = false;
      } else {
        if (surfacePrev || closePrev) a.push_back(OP_INTERSECT);
        a.push_back(t); surfacePrev = true; closePrev = false;
      }
    }
    if (depth != 0) { err = "Inconsistent use of parentheses in cell definition"; return false; }
    if (a.back() == OP_UNION) { err = "Cell definition ends with a union"; return false; }
    if (a.back() == OP_COMPLEM) { err = "Cell definition ends with a complement"; return false; }
    // deMorgan: 1-based i while i < sz
    int sz = (int)a.size();
    int i = 1;
    while (i < sz) {
      if (a[i - 1] == OP_COMPLEM) {
        for (int k = i; k < sz; ++k) a[k - 1] = a[k];
        sz -= 1;
        int endPos = i;
        if (a[i - 1] == OP_OPEN) {
          int d = 1, j;
          for (j = i + 1; j <= sz; ++j) {
            if (a[j - 1] == OP_OPEN) d += 1;
            else if (a[j - 1] == OP_CLOSE) d -= 1;
            if (d == 0) break;
          }
          endPos = std::min(j, sz);
        }
        for (int j = i; j <= endPos; ++j) {
          int e = a[j - 1];
          if (!isOp(e)) a[j - 1] = -e;
          else if (e == OP_UNION) a[j - 1] = OP_INTERSECT;
          else if (e == OP_INTERSECT) a[j - 1] = OP_UNION;
        }
      }
      i += 1;
    }
    a.resize(sz);
    // checkPrecedence
    i = 1;
    while (i < sz) {
      int e1 = a[i - 1];
      bool cycled = false;
      if (e1 == OP_UNION || e1 == OP_INTERSECT) {
        for (int j = i + 1; j <= sz; ++j) {
          int e2 = a[j - 1];
          if (e2 == OP_INTERSECT || e2 == OP_UNION) {
            if (e2 != e1) { err = "The order of operations in a cell is ambiguous"; return false; }
            i = j; cycled = true; break;
          } else if (e2 == OP_OPEN || e2 == OP_CLOSE) { i = j + 1; cycled = true; break; }
        }
      }
      if (!cycled) i += 1;
    }
    for (int e : a) if (e == OP_UNION) cx = true;
    if (!cx) {
      std::vector<int> ids;
      for (int e : a) if (!isOp(e)) ids.push_back(std::abs(e));
      std::sort(ids.begin(), ids.end());
      for (size_t k = 1; k < ids.size(); ++k)
        if (ids[k] == ids[k - 1]) { err = "There are repeated surfaces in definition of cell"; return false; }
    }
    ev = a;
    return true;
  }
  std::vector<Universe> unis;
  std::vector<int> graphIdx, graphId;   // geomGraph array (1-based locations)
  std::vector<int> uniBase;             // uniRootID per universe (1-based), shrunk graph
  int rootIdx = 0;                      // 0-based
  int borderIdx = 0;                    // 0-based
  int uniqueCells = 0;

  int build(const sg_geometry_desc* g, std::string& err) {
    surfs.resize(g->n_surf);
    for (int i = 0; i < g->n_surf; ++i) surfs[i].build(g->surf_type[i], g->surf_par + SG_SURF_NPAR * i);
    borderIdx = g->border_surf;
    for (int i = 0; i < 6; ++i) surfs[borderIdx].bc[i] = g->bc[i];
    cells.resize(g->n_cell);
    cellComplex.assign(g->n_cell, 0);
    for (int c = 0; c < g->n_cell; ++c) {
      std::vector<int> in(g->cell_surf + g->cell_ptr[c], g->cell_surf + g->cell_ptr[c + 1]);
      bool cx = false;
      if (!unionCellInit(in, cells[c], cx, err)) return SG_ERR_BAD_ARG;
      cellComplex[c] = cx;
    }
    unis.resize(g->n_uni);
    for (int u = 0; u < g->n_uni; ++u) {
      Universe& U = unis[u];
      U.type = g->uni_type[u];
      for (int i = 0; i < 3; ++i) U.origin[i] = g->uni_origin[3 * u + i];
      if (g->uni_rot) {                                // universe%setTransform (:358-375)
        const double* a = g->uni_rot + 3 * u;
        if (!(a[0] == 0.0 && a[1] == 0.0 && a[2] == 0.0)) {
          if (U.type == SG_UNI_ROOT) { err = "root universe: rotation is not supported"; return SG_ERR_BAD_ARG; }
          if (!(a[0] >= 0.0 && a[0] < 360.0) || !(a[1] >= 0.0 && a[1] <= 180.0) || !(a[2] >= 0.0 && a[2] < 360.0)) {
            err = "universe rotation: angles out of range";
            return SG_ERR_BAD_ARG;
          }
          U.rot = true;
          rotationMatrix(a[0], a[1], a[2], U.rotMat);
        }
      }
      for (int k = g->uni_iptr[u]; k < g->uni_iptr[u + 1]; ++k) U.ip.push_back(g->uni_ipar[k]);
      for (int k = g->uni_dptr[u]; k < g->uni_dptr[u + 1]; ++k) U.dp.push_back(g->uni_dpar[k]);
      for (int k = g->uni_fptr[u]; k < g->uni_fptr[u + 1]; ++k) U.fill.push_back(g->uni_fill[k]);
      if (U.type == SG_UNI_ROOT) {                     // rootUniverse_class.f90:100-119
        U.fill.resize(1);
        U.fill.push_back(OUTSIDE_MAT);
        U.nLocal = 2;
      } else if (U.type == SG_UNI_CELL) {              // cellUniverse_class.f90:145-151
        U.fill.push_back(UNDEF_MAT);
        U.fill.push_back(OVERLAP_MAT);
        U.nLocal = (int)U.fill.size();
      } else if (U.type == SG_UNI_PIN) {               // pinUniverse_class.f90:76-139
        int N = (int)U.dp.size() + 1;
        std::vector<double> radii(U.dp);
        radii.push_back(INF * 1.1);
        for (int i = 0; i < N; ++i) { U.r_sq.push_back(radii[i] * radii[i]); U.ptol.push_back(2.0 * radii[i] * SURF_TOL); }
        U.nLocal = N;
        if ((int)U.fill.size() != N) { err = "pin universe fills mismatch"; return -1; }
      } else if (U.type == SG_UNI_LAT) {               // latUniverse_class.f90:113-260
        for (int i = 0; i < 3; ++i) { U.pitch[i] = U.dp[i]; U.sizeN[i] = U.ip[i]; }
        U.offset = U.ip.size() > 3 ? U.ip[3] != 0 : true;
        if (U.sizeN[2] == 0) { U.sizeN[2] = 1; U.pitch[2] = 2.0 * INF; }
        for (int i = 0; i < 3; ++i) {
          U.a_bar[i] = U.pitch[i] * 0.5 - U.pitch[i] * SURF_TOL;
          U.corner[i] = -(U.sizeN[i] * 0.5 * U.pitch[i]);
        }
        U.outLocalID = U.sizeN[0] * U.sizeN[1] * U.sizeN[2] + 1;
        double ob[SG_SURF_NPAR] = {0, 0, 0, std::fabs(U.corner[0]), std::fabs(U.corner[1]), std::fabs(U.corner[2])};
        U.outline.build(SG_SURF_BOX, ob);
        U.nLocal = U.outLocalID;
        if ((int)U.fill.size() != U.nLocal) { err = "lattice fills mismatch"; return -1; }
      }
    }
    rootIdx = g->root_uni;
    // shrunk geomGraph (geomGraph_class.f90:172-232): BFS layout from root, then enumerate sinks
    uniBase.assign(unis.size(), -1);
    int top = 1;
    auto layout = [&](int u) {
      uniBase[u] = top;
      for (int f : unis[u].fill) { graphIdx.push_back(f); graphId.push_back(0); }
      top += (int)unis[u].fill.size();
    };
    layout(rootIdx);
    for (size_t loc = 0; loc < graphIdx.size(); ++loc) {
      int f = graphIdx[loc];
      if (f < 0) {
        int u = -f - 1;
        if (u < 0 || u >= (int)unis.size()) { err = "bad universe fill"; return -1; }
        if (uniBase[u] < 0) layout(u);
        graphId[loc] = uniBase[u];
      }
    }
    int cellsN = 0;                                 // setUniqueIDs (:309-345)
    for (size_t i = 0; i < graphIdx.size(); ++i) if (graphIdx[i] > 0) graphId[i] = ++cellsN;
    uniqueCells = cellsN;
    return 0;
  }

  // universe%enter (universe_inter.f90:400-424) with findCell
  void enter(int u, Coord& nw, const double r[3], const double dir[3]) {
    Universe& U = unis[u];
    for (int i = 0; i < 3; ++i) { nw.r[i] = r[i]; nw.dir[i] = dir[i]; }
    nw.uniIdx = u + 1;
    nw.isRotated = U.rot;
    if (U.rot) {
      for (int i = 0; i < 9; ++i) nw.rotMat[i] = U.rotMat[i];
      matVec(U.rotMat, r, nw.r);
      matVec(U.rotMat, dir, nw.dir);
    }
    for (int i = 0; i < 3; ++i) nw.r[i] = nw.r[i] - U.origin[i];
    findCell(u, nw.localID, nw.cellIdx, nw.r, nw.dir);
  }

  void findCell(int u, int& localID, int& cellIdx, const double r[3], const double dir[3]) {
    Universe& U = unis[u];
    cellIdx = 0;
    switch (U.type) {
      case SG_UNI_ROOT:                                 // rootUniverse_class.f90:127-145
        localID = surfs[U.ip[0]].halfspace(r, dir) ? 2 : 1;
        return;
      case SG_UNI_CELL: {                               // cellUniverse_class.f90:203-246 (fixed order)
        int nc = (int)U.ip.size();
        for (int i = 0; i < nc; ++i) {
          if (cellInside(U.ip[i], r, dir)) { localID = i + 1; cellIdx = U.ip[i] + 1; return; }
        }
        localID = nc + 1;
        return;
      }
      case SG_UNI_PIN: {                                // pinUniverse_class.f90:150-173
        double rsq = r[0] * r[0] + r[1] * r[1];
        double mul = (r[0] * dir[0] + r[1] * dir[1] >= 0.0) ? -1.0 : 1.0;
        int N = (int)U.r_sq.size();
        for (localID = 1; localID <= N; ++localID)
          if (rsq < U.r_sq[localID - 1] + mul * U.ptol[localID - 1]) return;
        return;   // localID = N + 1
      }
      case SG_UNI_LAT: {                                // latUniverse_class.f90:270-312
        int ijk[3];
        for (int i = 0; i < 3; ++i) ijk[i] = (int)std::floor((r[i] - U.corner[i]) / U.pitch[i]) + 1;
        for (int i = 0; i < 3; ++i) {
          double r_bar = r[i] - U.corner[i] - ijk[i] * U.pitch[i] + 0.5 * U.pitch[i];
          if (std::fabs(r_bar) > U.a_bar[i] && r_bar * dir[i] > 0.0) ijk[i] += (dir[i] < 0.0) ? -1 : 1;
        }
        bool out = false;
        for (int i = 0; i < 3; ++i) if (ijk[i] <= 0 || ijk[i] > U.sizeN[i]) out = true;
        localID = out ? U.outLocalID : ijk[0] + U.sizeN[0] * (ijk[1] - 1 + U.sizeN[1] * (ijk[2] - 1));
        return;
      }
    }
  }

  bool cellInside(int c, const double r[3], const double u[3]) {    // simpleCell_class.f90:90-111
    if (cellComplex[c]) return insideComplex(c, r, u);
    bool isIt = false;
    for (int s : cells[c]) {
      if (isOp(s)) continue;                                          // unionCell%inside, isSimple
      bool sense = s > 0;
      bool hs = surfs[std::abs(s) - 1].halfspace(r, u);
      isIt = (hs == sense);
      if (!isIt) return false;
    }
    return isIt;
  }

  bool insideComplex(int c, const double r[3], const double u[3]) {  // unionCell_class.f90:365-422
    const std::vector<int>& a = cells[c];
    bool isIt = true;
    int depth = 0;
    int n = (int)a.size();
    for (int i = 1; i <= n; ++i) {
      int el = a[i - 1];
      if (!isOp(el)) {
        bool sense = el > 0;
        bool hs = surfs[std::abs(el) - 1].halfspace(r, u);
        isIt = (hs == sense);
      } else if ((el == OP_UNION && isIt) || (el == OP_INTERSECT && !isIt)) {
        if (depth == 0) return isIt;
        depth -= 1;
        int d = 1;                                                    // shortCircuit
        while (d > 0) {
          i += 1;
          int e2 = a[i - 1];
          if (e2 == OP_OPEN) d += 1;
          else if (e2 == OP_CLOSE) d -= 1;
        }
      } else if (el == OP_OPEN) depth += 1;
      else if (el == OP_CLOSE) depth -= 1;
    }
    return isIt;
  }

  static void get_ijk(int localID, const int sizeN[3], int ijk[3]) {  // latUniverse_class.f90:489-506
    int temp = localID - 1;
    int base = temp / sizeN[0];
    ijk[0] = temp - sizeN[0] * base + 1;
    temp = base;
    base = temp / sizeN[1];
    ijk[1] = temp - sizeN[1] * base + 1;
    ijk[2] = base + 1;
  }

  void uniDistance(int u, double& d, int& surfIdx, const Coord& c) {
    Universe& U = unis[u];
    switch (U.type) {
      case SG_UNI_ROOT:                                  // rootUniverse_class.f90:152-162
        surfIdx = U.ip[0] + 1;
        d = surfs[U.ip[0]].distance(c.r, c.dir);
        return;
      case SG_UNI_CELL: {                                // cellUniverse_class.f90:343-362, simpleCell :120-141
        int cidx = U.ip[c.localID - 1];
        d = INF; surfIdx = 0;
        for (int s : cells[cidx]) {
          if (isOp(s)) continue;
          double td = surfs[std::abs(s) - 1].distance(c.r, c.dir);
          if (td < d) { d = td; surfIdx = std::abs(s); }
        }
        return;
      }
      case SG_UNI_PIN: {                                 // pinUniverse_class.f90:185-226
        int id = c.localID, N = (int)U.r_sq.size();
        double d_out, d_in;
        if (id > N) d_out = INF;
        else d_out = pinCylDist(U, id - 1, c.r, c.dir);
        if (id == 1) d_in = INF;
        else d_in = pinCylDist(U, id - 2, c.r, c.dir);
        if (d_in < d_out) { surfIdx = -1; d = d_in; } else { surfIdx = -2; d = d_out; }
        return;
      }
      case SG_UNI_LAT: {                                 // latUniverse_class.f90:319-373
        if (c.localID == U.outLocalID) { surfIdx = -7; d = U.outline.distance(c.r, c.dir); return; }
        int ijk[3]; get_ijk(c.localID, U.sizeN, ijk);
        double r_bar[3], bounds[3];
        for (int i = 0; i < 3; ++i) {
          r_bar[i] = c.r[i] - U.corner[i];
          r_bar[i] = r_bar[i] - (ijk[i] - 0.5) * U.pitch[i];
          bounds[i] = sgn(U.pitch[i] * 0.5, c.dir[i]);
        }
        d = INF; int ax = 0;
        for (int i = 0; i < 3; ++i) {
          double td = (bounds[i] - r_bar[i]) / c.dir[i];
          if (td < d) { d = td; ax = i; }
        }
        d = std::max(0.0, d);
        d = std::min(INF, d);
        int s = (ax + 1) * 2;
        if (c.dir[ax] < 0.0) s -= 1;
        surfIdx = -s;
        return;
      }
    }
  }

  double pinCylDist(const Universe& U, int k, const double r[3], const double u[3]) {
    // annulus k is a zCylinder at the origin with r_sq and surfTol = 2 r SURF_TOL
    double c = (r[0] * r[0] + r[1] * r[1]) - U.r_sq[k];
    double kk = r[0] * u[0] + r[1] * u[1];
    double a = 1.0 - u[2] * u[2];
    double delta = kk * kk - a * c, d;
    if (delta < 0.0 || a == 0.0) d = INF;
    else if (std::fabs(c) < U.ptol[k]) {
      if (kk >= 0.0) d = INF;
      else { d = -kk + std::sqrt(delta); d = d / a; }
    } else if (c < 0.0) { d = -kk + std::sqrt(delta); d = d / a; }
    else { d = -kk - std::sqrt(delta); d = d / a; if (d <= 0.0) d = INF; }
    return std::min(d, INF);
  }

  void cross(int u, Coord& c, int surfIdx) {
    Universe& U = unis[u];
    switch (U.type) {
      case SG_UNI_ROOT: findCell(u, c.localID, c.cellIdx, c.r, c.dir); return;   // rootUniverse :170-178
      case SG_UNI_CELL:                                                             // cellUniverse :388-431
        for (int i = 0; i < 3; ++i) c.r[i] = c.r[i] + c.dir[i] * NUDGE;
        findCell(u, c.localID, c.cellIdx, c.r, c.dir);
        return;
      case SG_UNI_PIN:                                                              // pinUniverse :236-253
        if (surfIdx == -1) c.localID -= 1; else c.localID += 1;
        return;
      case SG_UNI_LAT: findCell(u, c.localID, c.cellIdx, c.r, c.dir); return;      // latUniverse :380-387
    }
  }

  void cellOffset(int u, const Coord& c, double off[3]) {
    Universe& U = unis[u];
    off[0] = off[1] = off[2] = 0.0;
    if (U.type == SG_UNI_LAT && U.offset && c.localID != U.outLocalID) {         // latUniverse :394-414
      int ijk[3]; get_ijk(c.localID, U.sizeN, ijk);
      for (int i = 0; i < 3; ++i) off[i] = (ijk[i] - 0.5) * U.pitch[i] + U.corner[i];
    }
  }

  // geometryStd%diveToMat (geometryStd_class.f90:565-619)
  bool diveToMat(CoordList& co, int start) {
    for (int i = start; i <= MAX_NEST; ++i) {
      Coord& L = co.lvl[i - 1];
      int loc = L.uniRootID + L.localID - 1;
      int fill = graphIdx[loc - 1], id = graphId[loc - 1];
      if (fill >= 0) { co.matIdx = fill; co.uniqueID = id; return true; }
      if (i == MAX_NEST) break;
      int nu = -fill - 1;
      double off[3]; cellOffset(L.uniIdx - 1, L, off);
      double r[3];
      for (int k = 0; k < 3; ++k) r[k] = L.r[k] - off[k];
      co.nesting += 1;
      enter(nu, co.lvl[i], r, L.dir);
      co.lvl[i].uniRootID = id;
    }
    return false;
  }

  // geometryStd%placeCoord (:119-147)
  void placeCoord(CoordList& co) {
    co.takeAboveGeom();
    double r[3], dir[3];
    for (int i = 0; i < 3; ++i) { r[i] = co.lvl[0].r[i]; dir[i] = co.lvl[0].dir[i]; }
    enter(rootIdx, co.lvl[0], r, dir);
    co.lvl[0].uniRootID = 1;
    diveToMat(co, 1);
  }

  void whatIsAt(int& matIdx, int& uniqueID, const double r[3], const double u[3]) {  // :152-180
    CoordList co; co.init(r, u); placeCoord(co);
    matIdx = co.matIdx; uniqueID = co.uniqueID;
  }

  void bounds(double bb[6]) {   // :186-205
    surfs[borderIdx].boundingBox(bb);
    for (int i = 0; i < 3; ++i)
      if (bb[i] <= -INF && bb[i + 3] >= INF) { bb[i] = 0.0; bb[i + 3] = 0.0; }
  }

  // closestDist / closestDist_cache (:633-717)
  void closestDist(double& dist, int& surfIdx, int& lvl, const CoordList& co) {
    dist = INF; surfIdx = 0; lvl = 0;
    for (int l = 1; l <= co.nesting; ++l) {
      double td; int ti;
      uniDistance(co.lvl[l - 1].uniIdx - 1, td, ti, co.lvl[l - 1]);
      if ((dist - td) >= dist * FP_REL_TOL) { dist = td; surfIdx = ti; lvl = l; }
    }
  }
  void closestDist_cache(double& dist, int& surfIdx, int& lvl, const CoordList& co, distCache& cache) {
    dist = INF; surfIdx = 0; lvl = 0;
    for (int l = 1; l <= co.nesting; ++l) {
      if (cache.lvl < l) {
        uniDistance(co.lvl[l - 1].uniIdx - 1, cache.dist[l - 1], cache.surf[l - 1], co.lvl[l - 1]);
        cache.lvl += 1;
      }
      double td = cache.dist[l - 1]; int ti = cache.surf[l - 1];
      if ((dist - td) >= dist * FP_REL_TOL) { dist = td; surfIdx = ti; lvl = l; }
    }
  }

  // move_noCache (:214-272) / move_withCache (:285-352); no fields: fieldDist = INF
  void move(CoordList& co, double& maxDist, int& event, distCache* cache) {
    double dist; int surfIdx, level;
    if (cache) closestDist_cache(dist, surfIdx, level, co, *cache);
    else closestDist(dist, surfIdx, level, co);
    if (maxDist < dist) {
      co.moveLocal(maxDist, co.nesting);
      event = COLL_EV;
      if (cache) cache->lvl = 0;
    } else if (surfIdx == borderIdx + 1 && level == 1) {
      co.moveGlobal(dist);
      event = BOUNDARY_EV;
      maxDist = dist;
      if (cache) cache->lvl = 0;
      surfs[borderIdx].explicitBC(co.lvl[0].r, co.lvl[0].dir);
      placeCoord(co);
    } else {
      co.moveLocal(dist, level);
      event = CROSS_EV;
      maxDist = dist;
      if (cache) {
        for (int l = 0; l < level - 1; ++l) cache->dist[l] = cache->dist[l] - dist;
        cache->lvl = level - 1;
      }
      cross(co.lvl[level - 1].uniIdx - 1, co.lvl[level - 1], surfIdx);
      diveToMat(co, level);
    }
  }

  // geometryStd%moveGlobal (:355-392)
  void moveGlobalGeom(CoordList& co, double& maxDist, int& event) {
    const Surface& s = surfs[borderIdx];
    double dist = s.distance(co.lvl[0].r, co.lvl[0].dir);
    if (maxDist < dist) { co.moveGlobal(maxDist); event = COLL_EV; }
    else { co.moveGlobal(dist); event = BOUNDARY_EV; s.explicitBC(co.lvl[0].r, co.lvl[0].dir); maxDist = dist; }
    placeCoord(co);
  }

  // teleport (:492-514)
  void teleport(CoordList& co, double dist) {
    co.moveGlobal(dist);
    placeCoord(co);
    if (co.matIdx == OUTSIDE_MAT) {
      surfs[borderIdx].transformBC(co.lvl[0].r, co.lvl[0].dir);
      placeCoord(co);
    }
  }
};

// ---------------------------------------------------------------- MG data
// baseMgNeutronMaterial_class.f90:158-291, multiScatterMG_class.f90:199-336, fissionMG_class.f90:183-274
struct MGData {
  int nMat = 0, nG = 0;
  std::vector<double> total, scatter, capture, fission, nuFission, chi, P0, prod;  // [m][g], P0/prod [m][gin][gout]
  std::vector<double> P1;                              // multiScatterP1MG: 3 P1/P0 [m][gin][gout]; empty for P0
  std::vector<int> fissile;
  std::vector<double> majorant;
  double collisionXS = 0.0;

  int build(const sg_mg_desc* d, std::string& err) {
    nMat = d->n_mat; nG = d->n_g;
    size_t M = (size_t)nMat * nG;
    total.assign(M, 0); scatter.assign(M, 0); capture.assign(M, 0); fission.assign(M, 0);
    nuFission.assign(M, 0); chi.assign(M, 0);
    P0.assign(M * nG, 0); prod.assign(M * nG, 0); fissile.assign(nMat, 0);
    for (int m = 0; m < nMat; ++m) {
      fissile[m] = d->fissile[m];
      for (int gi = 0; gi < nG; ++gi)
        for (int go = 0; go < nG; ++go) {
          size_t k = ((size_t)m * nG + gi) * nG + go;
          P0[k] = d->p0[k]; prod[k] = d->prod[k];
        }
      for (int g = 0; g < nG; ++g) {
        size_t k = (size_t)m * nG + g;
        double s = 0.0;                                   // scatterXSs = sum(P0, 1)
        for (int go = 0; go < nG; ++go) s = s + P0[((size_t)m * nG + g) * nG + go];
        scatter[k] = s;
        capture[k] = d->capture[k];
        if (fissile[m]) { fission[k] = d->fission[k]; nuFission[k] = d->nu[k] * d->fission[k]; }
        total[k] = scatter[k] + capture[k];
        if (fissile[m]) total[k] = total[k] + fission[k];
      }
      if (fissile[m]) {                                   // fissionMG buildFromDict chi normalisation
        double S = 0.0;
        for (int g = 0; g < nG; ++g) S = S + d->chi[(size_t)m * nG + g];
        for (int g = 0; g < nG; ++g) {
          double c = d->chi[(size_t)m * nG + g];
          if (std::fabs(S - 1.0) > 0.01 * FP_REL_TOL) c = c / S;
          chi[(size_t)m * nG + g] = c;
        }
      }
    }
    if (d->avg_dist > 0.0) collisionXS = 1.0 / d->avg_dist;
    P1.clear();
    if (d->p1) {                                         // multiScatterP1MG buildFromDict (:117-126)
      P1.assign(M * nG, 0.0);
      for (size_t k = 0; k < M * nG; ++k)
        if (P0[k] != 0.0) P1[k] = d->p1[k] / P0[k] * 3.0;
    }
    (void)err;
    return 0;
  }
  void initMajorant(const std::vector<int>& activeMats) {   // baseMgNeutronDatabase_class.f90:458-503
    majorant.assign(nG, 0.0);
    for (int g = 0; g < nG; ++g) {
      double xs = 0.0;
      for (int m : activeMats) xs = std::max(xs, total[(size_t)(m - 1) * nG + g]);
      majorant[g] = xs * 1.0;
    }
  }
  double T(int m, int g) const { return total[(size_t)(m - 1) * nG + (g - 1)]; }
};

// ---------------------------------------------------------------- continuous-energy data
// genericProcedures.f90:132-166 binaryFloorIdxClosed_Real: 1-based floor index of v in a(1:N);
// v == a(N) gives N-1; <= 0 when v is outside [a(1), a(N)] or the search does not end in 70 steps.
static int binaryFloorIdx(const double* a, int N, double v) {
  int bottom = 1, top = N;
  if (v < a[bottom - 1] || v > a[top - 1]) return -1;
  for (int i = 1; i <= 70; ++i) {
    int idx = (top + bottom) / 2;
    if (bottom == idx) return idx;
    if (a[idx - 1] <= v) bottom = idx;
    else top = idx;
  }
  return -2;
}

static const double neutronMass = 939.56542194;     // universalVariables.f90:90
static const double lightSpeed = 2.99792458e10;     // universalVariables.f90:91
static const double SQRT_PI = std::sqrt(PI);        // numPrecision.f90:24
static const double MAJ_NUDGE = 1.0e-06;            // aceNeutronDatabase_class.f90:1345

// aceNeutronNuclide (aceNeutronNuclide_class.f90:44-51,116): eGrid and mainData(TOTAL, ESCATTER,
// IESCATTER, CAPTURE) of a non-fissile nuclide
struct CENuclide {
  std::vector<double> e;
  std::vector<double> d;   // [N][4]
  int N = 0;
  double A = 1.0, kT = 0.0;
  // search (:342-359): floor index (1-based) and interpolation factor
  bool search(double E, int& idx, double& f) const {
    idx = binaryFloorIdx(e.data(), N, E);
    if (idx <= 0) return false;
    double E_top = e[idx], E_low = e[idx - 1];
    f = (E - E_low) / (E_top - E_low);
    return true;
  }
  // totalXS / microXSs (:374-453): xs(idx+1)*f + (1-f)*xs(idx)
  double interp(int idx, double f, int k) const { return d[(size_t)idx * 4 + k] * f + (1.0 - f) * d[(size_t)(idx - 1) * 4 + k]; }
};

struct CEMaterial {
  std::vector<int> nuc;      // 0-based
  std::vector<double> dens;
};

struct CEData {
  std::vector<CENuclide> nucs;
  std::vector<CEMaterial> mats;
  double eBounds[2] = {0, 0};
  bool hasMajorant = true;
  std::vector<double> eGridUnion, majorant;
  std::vector<int> activeMat;   // 1-based
  double minE = 1.0e-11, maxE = 20.0, threshE = 400.0, threshA = 1.0, collisionXS = 0.0;

  int build(const sg_ce_desc* d, std::string& err) {
    nucs.assign(d->n_nuc, CENuclide());
    for (int i = 0; i < d->n_nuc; ++i) {
      CENuclide& n = nucs[i];
      int64_t a = d->nuc_ptr[i], b = d->nuc_ptr[i + 1];
      n.N = (int)(b - a);
      if (n.N < 2) { err = "nuclide grid needs >= 2 points"; return -1; }
      n.e.assign(d->e + a, d->e + b);
      n.d.assign(d->xs + 4 * a, d->xs + 4 * b);
      n.A = d->A[i]; n.kT = d->kT[i];
    }
    mats.assign(d->n_mat, CEMaterial());
    for (int m = 0; m < d->n_mat; ++m)
      for (int k = d->mat_ptr[m]; k < d->mat_ptr[m + 1]; ++k) {
        mats[m].nuc.push_back(d->mat_nuc[k]);
        mats[m].dens.push_back(d->mat_dens[k]);
      }
    // energy bounds over all nuclides (aceNeutronDatabase_class.f90:1043-1052)
    eBounds[0] = nucs[0].e[0]; eBounds[1] = nucs[0].e[nucs[0].N - 1];
    for (size_t i = 1; i < nucs.size(); ++i) {
      eBounds[0] = std::max(eBounds[0], nucs[i].e[0]);
      eBounds[1] = std::min(eBounds[1], nucs[i].e[nucs[i].N - 1]);
    }
    hasMajorant = d->majorant != 0;
    minE = d->min_e; maxE = d->max_e; threshE = d->thresh_e; threshA = d->thresh_a;
    collisionXS = d->avg_dist > 0.0 ? 1.0 / d->avg_dist : 0.0;
    return 0;
  }

  // updateTotalNucXS (aceNeutronDatabase_class.f90:702-727) without URR / S(a,b)
  bool nucTotal(int n, double E, double& xs) const {
    int idx; double f;
    if (!nucs[n].search(E, idx, f)) return false;
    xs = nucs[n].interp(idx, f, 0);
    return true;
  }
  // updateTotalMatXS (:517-570): sum over the composition in order, times densityFactor 1
  bool matTotal(int m, double E, double& total) const {
    const CEMaterial& M = mats[m - 1];
    total = 0.0;
    for (size_t i = 0; i < M.nuc.size(); ++i) {
      double s;
      if (!nucTotal(M.nuc[i], E, s)) return false;
      total = total + M.dens[i] * s;
    }
    total = total * 1.0;
    return true;
  }
  // updateMajorantXS (:346-394)
  bool majorantXS(double E, double& xs) const {
    if (hasMajorant) {
      int idx = binaryFloorIdx(eGridUnion.data(), (int)eGridUnion.size(), E);
      if (idx <= 0) return false;
      double E_top = eGridUnion[idx], E_low = eGridUnion[idx - 1];
      double f = (E - E_low) / (E_top - E_low);
      xs = majorant[idx] * f + (1.0 - f) * majorant[idx - 1];
      return true;
    }
    xs = 0.0;
    for (int m : activeMat) {
      double t;
      if (!matTotal(m, E, t)) return false;
      xs = std::max(xs, t);
    }
    return true;
  }
  // initMajorant (:1330-1621) without URR / S(a,b) / TMS.  The merge loop adds each nuclide's grid
  // points in ascending order until its first point outside eBounds (that nuclide then stops
  // contributing); the temporary grid starts filled with eBounds(2); duplicates are removed.
  void initMajorant(const std::vector<int>& act) {
    activeMat = act;
    std::vector<int> nucSet;
    for (int m : act) for (int n : mats[m - 1].nuc)
      if (std::find(nucSet.begin(), nucSet.end(), n) == nucSet.end()) nucSet.push_back(n);
    std::vector<double> g;
    for (int n : nucSet) {
      const CENuclide& N = nucs[n];
      for (int i = 0; i < N.N; ++i) {
        if (N.e[i] < eBounds[0] || N.e[i] > eBounds[1]) break;
        g.push_back(N.e[i]);
      }
    }
    g.push_back(eBounds[1]);
    std::sort(g.begin(), g.end());
    eGridUnion.clear();
    for (double x : g) if (eGridUnion.empty() || x != eGridUnion.back()) eGridUnion.push_back(x);
    majorant.assign(eGridUnion.size(), 0.0);
    for (size_t i = 0; i < eGridUnion.size(); ++i) {
      double E = eGridUnion[i];
      if (E < eBounds[0]) E = eBounds[0];
      if (E > eBounds[1]) E = eBounds[1];
      double maj = 0.0;
      for (int m : act) {
        double t = 0.0;
        matTotal(m, E, t);
        t = t * 1.0;                                     // rho = densityFactor = 1
        maj = std::max(maj, t);
      }
      majorant[i] = maj * (1.0 + MAJ_NUDGE);
    }
  }
};

// scatteringKernels_func.f90:281-334 (Gamma(3/2) and Gamma(2) samples of X)
template <class RNGT>
static double sample_x2expx2(RNGT& rand) {
  double r1 = rand.get(), r2 = rand.get(), r3 = rand.get();
  double cosine = std::cos(0.5 * PI * r1);
  double beta = cosine * cosine;
  double gamma05 = -std::log(r2) * beta;
  double sample = -std::log(r3) + gamma05;
  return std::sqrt(sample);
}
template <class RNGT>
static double sample_x3expx2(RNGT& rand) {
  double r1 = rand.get(), r2 = rand.get();
  double sample = -std::log(r1) - std::log(r2);
  return std::sqrt(sample);
}
// targetVelocity_constXS + sample_targetVelocity (scatteringKernels_func.f90:101-139,340-380)
template <class RNGT>
static void targetVelocity_constXS(double E, const double dir[3], double A, double kT, RNGT& rand, double V_t[3]) {
  double Y = std::sqrt(A * E / kT);
  double alpha = 2.0 / (Y * SQRT_PI + 2.0);
  double X, mu;
  while (true) {
    double r1 = rand.get(), r2 = rand.get(), r3 = rand.get();
    if (r1 > alpha) X = sample_x2expx2(rand);
    else X = sample_x3expx2(rand);
    mu = 2.0 * r2 - 1.0;
    double rel_v = std::sqrt(Y * Y + X * X - 2.0 * X * Y * mu);
    double P_acc = rel_v / (Y + X);
    if (P_acc > r3) break;
  }
  double r1 = rand.get();
  double phi = 2.0 * PI * r1;
  rotateVector(dir, mu, phi, V_t);
  double s = X * std::sqrt(kT / A);
  for (int i = 0; i < 3; ++i) V_t[i] = V_t[i] * s;
}
// asymptoticScatter (scatteringKernels_func.f90:38-58)
static void asymptoticScatter(double& E, double& mu, double A) {
  double E_in = E;
  double inv_Ap1 = 1.0 / (A + 1.0);
  E = (1.0 + A * A + 2 * A * mu) * E_in * inv_Ap1 * inv_Ap1;
  mu = (A * mu + 1) * std::sqrt(E_in / E) * inv_Ap1;
  if (mu > 1.0) mu = 1.0;
}

// ---------------------------------------------------------------- scoreMemory (Tallies/scoreMemory_class.f90)
struct ScoreMemory {
  std::vector<double> bin, csum, csum2;
  std::vector<double> parallel;   // accumulating scores of the running batch
  int64_t N = 0;
  int batchN = 0, cycles = 0, batchSize = 1;
  void init(int64_t n, int bs) {
    N = n; bin.assign(n, 0); csum.assign(n, 0); csum2.assign(n, 0); parallel.assign(n, 0);
    batchN = 0; cycles = 0; batchSize = bs > 0 ? bs : 1;
  }
  void score(double s, int64_t idx) { parallel[idx - 1] += s; }          // :215-233
  void accumulate(double s, int64_t idx) {                                // :255-270
    csum[idx - 1] = csum[idx - 1] + s; csum2[idx - 1] = csum2[idx - 1] + s * s;
  }
  bool lastCycle() const { return (cycles + 1) % batchSize == 0; }       // :377-381
  void reduceBins() {                                                     // :403-432
    if (lastCycle()) for (int64_t i = 0; i < N; ++i) { bin[i] = parallel[i]; parallel[i] = 0.0; }
  }
  void closeCycle(double normFactor) {                                    // :319-345
    cycles += 1;
    if (cycles % batchSize == 0) {
      for (int64_t i = 0; i < N; ++i) {
        double res = bin[i] * normFactor;
        bin[i] = 0.0;
        csum[i] = csum[i] + res;
        csum2[i] = csum2[i] + res * res;
      }
      batchN += 1;
    }
  }
  void closeBin(double normFactor, int64_t idx) {                          // :356-375
    double res = bin[idx - 1] * normFactor;
    csum[idx - 1] = csum[idx - 1] + res;
    csum2[idx - 1] = csum2[idx - 1] + res * res;
    bin[idx - 1] = 0.0;
  }
  double getScore(int64_t idx) const { return (idx <= 0 || idx > N) ? 0.0 : bin[idx - 1]; }  // :597-608
  void getResult(double& mean, double& STD, int64_t idx, int samples = -1) const {          // :537-573
    if (idx < 1 || idx > N) { mean = 0.0; STD = 0.0; return; }
    int n = samples > 0 ? samples : batchN;
    mean = csum[idx - 1] / n;
    double inv_N = 1.0 / n;
    double inv_Nm1 = (n != 1) ? 1.0 / (n - 1) : 1.0;
    STD = csum2[idx - 1] * inv_N * inv_Nm1 - mean * mean * inv_Nm1;
    STD = std::sqrt(STD);
  }
};

// ---------------------------------------------------------------- particle (ParticleObjects/particle_class.f90)
struct PState {   // particleState subset carried by the banks
  double wgt = 0, r[3] = {0, 0, 0}, dir[3] = {0, 0, 0}, time = 0, E = 0;
  int G = 0, broodID = 0, matIdx = -1;
};

struct Particle {
  CoordList coords;
  int G = 1;
  double E = 0.0;         // CE energy [MeV]
  bool isMG = true;
  double w = 1.0, w0 = 1.0, time = 0.0;
  bool isDead = false;
  int fate = NO_FATE;
  int collisionN = 0, broodID = 0;
  int splitCount = 0;                     // particle_class.f90:137
  std::vector<PState> buffer;             // the gen loop's `buffer`: split particles, LIFO
  double k_eff = 1.0;
  RNG rng;
  double preHistWgt = 1.0, preCollWgt = 1.0;
  // prePath snapshot used by track clerks
  double prePathR[3] = {0, 0, 0};
  int prePathMat = 0, prePathG = 1, prePathCell = 0;
  double prePathE = 0.0;
  int matIdx() const { return coords.matIdx; }
};

// ---------------------------------------------------------------- tallies
struct Clerk {
  sg_clerk_desc d;
  int64_t addr = 1;   // 1-based memory address
  int width = 1;
  int64_t nbins = 1;
  int64_t multi[3] = {1, 1, 1};
  double step[3] = {0, 0, 0};
  int grid[3] = {0, 0, 0};                // SG_GRID_LIN / LOG / UNSTRUCT
  std::vector<double> bounds[3];          // unstructured grid bounds
  std::vector<int> cellBin[3];            // cellMap: bin of every 1-based cell index ([0]: no cell)
  int64_t size() const {
    if (d.type == SG_CLERK_KEFF_ANALOG) return 3;
    if (d.type == SG_CLERK_KEFF_IMPLICIT) return 5;
    if (d.type == SG_CLERK_SURFACE_CURRENT) return (int64_t)d.n_planes * nbins * 2;
    return (int64_t)width * nbins;
  }
};

struct TallyAdmin {
  std::vector<Clerk> clerks;
  ScoreMemory mem;
  int atch = -1;
  int64_t normAddr = -1;
  double normVal = 1.0;
};

struct Oracle {
  Geometry geom;
  MGData mg;
  CEData ce;
  bool isCE = false;
  std::vector<TallyAdmin> admins;
  int transport = SG_TRANSPORT_ST;
  double htCutoff = 0.9;                             // transportOperatorHT `cutoff` (:297)
  // neutronMGimp / neutronCEimp (SG_COLL_IMP) options and the weight-window field
  bool collImp = false;
  sg_collision_desc coll{};
  Clerk wwMap;
  std::vector<double> wwLo, wwUp;
  std::string err;
  sg_point_source_desc src{};
  std::vector<double> srcProbG;
  bool hasSource = false;
  // per-history records of the last gen loop
  std::vector<int32_t> recColl;
  std::vector<uint64_t> recRng;
  // eigen state
  std::vector<PState> thisCycle;
  RNG master;
  double k_new = 1.0, keff0 = 1.0;
  int pop = 0;
  double nextK = 1.0;   // k_eff attached to the next-cycle dungeon
  // probe coords for geometry unit tests
  CoordList probe;
  distCache probeCache;
  int64_t nEvents = 0, nColl = 0;

  // ----- clerk evaluation helpers (Tallies/TallyMaps, TallyFilters, TallyResponses)
  // binaryFloorIdxClosed_Real (genericProcedures.f90:132-166): 1-based floor index, 0 outside
  static int binaryFloor(const std::vector<double>& a, double v) {
    int bottom = 1, top = (int)a.size();
    if (v < a[bottom - 1] || v > a[top - 1]) return 0;
    for (int i = 0; i < 70; ++i) {
      int idx = (top + bottom) / 2;
      if (bottom == idx) return idx;
      if (a[idx - 1] <= v) bottom = idx;
      else top = idx;
    }
    return 0;
  }
  // grid%search (grid_class.f90:154-175)
  static int gridSearch(const Clerk& c, int a, double v) {
    const sg_axis_desc& ax = c.d.axes[a];
    int idx;
    if (c.grid[a] == SG_GRID_UNSTRUCT) idx = binaryFloor(c.bounds[a], v);
    else if (c.grid[a] == SG_GRID_LOG) idx = (int)std::floor(std::log(v / ax.min) / c.step[a]) + 1;
    else idx = (int)std::floor((v - ax.min) / c.step[a]) + 1;
    if (idx < 1 || idx >= ax.n + 1) idx = 0;
    return idx;
  }
  int mapState(const Clerk& c, const double r[3], int G, int mat, int cell, double E = 0.0, bool isMG = true) const {
    if (c.d.n_axes == 0) return 1;
    int64_t idx = 1;
    for (int a = 0; a < c.d.n_axes; ++a) {
      const sg_axis_desc& ax = c.d.axes[a];
      int b = 0;
      if (ax.kind >= SG_AXIS_X && ax.kind <= SG_AXIS_Z) {        // spaceMap (spaceMap_class.f90:211-221)
        b = gridSearch(c, a, r[ax.kind - SG_AXIS_X]);
      } else if (ax.kind == SG_AXIS_GROUP) {
        b = (G >= 1 && G <= ax.n) ? G : 0;
      } else if (ax.kind == SG_AXIS_MATERIAL) {
        b = (mat >= 1 && mat <= ax.n) ? mat : 0;
      } else if (ax.kind == SG_AXIS_ENERGY) {                     // energyMap (energyMap_class.f90:278-293)
        b = isMG ? 0 : gridSearch(c, a, E);
      } else if (ax.kind == SG_AXIS_CELL) {                       // cellMap (cellMap_class.f90:198-205)
        b = c.cellBin[a][cell];
      }
      if (b == 0) return 0;                                       // multiMap (multiMap_class.f90:153-173)
      idx = idx + (int64_t)(b - 1) * c.multi[a];
    }
    return (int)idx;
  }
  double macroXS(int mat, int G, int MT) const {                 // neutronMacroXSs%get (:143-190)
    if (mat <= 0 || mat == VOID_MAT) return 0.0;
    size_t k = (size_t)(mat - 1) * mg.nG + (G - 1);
    bool f = mg.fissile[mat - 1] != 0;
    double tot = mg.total[k], ie = mg.scatter[k], cap = mg.capture[k];
    double fis = f ? mg.fission[k] : 0.0, nuf = f ? mg.nuFission[k] : 0.0;
    switch (MT) {
      case macroTotal: return tot;
      case macroDisappearance: return cap;
      case macroEscatter: return 0.0;
      case macroNonElastic: return ie + fis + cap;
      case macroIEscatter: return ie;
      case macroAllScatter: return 0.0 + ie;
      case macroFission: return fis;
      case macroNuFission: return nuf;
      case macroAbsorbtion: return cap + fis;
      default: return 0.0;
    }
  }
  // ceNeutronMaterial%getMacroXSs -> updateMacroXSs (aceNeutronDatabase_class.f90:577-640) and
  // neutronMacroXSs%get (neutronXsPackages_class.f90:115-190) for a non-fissile CE material
  double macroXSce(int mat, double E, int MT) const {
    if (mat <= 0 || mat == VOID_MAT) return 0.0;
    const CEMaterial& M = ce.mats[mat - 1];
    double x[4] = {0.0, 0.0, 0.0, 0.0};
    for (size_t i = 0; i < M.nuc.size(); ++i) {
      const CENuclide& N = ce.nucs[M.nuc[i]];
      int idx; double f;
      if (!N.search(E, idx, f)) return 0.0;
      double dens = M.dens[i] * 1.0;
      for (int k = 0; k < 4; ++k) x[k] = x[k] + dens * N.interp(idx, f, k);
    }
    switch (MT) {
      case macroTotal: return x[0];
      case macroDisappearance: return x[3];
      case macroEscatter: return x[1];
      case macroNonElastic: return x[2] + 0.0 + x[3];
      case macroIEscatter: return x[2];
      case macroAllScatter: return x[1] + x[2];
      case macroAbsorbtion: return 0.0 + x[3];
      default: return 0.0;
    }
  }
  double response(int code, int mat, int G, double E = 0.0) const {
    if (code == SG_RESP_FLUX) return 1.0;
    if (isCE) return macroXSce(mat, E, code);
    return macroXS(mat, G, code);                                // macroResponse_class.f90:141-172
  }
  bool filterPass(const Clerk& c, int G) const {                 // energyFilter_class.f90:109-127 (MG)
    if (c.d.filter_g_top <= 0) return true;
    return (c.d.filter_g_top <= G) && (G <= c.d.filter_g_low);
  }

  // tallyAdmin report dispatch (tallyAdmin_class.f90:466-704): attachment first, then own clerks
  void reportInColl(int a, Particle& p, bool virt, double trackXS) {
    if (a < 0) return;
    TallyAdmin& A = admins[a];
    reportInColl(A.atch, p, virt, trackXS);
    for (Clerk& c : A.clerks) {
      if (c.d.type == SG_CLERK_COLLISION) {                      // collisionClerk_class.f90:192-242
        if (!c.d.handle_virtual && virt) continue;
        if (!filterPass(c, p.G)) continue;
        int bin = mapState(c, p.coords.lvl[0].r, p.G, p.matIdx(), p.coords.cell(), p.E, p.isMG);
        if (bin == 0) continue;
        double flux;
        if (c.d.handle_virtual) flux = p.w / trackXS;
        else if (isCE) { double t = 0.0; ce.matTotal(p.matIdx(), p.E, t); flux = p.w / t; }
        else flux = p.w / mg.T(p.matIdx(), p.G);
        int64_t addr = c.addr + (int64_t)c.width * (bin - 1) - 1;
        for (int i = 0; i < c.width; ++i) A.mem.score(response(c.d.resp[i], p.matIdx(), p.G, p.E) * flux, addr + i + 1);
      } else if (c.d.type == SG_CLERK_KEFF_IMPLICIT) {           // keffImplicitClerk_class.f90:180-227
        if (p.matIdx() == VOID_MAT) continue;
        double flux = p.w / trackXS;
        size_t k = (size_t)(p.matIdx() - 1) * mg.nG + (p.G - 1);
        bool f = mg.fissile[p.matIdx() - 1] != 0;
        double nuFiss = f ? mg.nuFission[k] : 0.0;
        double absXS = mg.capture[k] + (f ? mg.fission[k] : 0.0);
        double s1 = nuFiss * flux, s2 = absXS * flux;
        A.mem.score(s1, c.addr + 0);
        A.mem.score(s2, c.addr + 2);
      }
    }
  }
  void reportOutColl(int a, Particle& p, int MT) {
    if (a < 0) return;
    TallyAdmin& A = admins[a];
    reportOutColl(A.atch, p, MT);
    for (Clerk& c : A.clerks) {
      if (c.d.type == SG_CLERK_KEFF_IMPLICIT) {                  // keffImplicitClerk_class.f90:241-268
        double score = 0.0;
        if (MT == macroAllScatter || MT == macroIEscatter) score = std::max(p.w - p.preCollWgt, 0.0);
        if (score > 0.0) A.mem.score(score, c.addr + 1);
      }
    }
  }
  void reportPath(int a, Particle& p, double L) {
    if (a < 0) return;
    TallyAdmin& A = admins[a];
    reportPath(A.atch, p, L);
    for (Clerk& c : A.clerks) {
      if (c.d.type == SG_CLERK_TRACK) {                          // trackClerk_class.f90:185-232
        if (!filterPass(c, p.prePathG)) continue;
        int bin = mapState(c, p.prePathR, p.prePathG, p.prePathMat, p.prePathCell, p.prePathE, p.isMG);
        if (bin == 0) continue;
        int64_t addr = c.addr + (int64_t)c.width * (bin - 1) - 1;
        for (int i = 0; i < c.width; ++i)
          A.mem.score(response(c.d.resp[i], p.prePathMat, p.G, p.E) * p.w * L, addr + i + 1);
      }
    }
  }
  // Surface-current clerk (no SCONE counterpart): for every flight from x0 to x1 (global
  // coordinates), each tally plane the flight crosses scores the weight in the bin of the
  // pre-flight state and the crossing direction.  A plane is crossed when x0 and x1 lie on
  // different sides of it (side: coordinate < plane); a leaking flight crosses every plane ahead of
  // x0 in its direction of flight.
  void reportCurrent(int a, Particle& p, const double x0[3], const double x1[3], const double u0[3], bool leaked) {
    if (a < 0) return;
    TallyAdmin& A = admins[a];
    reportCurrent(A.atch, p, x0, x1, u0, leaked);
    for (Clerk& c : A.clerks) {
      if (c.d.type != SG_CLERK_SURFACE_CURRENT) continue;
      int ax = c.d.current_axis - SG_AXIS_X;
      double a0 = x0[ax], a1 = x1[ax], u = u0[ax];
      int bin = 0;
      for (int k = 0; k < c.d.n_planes; ++k) {
        double pl = c.d.planes[k];
        bool crossed;
        if (leaked) crossed = (u > 0.0) ? (a0 < pl) : (u < 0.0 && a0 >= pl);
        else crossed = (a0 < pl) != (a1 < pl);
        if (!crossed) continue;
        if (bin == 0) bin = mapState(c, p.prePathR, p.prePathG, p.prePathMat, p.prePathCell, p.prePathE, p.isMG);
        if (bin == 0) return;
        int dirBin = (leaked ? u > 0.0 : a1 > a0) ? 1 : 0;
        int64_t idx = ((int64_t)k * c.nbins + (bin - 1)) * 2 + dirBin;
        A.mem.score(p.w, c.addr + idx);
      }
    }
  }
  void reportHist(int a, Particle& p) {
    if (a < 0) return;
    TallyAdmin& A = admins[a];
    reportHist(A.atch, p);
    for (Clerk& c : A.clerks)
      if (c.d.type == SG_CLERK_KEFF_IMPLICIT && p.fate == LEAK_FATE) A.mem.score(p.w, c.addr + 3);   // :276-290
  }
  void reportCycleStart(int a, double startW) {
    if (a < 0) return;
    TallyAdmin& A = admins[a];
    reportCycleStart(A.atch, startW);
    for (Clerk& c : A.clerks) if (c.d.type == SG_CLERK_KEFF_ANALOG) A.mem.score(startW, c.addr + 0);  // keffAnalog :140-147
  }
  void reportCycleEnd(int a, double endW, double kEnd) {          // tallyAdmin_class.f90:721-788
    if (a < 0) return;
    TallyAdmin& A = admins[a];
    reportCycleEnd(A.atch, endW, kEnd);
    for (Clerk& c : A.clerks) if (c.d.type == SG_CLERK_KEFF_ANALOG) A.mem.score(endW, c.addr + 1);
    A.mem.reduceBins();
    for (Clerk& c : A.clerks) {
      if (c.d.type == SG_CLERK_KEFF_ANALOG && A.mem.lastCycle()) {                 // keffAnalog :162-181
        double startW = A.mem.getScore(c.addr + 0), endWs = A.mem.getScore(c.addr + 1);
        double k = endWs / startW * kEnd;
        A.mem.accumulate(k, c.addr + 2);
      } else if (c.d.type == SG_CLERK_KEFF_IMPLICIT && A.mem.lastCycle()) {        // keffImplicit :306-326
        double nuFiss = A.mem.getScore(c.addr + 0), absorb = A.mem.getScore(c.addr + 2);
        double leak = A.mem.getScore(c.addr + 3), scatterMul = A.mem.getScore(c.addr + 1);
        double k = nuFiss / (absorb + leak - scatterMul);
        A.mem.accumulate(k, c.addr + 4);
      }
    }
    double normFactor = 1.0;
    if (A.normAddr > 0) {
      double ns = A.mem.getScore(A.normAddr);
      normFactor = A.normVal / ns;
    }
    A.mem.closeCycle(normFactor);
  }
  bool getKeff(int a, double& k, double& sd) {
    TallyAdmin& A = admins[a];
    for (Clerk& c : A.clerks) {
      if (c.d.type == SG_CLERK_KEFF_ANALOG) { A.mem.getResult(k, sd, c.addr + 2); return true; }
      if (c.d.type == SG_CLERK_KEFF_IMPLICIT) { A.mem.getResult(k, sd, c.addr + 4); return true; }
    }
    return false;
  }

  // ----- transport (TransportOperator)
  double trackingXS_material(Particle& p) {          // getTrackingXS(MATERIAL_XS) (baseMgNeutronDatabase :95-133)
    int m = p.matIdx();
    if (isCE) {                                      // ceNeutronDatabase_inter.f90:331-415
      if (m == VOID_MAT) return std::max(0.0, ce.collisionXS);
      return std::max(trackMatXS(p), ce.collisionXS);
    }
    if (m == VOID_MAT) return mg.collisionXS;
    return std::max(mg.T(m, p.G), mg.collisionXS);
  }
  double trackMatXS(Particle& p) {                   // getTrackMatXS (:137-160)
    int m = p.matIdx();
    if (m == VOID_MAT) return 0.0;
    if (isCE) {                                      // ceNeutronDatabase_inter.f90:384-415
      double t = 0.0;
      if (!ce.matTotal(m, p.E, t)) { err = "energy outside the nuclide data"; p.isDead = true; }
      return t + 0.0;
    }
    return mg.T(m, p.G);
  }
  double majorantXS(Particle& p) {                   // getTrackingXS(MAJORANT_XS)
    if (isCE) {
      double x = 0.0;
      if (!ce.majorantXS(p.E, x)) { err = "energy outside the majorant grid"; p.isDead = true; }
      return std::max(x + 0.0, ce.collisionXS);
    }
    return std::max(mg.majorant[p.G - 1], mg.collisionXS);
  }
  double speed(const Particle& p) const {            // particle_class.f90:481-503
    if (p.isMG) return 1.0;
    return std::sqrt(2.0 * p.E / neutronMass) * lightSpeed;
  }

  // surfaceTracking (transportOperatorST_class.f90:48-166); returns tracking XS cache value
  void surfaceTracking(Particle& p, int admin, double& trackXS, bool useCache) {
    distCache cache;
    while (true) {
      double sigmaTrack = trackingXS_material(p);
      trackXS = sigmaTrack;
      double dist, invSigmaTrack, sigmaT;
      if (sigmaTrack < ST_TOL) { dist = INF; invSigmaTrack = INF; sigmaT = 0.0; }
      else {
        invSigmaTrack = 1.0 / sigmaTrack;
        dist = -std::log(p.rng.get()) * invSigmaTrack;
        sigmaT = trackMatXS(p);
      }
      if (p.isDead) break;
      double spd = speed(p);                         // timeMax = 0 -> no ageing
      for (int i = 0; i < 3; ++i) p.prePathR[i] = p.coords.lvl[0].r[i];
      p.prePathMat = p.matIdx(); p.prePathG = p.G; p.prePathE = p.E; p.prePathCell = p.coords.cell();
      double u0[3] = {p.coords.lvl[0].dir[0], p.coords.lvl[0].dir[1], p.coords.lvl[0].dir[2]};
      int event;
      geom.move(p.coords, dist, event, useCache ? &cache : nullptr);
      p.time = p.time + dist / spd;
      nEvents++;
      reportPath(admin, p, dist);
      reportCurrent(admin, p, p.prePathR, p.coords.lvl[0].r, u0, p.matIdx() == OUTSIDE_MAT);
      if (p.matIdx() == OUTSIDE_MAT) { p.isDead = true; p.fate = LEAK_FATE; }
      else if (p.matIdx() == UNDEF_MAT) { err = "Particle is in undefined material"; p.isDead = true; }
      else if (p.matIdx() == OVERLAP_MAT) { err = "Particle is in overlapping cells"; p.isDead = true; }
      if (p.isDead) break;
      if (event == COLL_EV) {
        if (p.rng.get() < sigmaT * invSigmaTrack) break;
        else reportInColl(admin, p, true, trackXS);
      }
    }
  }

  // deltaTracking (transportOperatorDT_class.f90:47-131)
  void deltaTracking(Particle& p, int admin, double& trackXS) {
    double maj = majorantXS(p);
    if (p.isDead) return;
    trackXS = maj;
    double majorant_inv = 1.0 / maj;
    while (true) {
      double distance = -std::log(p.rng.get()) * majorant_inv;
      double spd = speed(p);
      double x0[3] = {p.coords.lvl[0].r[0], p.coords.lvl[0].r[1], p.coords.lvl[0].r[2]};
      double u0[3] = {p.coords.lvl[0].dir[0], p.coords.lvl[0].dir[1], p.coords.lvl[0].dir[2]};
      int m0 = p.matIdx(), c0 = p.coords.cell();
      geom.teleport(p.coords, distance);
      p.time = p.time + distance / spd;
      nEvents++;
      int m = p.matIdx();
      for (int i = 0; i < 3; ++i) p.prePathR[i] = x0[i];
      p.prePathMat = m0; p.prePathG = p.G; p.prePathE = p.E; p.prePathCell = c0;
      reportCurrent(admin, p, x0, p.coords.lvl[0].r, u0, m == OUTSIDE_MAT);
      if (m == OUTSIDE_MAT) { p.fate = LEAK_FATE; p.isDead = true; break; }
      if (m == VOID_MAT) { reportInColl(admin, p, true, trackXS); continue; }
      if (m == UNDEF_MAT || m == OVERLAP_MAT) { err = "Particle is in undefined/overlap material"; p.isDead = true; break; }
      double sigmaT = trackMatXS(p);
      if (p.isDead) break;
      if (p.rng.get() < sigmaT * majorant_inv) break;
      else reportInColl(admin, p, true, trackXS);
    }
  }

  // collisionProcessor%collide + neutronMGstd (collisionProcessor_inter.f90:114-195,
  // neutronMGstd_class.f90:85-297)
  void collide(Particle& p, int admin, double trackXS, std::vector<PState>* sites) {
    int matIdx = p.matIdx();
    // sampleCollision (:85-129): alpha test drawn even for alpha = 0
    (void)p.rng.get();
    size_t k = (size_t)(matIdx - 1) * mg.nG + (p.G - 1);
    bool fiss = mg.fissile[matIdx - 1] != 0;
    double total = mg.total[k], elastic = 0.0, inel = mg.scatter[k], capture = mg.capture[k];
    double r = p.rng.get();
    // neutronMacroXSs%invert (neutronXsPackages_class.f90:211-250)
    int C = 1;
    double xs = total * r - elastic;
    if (xs > 0.0) C = C + 1;
    xs = xs - inel;
    if (xs > 0.0) C = C + 1;
    xs = xs - capture;
    if (xs > 0.0) C = C + 1;
    int MT = (C == 1) ? macroEscatter : (C == 2) ? macroIEscatter : (C == 3) ? macroDisappearance : macroFission;
    reportInColl(admin, p, false, trackXS);
    p.preCollWgt = p.w;
    // implicit (:134-201): fission sites
    if (fiss) {
      double wgt = p.w, w0 = p.preHistWgt, k_eff = p.k_eff;
      double rand1 = p.rng.get();
      double sig_tot = total, sig_nuFiss = mg.nuFission[k];
      int n = (int)(std::fabs((wgt * sig_nuFiss) / (w0 * sig_tot * k_eff)) + rand1);
      if (n >= 1) {
        double sw = sgn(w0, wgt);
        double r0[3] = {p.coords.lvl[0].r[0], p.coords.lvl[0].r[1], p.coords.lvl[0].r[2]};
        for (int i = 0; i < n; ++i) {
          // fissionMG%sampleOut (fissionMG_class.f90:183-206)
          double mu = 2.0 * p.rng.get() - 1.0;
          double phi = TWO_PI * p.rng.get();
          double rem = p.rng.get();
          int Gout = 1;
          for (Gout = 1; Gout <= mg.nG; ++Gout) {
            rem = rem - mg.chi[(size_t)(matIdx - 1) * mg.nG + (Gout - 1)];
            if (rem < 0.0) break;
          }
          if (Gout > mg.nG) { err = "fission G_out sampling failed"; Gout = mg.nG; }
          PState s;
          rotateVector(p.coords.lvl[0].dir, mu, phi, s.dir);
          for (int q = 0; q < 3; ++q) s.r[q] = r0[q];
          s.G = Gout; s.wgt = sw; s.time = p.time; s.broodID = p.broodID; s.matIdx = matIdx;
          if (sites) sites->push_back(s);
        }
      }
    }
    // reaction
    if (MT == macroIEscatter || MT == macroEscatter) {
      // inelastic (:221-252): multiScatterMG%sampleOut (:199-238)
      double rem = p.rng.get() * inel;
      int Gout;
      for (Gout = 1; Gout <= mg.nG; ++Gout) {
        rem = rem - mg.P0[((size_t)(matIdx - 1) * mg.nG + (p.G - 1)) * mg.nG + (Gout - 1)];
        if (rem < 0.0) break;
      }
      if (Gout > mg.nG) { err = "scatter G_out sampling failed"; Gout = mg.nG; }
      double mu;
      if (!mg.P1.empty())                                // multiScatterP1MG%sampleOut (:69-85)
        mu = sampleLegendreP1(mg.P1[((size_t)(matIdx - 1) * mg.nG + (p.G - 1)) * mg.nG + (Gout - 1)], p.rng, err);
      else mu = 2.0 * p.rng.get() - 1.0;
      double phi = TWO_PI * p.rng.get();
      double w_mul = mg.prod[((size_t)(matIdx - 1) * mg.nG + (p.G - 1)) * mg.nG + (Gout - 1)];
      MT = macroIEscatter;
      p.G = Gout;
      p.w = p.w * w_mul;
      p.coords.rotate(mu, phi);
    } else {
      p.isDead = true;   // capture / fission
    }
    if (collImp) impCutoffs(p);                          // neutronMGimp cutoffs (:319-351)
    p.collisionN += 1;
    nColl++;
    reportOutColl(admin, p, MT);
    if (p.isDead) { p.fate = ABS_FATE; reportHist(admin, p); }
  }

  // neutronCEimp%cutoffs (neutronCEimp_class.f90:633-678); neutronMGimp%cutoffs acts through weight
  // windows only (neutronMGimp_class.f90:319-351)
  void impCutoffs(Particle& p) {
    if (p.isDead) return;
    if (isCE && p.E < ce.minE) { p.isDead = true; return; }
    if (coll.weight_windows) {
      // weightWindowsField%atP (weightWindowsField_class.f90:148-171)
      int bin = mapState(wwMap, p.coords.lvl[0].r, p.G, p.matIdx(), p.coords.cell(), p.E, p.isMG);
      double minW = 0.0, maxW = 0.0, avW = 0.0;
      if (bin != 0) { minW = wwLo[bin - 1]; maxW = wwUp[bin - 1]; avW = minW * coll.ww_const_survival; }
      if ((p.w > maxW) && (maxW != 0.0) && (p.splitCount < coll.max_split)) split(p, maxW);
      else if (p.w < minW) russianRoulette(p, avW);
      return;
    }
    if (!isCE) return;
    if (coll.split && p.w > coll.max_wgt) split(p, coll.max_wgt);
    else if (coll.roulette && p.w < coll.min_wgt) russianRoulette(p, coll.av_wgt);
  }
  // russianRoulette (neutronCEimp_class.f90:683-694)
  void russianRoulette(Particle& p, double avWgt) {
    if (p.rng.get() < (1.0 - p.w / avWgt)) p.isDead = true;
    else p.w = avWgt;
  }
  // split (neutronCEimp_class.f90:699-734): mult - 1 copies into the history's buffer
  void split(Particle& p, double maxWgt) {
    int mult = (int)std::ceil(p.w / maxWgt);
    if (mult + p.splitCount > coll.max_split) mult = coll.max_split - p.splitCount + 1;
    PState t;
    t.wgt = p.w / mult;
    for (int i = 0; i < 3; ++i) { t.r[i] = p.coords.lvl[0].r[i]; t.dir[i] = p.coords.lvl[0].dir[i]; }
    t.E = p.E; t.G = p.G; t.time = p.time; t.broodID = p.broodID;
    for (int i = 1; i <= mult - 1; ++i) p.buffer.push_back(t);
    p.splitCount = p.splitCount + mult;
    p.w = p.w / mult;
  }

  // collisionProcessor%collide with neutronCEstd (collisionProcessor_inter.f90:114-195,
  // neutronCEstd_class.f90:157-588) for non-fissile nuclides with CM-isotropic elastic scattering
  void collideCE(Particle& p, int admin, double trackXS) {
    const int matIdx = p.matIdx();
    // sampleCollision (:157-214)
    double denom = trackMatXS(p);
    double probAlpha = 0.0 / denom;                      // getAlphaAbsorption = 0 (alpha = 0)
    (void)(p.rng.get() < probAlpha);
    const CEMaterial& M = ce.mats[matIdx - 1];
    // ceNeutronMaterial%sampleNuclide (ceNeutronMaterial_class.f90:338-455), TMS off
    double trackMat = 0.0;
    ce.matTotal(matIdx, p.E, trackMat);
    double xi = trackMat * p.rng.get();
    int nucIdx = -1;
    for (size_t i = 0; i < M.nuc.size(); ++i) {
      double tot = 0.0;
      ce.nucTotal(M.nuc[i], p.E, tot);
      xi = xi - tot * (M.dens[i] * 1.0);
      if (xi < 0.0) { nucIdx = M.nuc[i]; break; }
    }
    if (nucIdx < 0) { err = "Nuclide sampling loop failed to terminate"; p.isDead = true; return; }
    const CENuclide& N = ce.nucs[nucIdx];
    int idx = 1; double f = 0.0;
    N.search(p.E, idx, f);
    double micro[4];
    for (int k = 0; k < 4; ++k) micro[k] = N.interp(idx, f, k);
    // neutronMicroXSs%invert (neutronXsPackages_class.f90:273-310): no fission data
    double r = p.rng.get();
    int C = 1;
    double xs = micro[0] * r - micro[1];
    if (xs > 0.0) C = C + 1;
    xs = xs - micro[2];
    if (xs > 0.0) C = C + 1;
    xs = xs - micro[3];
    if (xs > 0.0) C = C + 1;
    reportInColl(admin, p, false, trackXS);
    p.preCollWgt = p.w;
    // implicit (:220-311): non-fissile nuclide, no sites; neutronCEimp implicit absorption (:406-424)
    if (collImp && coll.imp_abs) {
      double sig_scatter = micro[1] + micro[2];
      double sig_tot = micro[0];
      p.w = p.w * sig_scatter / sig_tot;
      double totalElastic = micro[1] + micro[2];
      C = (p.rng.get() < micro[1] / totalElastic) ? 1 : 2;
    }
    int MT;
    if (C == 1) {                                        // elastic (:340-384)
      MT = 2;                                            // N_N_elastic
      double A = N.A, kT = N.kT;
      bool isFixed = (p.E > kT * ce.threshE) && (A > ce.threshA);
      if (isFixed) {                                     // scatterFromFixed (:460-491)
        double mu = 2.0 * p.rng.get() - 1.0;             // elasticNeutronScatter%sampleOut (:168-195)
        double phi = p.rng.get() * TWO_PI;
        double E_out = p.E;
        asymptoticScatter(E_out, mu, A);
        p.coords.rotate(mu, phi);
        p.E = E_out;
      } else {                                           // scatterFromMoving (:495-585)
        double dir_pre[3] = {p.coords.lvl[0].dir[0], p.coords.lvl[0].dir[1], p.coords.lvl[0].dir[2]};
        double sE = std::sqrt(p.E);
        double V_n[3], V_t[3], V_cm[3];
        for (int i = 0; i < 3; ++i) V_n[i] = dir_pre[i] * sE;
        targetVelocity_constXS(p.E, dir_pre, A, kT, p.rng, V_t);
        for (int i = 0; i < 3; ++i) V_cm[i] = (V_n[i] + V_t[i] * A) / (A + 1);
        for (int i = 0; i < 3; ++i) V_n[i] = V_n[i] - V_cm[i];
        double U_n = norm2_3(V_n);
        for (int i = 0; i < 3; ++i) V_n[i] = V_n[i] / U_n;
        double mu = 2.0 * p.rng.get() - 1.0;
        double phi = p.rng.get() * TWO_PI;
        double rv[3];
        rotateVector(V_n, mu, phi, rv);
        for (int i = 0; i < 3; ++i) V_n[i] = rv[i] * U_n;
        for (int i = 0; i < 3; ++i) V_n[i] = V_n[i] + V_cm[i];
        U_n = norm2_3(V_n);
        double dir_post[3];
        for (int i = 0; i < 3; ++i) dir_post[i] = V_n[i] / U_n;
        p.E = U_n * U_n;
        p.coords.assignDirection(dir_post);
      }
    } else if (C == 2) {
      err = "inelastic scattering is not supported by the CE data"; p.isDead = true; return;
    } else {                                             // capture / fission: kill
      MT = (C == 3) ? 101 : 18;
      p.isDead = true;
    }
    if (collImp) impCutoffs(p);                          // neutronCEimp cutoffs (:633-678)
    else if (p.E < ce.minE) p.isDead = true;             // cutoffs (:434-444)
    p.collisionN += 1;
    nColl++;
    reportOutColl(admin, p, MT);
    if (p.isDead) { p.fate = ABS_FATE; reportHist(admin, p); }
  }

  // one history: copy from the bank, place, history loop (eigenPhysicsPackage_class.f90:211-246)
  void runHistory(const PState& st, int n, uint64_t master, double k, int admin,
                  std::vector<PState>* sites, int32_t* recC, uint64_t* recR) {
    Particle p;
    p.rng.s = master;
    p.rng.stride(n);
    p.w = st.wgt; p.w0 = st.wgt;
    p.coords.takeAboveGeom();
    for (int i = 0; i < 3; ++i) { p.coords.lvl[0].r[i] = st.r[i]; p.coords.lvl[0].dir[i] = st.dir[i]; }
    p.G = st.G; p.time = st.time; p.fate = NO_FATE; p.collisionN = 0; p.isDead = false;
    p.E = st.E; p.isMG = !isCE;
    p.broodID = n;
    geom.placeCoord(p.coords);
    p.k_eff = k;
    p.preHistWgt = p.w; p.preCollWgt = p.w;
    while (true) {
      double trackXS = 0.0;
      if (transport == SG_TRANSPORT_DT) deltaTracking(p, admin, trackXS);
      else if (transport == SG_TRANSPORT_HT || transport == SG_TRANSPORT_HT_NOCACHE) {
        // tracking_selection (transportOperatorHT_class.f90:49-81): DT if Sigma_t/Sigma_maj > 1 - cutoff
        double majorant_inv = 1.0 / majorantXS(p);
        double sigmaT = (p.matIdx() == VOID_MAT) ? 0.0 : trackMatXS(p);
        if (sigmaT * majorant_inv > 1.0 - htCutoff) deltaTracking(p, admin, trackXS);
        else surfaceTracking(p, admin, trackXS, transport == SG_TRANSPORT_HT);
      } else surfaceTracking(p, admin, trackXS, transport == SG_TRANSPORT_ST);
      if (!p.isDead) {
        if (isCE) collideCE(p, admin, trackXS);
        else collide(p, admin, trackXS, sites);
        if (!p.isDead) continue;
      } else reportHist(admin, p);
      if (p.buffer.empty()) break;
      // buffer%release and the restart of bufferLoop (fixedSourcePhysicsPackage_class.f90:209-216,
      // 235-239): the last split particle, placed; the RNG stream continues
      const PState b = p.buffer.back();
      p.buffer.pop_back();
      p.coords.takeAboveGeom();
      for (int i = 0; i < 3; ++i) { p.coords.lvl[0].r[i] = b.r[i]; p.coords.lvl[0].dir[i] = b.dir[i]; }
      p.w = b.wgt; p.G = b.G; p.E = b.E; p.time = b.time;
      p.splitCount = 0; p.isDead = false; p.fate = NO_FATE;
      geom.placeCoord(p.coords);
      p.preHistWgt = p.w; p.preCollWgt = p.w;
    }
    if (recC) *recC = p.collisionN;
    if (recR) *recR = p.rng.s;
  }

  int transportBank(int admin, const std::vector<PState>& in, uint64_t master, double k,
                    std::vector<PState>& next) {
    int n = (int)in.size();
    recColl.assign(n, 0); recRng.assign(n, 0);
    nEvents = 0; nColl = 0;
    next.clear();
    for (int i = 0; i < n; ++i) {
      std::vector<PState> s;
      runHistory(in[i], i + 1, master, k, admin, &s, &recColl[i], &recRng[i]);
      next.insert(next.end(), s.begin(), s.end());
      if (!err.empty()) return SG_ERR_LOST;
    }
    return SG_OK;
  }

  // pointSource / configSource sampleParticle (pointSource_class.f90:189-270)
  // fileSource (fileSource_class.f90:47-190): the particle table and its sampling
  std::vector<PState> fileSrc;
  int sampleFile(RNG& rand, PState& s) {
    const long long N = (long long)fileSrc.size();
    const long long idx = (long long)(rand.get() * (double)N) + 1;
    if (idx > N) return SG_ERR_STATE;
    s = fileSrc[idx - 1];
    int matIdx, uid;
    double u0[3] = {1.0, 0.0, 0.0};
    geom.whatIsAt(matIdx, uid, s.r, u0);
    if (matIdx == OUTSIDE_MAT || matIdx == UNDEF_MAT) return SG_ERR_UNDEF_MAT;
    s.time = 0.0;
    s.broodID = 0;
    return SG_OK;
  }

  PState samplePoint(RNG& rand) {
    PState s;
    for (int i = 0; i < 3; ++i) s.r[i] = src.r[i];
    if (src.isotropic) {
      double mu = 2.0 * rand.get() - 1.0;
      double phi = TWO_PI * rand.get();
      double x[3] = {1.0, 0.0, 0.0};
      rotateVector(x, mu, phi, s.dir);
    } else for (int i = 0; i < 3; ++i) s.dir[i] = src.dir[i];
    if (!srcProbG.empty()) {
      double r = rand.get(); int g;
      for (g = 1; g <= (int)srcProbG.size(); ++g) { r = r - srcProbG[g - 1]; if (r < 0.0) break; }
      if (g > (int)srcProbG.size()) g = (int)srcProbG.size() + 1;   // Fortran do-loop exit value
      s.G = g;
    } else s.G = src.G;
    s.time = 0.0; s.wgt = 1.0;
    s.E = src.E;
    return s;
  }

  // fissionSource sampleParticle (fissionSource_class.f90:149-271), MG, G = 1
  int sampleFission(RNG& rand, PState& s) {
    double bb[6]; geom.bounds(bb);
    for (int i = 0; i < 10000; ++i) {
      double r3[3] = {rand.get(), rand.get(), rand.get()};
      double r[3];
      for (int q = 0; q < 3; ++q) r[q] = (bb[3 + q] - bb[q]) * r3[q] + bb[q];
      int matIdx, uid; double u0[3] = {1.0, 0.0, 0.0};
      geom.whatIsAt(matIdx, uid, r, u0);
      if (matIdx == VOID_MAT || matIdx == OUTSIDE_MAT) continue;
      if (matIdx == UNDEF_MAT || matIdx == OVERLAP_MAT) return -1;
      if (!mg.fissile[matIdx - 1]) continue;
      s.matIdx = matIdx; s.wgt = 1.0; s.time = 0.0;
      for (int q = 0; q < 3; ++q) s.r[q] = r[q];
      double mu = 2.0 * rand.get() - 1.0;
      double phi = TWO_PI * rand.get();
      double rem = rand.get(); int Gout;
      for (Gout = 1; Gout <= mg.nG; ++Gout) {
        rem = rem - mg.chi[(size_t)(matIdx - 1) * mg.nG + (Gout - 1)];
        if (rem < 0.0) break;
      }
      s.G = Gout;
      double x[3] = {1.0, 0.0, 0.0};
      rotateVector(x, mu, phi, s.dir);
      return 0;
    }
    return -1;
  }

  // particleDungeon%normSize_Repr for one rank (particleDungeon_class.f90:431-605)
  void sortByBroodID(std::vector<PState>& b) {   // stable counting sort (:923-981)
    std::stable_sort(b.begin(), b.end(), [](const PState& x, const PState& y) { return x.broodID < y.broodID; });
  }
  void normSizeRepr(std::vector<PState>& b, int totPop, const RNG& rand) {
    sortByBroodID(b);
    int totSites = (int)b.size();
    int excess = totSites - totPop;
    int heapSize, n_duplicates;
    if (excess < 0) { n_duplicates = (-excess) % totSites; heapSize = n_duplicates; }
    else heapSize = excess;
    double threshold = 1.0;
    uint64_t seed = 0;
    if (heapSize != 0) {
      RNG mr = rand;
      seed = mr.s;
      std::vector<double> rn(totSites);
      for (int j = 0; j < totSites; ++j) rn[j] = mr.get();
      std::vector<double> tmp(rn);
      std::nth_element(tmp.begin(), tmp.begin() + (heapSize - 1), tmp.end());
      threshold = tmp[heapSize - 1];      // heapSize-th smallest = max of the heap
    }
    RNG rr; rr.s = seed;
    if (excess > 0) {
      std::vector<PState> keep;
      for (int i = 0; i < totSites; ++i) if (rr.get() > threshold) keep.push_back(b[i]);
      b.swap(keep);
    } else if (excess < 0) {
      int ts = excess + totPop;
      int n_copies = (-excess) / ts;
      n_duplicates = (-excess) % ts;
      int p0 = (int)b.size();
      std::vector<PState> out(b);
      for (int c = 0; c < n_copies; ++c) out.insert(out.end(), b.begin(), b.begin() + p0);
      if (n_duplicates != 0)
        for (int i = 0; i < p0; ++i) if (rr.get() <= threshold) out.push_back(b[i]);
      b.swap(out);
      sortByBroodID(b);
    }
  }
  // normSize_Repr on one rank of an MPI run (the same routine, :431-590): popSizes gathered to the
  // master (:466), which draws one number per site of every rank in rank order into the heap and
  // records the state each rank's draws start from (:477-494); threshold, excess and seeds are
  // broadcast (:497-501) and the rank keeps or duplicates its own sites with its seed (:507-586).
  // `before` is the number of sites of the ranks below, `totSites` the sum of popSizes; `b` holds
  // this rank's sites.  loadBalancing (:593-700) is left to the caller.
  void normSizeReprRank(std::vector<PState>& b, int64_t before, int64_t totSites, int totPop, const RNG& rand) {
    sortByBroodID(b);
    const int64_t excess = totSites - totPop;
    int64_t heapSize = excess < 0 ? (-excess) % totSites : excess;
    double threshold = 1.0;
    uint64_t seed = 0;
    if (heapSize != 0) {                              // master: the heap over all ranks' draws
      RNG mr = rand;
      std::vector<double> rn((size_t)totSites);
      for (int64_t j = 0; j < totSites; ++j) {
        if (j == before) seed = mr.s;                 // seeds(rank + 1)
        rn[(size_t)j] = mr.get();
      }
      if (before == totSites) seed = mr.s;
      std::nth_element(rn.begin(), rn.begin() + (heapSize - 1), rn.end());
      threshold = rn[(size_t)(heapSize - 1)];
    }
    RNG rr; rr.s = seed;                              // rankRand%init(seeds(rank + 1))
    const int pop = (int)b.size();
    if (excess > 0) {
      std::vector<PState> keep;
      for (int i = 0; i < pop; ++i) if (rr.get() > threshold) keep.push_back(b[i]);
      b.swap(keep);
    } else if (excess < 0) {
      const int64_t n_copies = (-excess) / totSites;
      const int64_t n_duplicates = (-excess) % totSites;
      std::vector<PState> out(b);
      for (int64_t c = 0; c < n_copies; ++c) out.insert(out.end(), b.begin(), b.begin() + pop);
      if (n_duplicates != 0)
        for (int i = 0; i < pop; ++i) if (rr.get() <= threshold) out.push_back(b[i]);
      b.swap(out);
      sortByBroodID(b);
    }
  }
};

}  // namespace orc

using orc::Oracle;

// ====================================================================== C ABI
extern "C" {

typedef struct or_handle_t* or_handle;

static Oracle* O(or_handle h) { return reinterpret_cast<Oracle*>(h); }

static void bankToStates(const sg_bank* b, int n, std::vector<orc::PState>& v) {
  v.resize(n);
  for (int i = 0; i < n; ++i) {
    orc::PState& s = v[i];
    s.wgt = b->wgt ? b->wgt[i] : 1.0;
    for (int q = 0; q < 3; ++q) { s.r[q] = b->r[3 * i + q]; s.dir[q] = b->dir[3 * i + q]; }
    s.G = b->G ? b->G[i] : 1;
    s.time = b->time ? b->time[i] : 0.0;
    s.broodID = b->brood_id ? b->brood_id[i] : 0;
    s.E = b->E ? b->E[i] : 0.0;
  }
}
static void statesToBank(const std::vector<orc::PState>& v, sg_bank* b, int cap) {
  int n = std::min((int)v.size(), cap);
  for (int i = 0; i < n; ++i) {
    const orc::PState& s = v[i];
    if (b->wgt) b->wgt[i] = s.wgt;
    for (int q = 0; q < 3; ++q) { if (b->r) b->r[3 * i + q] = s.r[q]; if (b->dir) b->dir[3 * i + q] = s.dir[q]; }
    if (b->G) b->G[i] = s.G;
    if (b->time) b->time[i] = s.time;
    if (b->brood_id) b->brood_id[i] = s.broodID;
    if (b->E) b->E[i] = s.E;
  }
}

int32_t or_create(int32_t transport, or_handle* out) {
  Oracle* o = new Oracle();
  o->transport = transport;
  *out = reinterpret_cast<or_handle>(o);
  return SG_OK;
}
int32_t or_destroy(or_handle h) { delete O(h); return SG_OK; }
// n draws of sampleLegendre_P1 for the normalised coefficient a = 3 P1/P0 (state advanced)
int32_t or_sample_legendre_p1(double a, uint64_t* state, double* out, int32_t n) {
  orc::RNG r;
  r.s = *state;
  std::string err;
  for (int i = 0; i < n; ++i) out[i] = orc::sampleLegendreP1(a, r, err);
  *state = r.s;
  return err.empty() ? SG_OK : SG_ERR_BAD_ARG;
}
int32_t or_set_file_source(or_handle h, const sg_bank* p, int32_t n) {
  Oracle* o = O(h);
  o->fileSrc.assign(n, orc::PState());
  for (int i = 0; i < n; ++i) {
    orc::PState& s = o->fileSrc[i];
    for (int k = 0; k < 3; ++k) { s.r[k] = p->r[3 * i + k]; s.dir[k] = p->dir[3 * i + k]; }
    s.wgt = p->wgt ? p->wgt[i] : 1.0;
    s.E = p->E ? p->E[i] : 0.0;
    s.G = p->G ? p->G[i] : 0;
  }
  return SG_OK;
}
int32_t or_set_ht_cutoff(or_handle h, double c) {
  if (!(c > 0.0 && c < 1.0)) return SG_ERR_BAD_ARG;
  O(h)->htCutoff = c;
  return SG_OK;
}
int32_t or_last_error(or_handle h, char* buf, size_t len) {
  std::snprintf(buf, len, "%s", O(h)->err.c_str());
  return SG_OK;
}
int32_t or_upload_geometry(or_handle h, const sg_geometry_desc* g) {
  return O(h)->geom.build(g, O(h)->err) == 0 ? SG_OK : SG_ERR_BAD_ARG;
}
int32_t or_upload_mg(or_handle h, const sg_mg_desc* d) {
  Oracle* o = O(h);
  o->mg.build(d, o->err);
  // activeMats = materials present in the geometry graph (geometryStd%activeMats)
  std::vector<int> act;
  for (int f : o->geom.graphIdx) if (f > 0 && f <= o->mg.nMat) act.push_back(f);
  std::sort(act.begin(), act.end());
  act.erase(std::unique(act.begin(), act.end()), act.end());
  o->mg.initMajorant(act);
  return SG_OK;
}
int32_t or_upload_ce(or_handle h, const sg_ce_desc* d) {
  Oracle* o = O(h);
  if (o->ce.build(d, o->err) != 0) return SG_ERR_BAD_ARG;
  std::vector<int> act;
  for (int f : o->geom.graphIdx) if (f > 0 && f <= (int)o->ce.mats.size()) act.push_back(f);
  std::sort(act.begin(), act.end());
  act.erase(std::unique(act.begin(), act.end()), act.end());
  if (o->ce.hasMajorant) o->ce.initMajorant(act);
  else o->ce.activeMat = act;
  o->isCE = true;
  return SG_OK;
}
// CE probes: nuclide microscopic XSs [total elastic inelastic capture], material total, majorant
int32_t or_ce_micro(or_handle h, int32_t nuc, double E, double* out) {
  const orc::CENuclide& N = O(h)->ce.nucs[nuc];
  int idx; double f;
  if (!N.search(E, idx, f)) return SG_ERR_BAD_ARG;
  for (int k = 0; k < 4; ++k) out[k] = N.interp(idx, f, k);
  return SG_OK;
}
int32_t or_ce_mat_total(or_handle h, int32_t mat, double E, double* out) {
  return O(h)->ce.matTotal(mat, E, *out) ? SG_OK : SG_ERR_BAD_ARG;
}
int32_t or_ce_majorant(or_handle h, double E, double* out) {
  return O(h)->ce.majorantXS(E, *out) ? SG_OK : SG_ERR_BAD_ARG;
}
int32_t or_ce_union_size(or_handle h, int64_t* n) { *n = (int64_t)O(h)->ce.eGridUnion.size(); return SG_OK; }
int32_t or_asymptotic_scatter(double E, double mu, double A, double* out) {
  orc::asymptoticScatter(E, mu, A); out[0] = E; out[1] = mu; return SG_OK;
}
int32_t or_target_velocity(double E, const double* dir, double A, double kT, uint64_t* state, double* V_t) {
  orc::RNG r; r.s = *state;
  orc::targetVelocity_constXS(E, dir, A, kT, r, V_t);
  *state = r.s;
  return SG_OK;
}

static int64_t setupAxes(Oracle* o, orc::Clerk& c);

// one particle state through a multiMap of the given axes (tallyMap%map): 1-based bin, 0 outside
int32_t or_map_point(or_handle h, const sg_axis_desc* axes, int32_t n_axes, const double* r, int32_t G,
                     int32_t mat, int32_t cell, double E, int32_t isMG, int32_t* bin) {
  Oracle* o = O(h);
  orc::Clerk c{};
  c.d.n_axes = n_axes;
  for (int a = 0; a < n_axes; ++a) c.d.axes[a] = axes[a];
  setupAxes(o, c);
  if (cell < 0 || cell > (int)o->geom.cells.size()) return SG_ERR_BAD_ARG;
  *bin = o->mapState(c, r, G, mat, cell, E, isMG != 0);
  return SG_OK;
}

int32_t or_grid_search(const double* bounds, int32_t nb, double v) {
  std::vector<double> b(bounds, bounds + nb);
  return Oracle::binaryFloor(b, v);
}

// multiMap axes of one clerk (tallyMapFactory / grid%init / cellMap%build): grid types and steps,
// unstructured bounds and cell bins copied out of the caller's arrays; returns the number of bins
static int64_t setupAxes(Oracle* o, orc::Clerk& c) {
  int64_t mul = 1;
  for (int a = 0; a < c.d.n_axes; ++a) {
    const sg_axis_desc& ax = c.d.axes[a];
    int64_t nb = ax.n;
    c.grid[a] = ax.grid != SG_GRID_DEFAULT ? ax.grid : (ax.kind == SG_AXIS_ENERGY ? SG_GRID_LOG : SG_GRID_LIN);
    if (c.grid[a] == SG_GRID_LOG) c.step[a] = std::log(ax.max / ax.min) / ax.n;   // grid_class.f90:76-90
    else c.step[a] = (ax.max - ax.min) / ax.n;                                    // grid_class.f90:63-74
    if (c.grid[a] == SG_GRID_UNSTRUCT && (ax.kind <= SG_AXIS_Z || ax.kind == SG_AXIS_ENERGY))
      c.bounds[a].assign(ax.bounds, ax.bounds + ax.n + 1);
    if (ax.kind == SG_AXIS_CELL) {                            // cellMap%build (cellMap_class.f90:87-138)
      int rest = ax.cell_rest ? ax.n + 1 : 0;
      c.cellBin[a].assign(o->geom.cells.size() + 1, rest);
      for (int i = 0; i < ax.n; ++i) c.cellBin[a][ax.cells[i] + 1] = i + 1;
      if (ax.cell_rest) nb += 1;
    }
    c.d.axes[a].bounds = nullptr;                             // the caller's arrays are not kept
    c.d.axes[a].cells = nullptr;
    c.multi[a] = mul; mul *= nb;
  }
  return mul;
}

int32_t or_upload_tally(or_handle h, const sg_tally_desc* t, int32_t* admin) {
  Oracle* o = O(h);
  orc::TallyAdmin A;
  int64_t memLoc = 1;
  for (int i = 0; i < t->n_clerks; ++i) {
    orc::Clerk c; c.d = t->clerks[i];
    c.width = c.d.n_resp > 0 ? c.d.n_resp : 1;
    c.nbins = setupAxes(o, c);
    c.addr = memLoc;
    memLoc += c.size();
    A.clerks.push_back(c);
  }
  A.mem.init(memLoc - 1, t->batch_size);
  if (t->norm_clerk >= 0) { A.normAddr = A.clerks[t->norm_clerk].addr; A.normVal = t->norm_val; }
  o->admins.push_back(A);
  *admin = (int32_t)o->admins.size() - 1;
  return SG_OK;
}
// neutronMGimp / neutronCEimp options (neutronCEimp_class.f90:160-232) and weightWindowsField
// (weightWindowsField_class.f90:75-111)
int32_t or_set_collision(or_handle h, const sg_collision_desc* d) {
  Oracle* o = O(h);
  if (d->kind == SG_COLL_STD) { o->collImp = false; return SG_OK; }
  if (d->split && d->max_wgt < 2 * d->min_wgt) { o->err = "upper weight bound must be at least twice the lower"; return SG_ERR_BAD_ARG; }
  if (d->imp_abs && !d->roulette && !d->weight_windows) { o->err = "implicit absorption needs roulette or weight windows"; return SG_ERR_BAD_ARG; }
  o->coll = *d;
  if (d->weight_windows) {
    orc::Clerk c{};
    c.d.n_axes = d->ww_n_axes;
    for (int a = 0; a < d->ww_n_axes; ++a) c.d.axes[a] = d->ww_axes[a];
    const int64_t N = setupAxes(o, c);
    o->wwMap = c;
    o->wwLo.assign(d->ww_lower, d->ww_lower + N);
    o->wwUp.assign(d->ww_upper, d->ww_upper + N);
    if (!(d->ww_const_survival > 1.0)) { o->err = "survival constant must be bigger than one"; return SG_ERR_BAD_ARG; }
  }
  o->collImp = true;
  return SG_OK;
}
int32_t or_attach_tally(or_handle h, int32_t admin, int32_t atch) { O(h)->admins[admin].atch = atch; return SG_OK; }
int32_t or_set_point_source(or_handle h, const sg_point_source_desc* s) {
  Oracle* o = O(h);
  o->src = *s;
  o->srcProbG.assign(s->prob_g, s->prob_g + s->n_prob_g);
  o->hasSource = true;
  return SG_OK;
}
int32_t or_generate_source(or_handle h, uint64_t master, int32_t n, sg_bank* out) {
  Oracle* o = O(h);
  std::vector<orc::PState> v(n);
  for (int i = 1; i <= n; ++i) {                      // source_inter.f90:98-119
    orc::RNG r; r.s = master; r.stride(i);
    v[i - 1] = o->samplePoint(r);
  }
  statesToBank(v, out, n);
  return SG_OK;
}
int32_t or_transport_bank(or_handle h, int32_t admin, const sg_bank* in, int32_t n, uint64_t master,
                          double k, sg_bank* next, int32_t cap, sg_cycle_stats* st) {
  Oracle* o = O(h);
  std::vector<orc::PState> v, nx;
  bankToStates(in, n, v);
  int rc = o->transportBank(admin, v, master, k, nx);
  if (st) {
    st->n_histories = n; st->n_events = o->nEvents; st->n_collisions = o->nColl; st->n_next = (int64_t)nx.size();
    double sw = 0; for (auto& s : v) sw += s.wgt;
    double ew = 0; for (auto& s : nx) ew += s.wgt;
    st->start_weight = sw; st->end_weight = ew; st->k_eff = k; st->k_new = k;
  }
  if ((int)nx.size() > cap) return SG_ERR_BANK_OVERFLOW;
  if (next) statesToBank(nx, next, cap);
  return rc;
}
int32_t or_tally_cycle_start(or_handle h, int32_t admin, double w) { O(h)->reportCycleStart(admin, w); return SG_OK; }
int32_t or_tally_cycle_end(or_handle h, int32_t admin, double w, double k) { O(h)->reportCycleEnd(admin, w, k); return SG_OK; }
int32_t or_tally_size(or_handle h, int32_t admin, int64_t* n) { *n = O(h)->admins[admin].mem.N; return SG_OK; }
int32_t or_get_bins(or_handle h, int32_t admin, double* bins, int64_t n) {
  orc::ScoreMemory& m = O(h)->admins[admin].mem;
  for (int64_t i = 0; i < n && i < m.N; ++i) { bins[i] = m.bin[i]; bins[n + i] = m.csum[i]; bins[2 * n + i] = m.csum2[i]; }
  return SG_OK;
}
int32_t or_normalise_shard(or_handle h, const sg_bank* sites, int32_t n, int64_t before, int64_t tot_sites,
                           int32_t tot_pop, uint64_t master, sg_bank* out, int32_t cap, int32_t* n_out) {
  if (n < 0 || before < 0 || tot_sites < before + n || tot_pop <= 0) return SG_ERR_BAD_ARG;
  if (tot_sites == 0) return SG_ERR_STATE;
  std::vector<orc::PState> v;
  bankToStates(sites, n, v);
  orc::RNG r; r.s = master;
  O(h)->normSizeReprRank(v, before, tot_sites, tot_pop, r);
  *n_out = (int32_t)v.size();
  if ((int)v.size() > cap) return SG_ERR_BANK_OVERFLOW;
  statesToBank(v, out, cap);
  return SG_OK;
}
// normSize_Repr of a single-process run on a bank given by the caller (the sites sorted by brood)
int32_t or_normalise(or_handle h, const sg_bank* sites, int32_t n, int32_t tot_pop, uint64_t master, sg_bank* out,
                     int32_t cap, int32_t* n_out) {
  if (n <= 0 || tot_pop <= 0) return SG_ERR_BAD_ARG;
  std::vector<orc::PState> v;
  bankToStates(sites, n, v);
  orc::RNG r; r.s = master;
  O(h)->normSizeRepr(v, tot_pop, r);
  *n_out = (int32_t)v.size();
  if ((int)v.size() > cap) return SG_ERR_BANK_OVERFLOW;
  statesToBank(v, out, cap);
  return SG_OK;
}
// the running batch (parallelBins summed over threads), read and written around a sum over ranks
int32_t or_tally_get_scores(or_handle h, int32_t admin, double* s, int64_t n) {
  orc::ScoreMemory& m = O(h)->admins[admin].mem;
  if (n < m.N) return SG_ERR_BAD_ARG;
  for (int64_t i = 0; i < m.N; ++i) s[i] = m.parallel[i];
  return SG_OK;
}
int32_t or_tally_set_scores(or_handle h, int32_t admin, const double* s, int64_t n) {
  orc::ScoreMemory& m = O(h)->admins[admin].mem;
  if (n < m.N) return SG_ERR_BAD_ARG;
  for (int64_t i = 0; i < m.N; ++i) m.parallel[i] = s[i];
  return SG_OK;
}
int32_t or_get_keff(or_handle h, int32_t admin, double* k, double* sd) {
  return O(h)->getKeff(admin, *k, *sd) ? SG_OK : SG_ERR_BAD_ARG;
}
int32_t or_get_history_records(or_handle h, int32_t* c, uint64_t* r, int32_t n) {
  Oracle* o = O(h);
  for (int i = 0; i < n && i < (int)o->recColl.size(); ++i) { if (c) c[i] = o->recColl[i]; if (r) r[i] = o->recRng[i]; }
  return SG_OK;
}

// eigenvalue driver (eigenPhysicsPackage_class.f90:135-412) on the oracle's own banks
int32_t or_eigen_init(or_handle h, int32_t pop, uint64_t master, double k0) {
  Oracle* o = O(h);
  o->pop = pop; o->master.s = master; o->k_new = k0; o->keff0 = k0; o->nextK = 1.0;
  o->thisCycle.assign(pop, orc::PState());
  for (int i = 1; i <= pop; ++i) {                    // generateInitialState (:348-366)
    orc::RNG r = o->master; r.stride(i);
    if (o->sampleFission(r, o->thisCycle[i - 1]) != 0) { o->err = "fission source failed"; return SG_ERR_STATE; }
  }
  o->master.stride(pop);
  return SG_OK;
}
int32_t or_eigen_cycle(or_handle h, int32_t admin, int32_t atch, sg_cycle_stats* st) {
  Oracle* o = O(h);
  double startW = 0; for (auto& s : o->thisCycle) startW += s.wgt;
  o->reportCycleStart(admin, startW);
  std::vector<orc::PState> next;
  int rc = o->transportBank(admin, o->thisCycle, o->master.s, o->k_new, next);
  if (rc) return rc;
  int n = (int)o->thisCycle.size();
  o->master.stride(o->pop + 1);                       // :257
  double endW = 0; for (auto& s : next) endW += s.wgt;
  o->reportCycleEnd(admin, endW, o->nextK);            // :261 (end%k_eff = k used this cycle)
  if (next.empty()) { o->err = "empty fission bank"; return SG_ERR_STATE; }
  o->normSizeRepr(next, o->pop, o->master);            // :269
  o->master.stride(1);                                 // :275
  o->thisCycle.swap(next);                             // flip
  double k = o->k_new, sd = 0.0;
  o->getKeff(atch, k, sd);                             // :289-298
  double kUsed = o->k_new;
  o->k_new = k;
  o->nextK = k;                                        // nextCycle%k_eff = k_new
  if (st) {
    st->n_histories = n; st->n_events = o->nEvents; st->n_collisions = o->nColl; st->n_next = (int64_t)o->thisCycle.size();
    st->start_weight = startW; st->end_weight = endW; st->k_eff = kUsed; st->k_new = k;
  }
  return SG_OK;
}
// The same eigenvalue cycle as SCONE's OpenMP build runs it (eigenPhysicsPackage_class.f90:203-338):
// the gen loop over histories with dynamic scheduling on `threads` threads, each with private
// operators and private score memory (scoreMemory's per-thread parallelBins, scoreMemory_class.f90
// :215-233, summed into the shared bins at the cycle end), fission sites detained per thread and
// then ordered by brood ID (particleDungeon%sortByBroodID, particleDungeon_class.f90:923-981); the
// rest of the cycle (reportCycleEnd, normSize_Repr, k feedback) on the master thread.  The banks,
// RNG states and k equal or_eigen_cycle's; the tally sums differ only in their order.  CPU
// baseline of the bench, not used by the parity tests.
int32_t or_eigen_cycle_omp(or_handle h, int32_t admin, int32_t atch, int32_t threads, sg_cycle_stats* st) {
  Oracle* o = O(h);
  double startW = 0; for (auto& s : o->thisCycle) startW += s.wgt;
  o->reportCycleStart(admin, startW);
  const int n = (int)o->thisCycle.size();
  std::vector<orc::PState> bank;
  bank.swap(o->thisCycle);                            // kept out of the thread-private copies
  o->recColl.clear(); o->recRng.clear();
  const uint64_t master = o->master.s;
  const double k = o->k_new;
  std::vector<int> count(n + 1, 0);
  std::vector<std::vector<int>> tHist;
  std::vector<std::vector<orc::PState>> tSites;
  int64_t ev = 0, coll = 0;
  std::string err;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel reduction(+:ev, coll)
  {
    Oracle local = *o;
    for (auto& A : local.admins) std::fill(A.mem.parallel.begin(), A.mem.parallel.end(), 0.0);
    local.nEvents = 0; local.nColl = 0;
    std::vector<int> myHist;
    std::vector<orc::PState> mySites;
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i) {
      std::vector<orc::PState> s;
      local.runHistory(bank[i], i + 1, master, k, admin, &s, nullptr, nullptr);
      for (auto& x : s) { myHist.push_back(i + 1); mySites.push_back(x); }
    }
    ev += local.nEvents;
    coll += local.nColl;
#pragma omp critical
    {
      for (size_t a = 0; a < o->admins.size(); ++a) {
        auto& P = o->admins[a].mem.parallel;
        const auto& Q = local.admins[a].mem.parallel;
        for (size_t i = 0; i < P.size(); ++i) P[i] += Q[i];
      }
      if (!local.err.empty()) err = local.err;
      tHist.emplace_back(std::move(myHist));
      tSites.emplace_back(std::move(mySites));
    }
  }
  o->nEvents = ev; o->nColl = coll;
  if (!err.empty()) { o->err = err; bank.swap(o->thisCycle); return SG_ERR_LOST; }
  // sortByBroodID: a counting sort by history, each history's sites in their detain order
  for (const auto& v : tHist) for (int b : v) count[b] += 1;
  std::vector<int> pos(n + 2, 0);
  for (int i = 1; i <= n; ++i) pos[i + 1] = pos[i] + count[i];
  std::vector<orc::PState> next((size_t)pos[n + 1]);
  for (size_t t = 0; t < tHist.size(); ++t)
    for (size_t j = 0; j < tHist[t].size(); ++j) next[pos[tHist[t][j]]++] = tSites[t][j];
  o->master.stride(o->pop + 1);                       // :257
  double endW = 0; for (auto& s : next) endW += s.wgt;
  o->reportCycleEnd(admin, endW, o->nextK);            // :261
  if (next.empty()) { o->err = "empty fission bank"; return SG_ERR_STATE; }
  o->normSizeRepr(next, o->pop, o->master);            // :269
  o->master.stride(1);                                 // :275
  o->thisCycle.swap(next);
  double kn = o->k_new, sd = 0.0;
  o->getKeff(atch, kn, sd);                            // :289-298
  double kUsed = o->k_new;
  o->k_new = kn;
  o->nextK = kn;
  if (st) {
    st->n_histories = n; st->n_events = ev; st->n_collisions = coll; st->n_next = (int64_t)o->thisCycle.size();
    st->start_weight = startW; st->end_weight = endW; st->k_eff = kUsed; st->k_new = kn;
  }
  return SG_OK;
}
int32_t or_eigen_state(or_handle h, uint64_t* master, double* k) { *master = O(h)->master.s; *k = O(h)->k_new; return SG_OK; }
int32_t or_eigen_get_bank(or_handle h, sg_bank* out, int32_t cap, int32_t* pop) {
  Oracle* o = O(h);
  *pop = (int32_t)o->thisCycle.size();
  statesToBank(o->thisCycle, out, cap);
  return SG_OK;
}

// fixedSourcePhysicsPackage%cycles, one batch (fixedSourcePhysicsPackage_class.f90:183-289)
// fixedSourcePhysicsPackage%cycles, one cycle of this process's share n of `total` histories
// (fixedSourcePhysicsPackage_class.f90:183-289): the master is strided by the total population
// after the source and after the gen loop; `master` enters already strided by the process's offset
// (getOffset, mpi_func.f90:143-159).
int32_t or_fixed_source_cycle_shard(or_handle h, int32_t admin, int32_t n, int32_t total, uint64_t* master,
                                    sg_cycle_stats* st) {
  Oracle* o = O(h);
  std::vector<orc::PState> bank(n), next;
  for (int i = 1; i <= n; ++i) {
    orc::RNG r; r.s = *master; r.stride(i);
    if (o->fileSrc.empty()) bank[i - 1] = o->samplePoint(r);
    else {
      int rc = o->sampleFile(r, bank[i - 1]);
      if (rc) { o->err = "file source: particle outside the geometry or in an undefined cell"; return rc; }
    }
  }
  orc::RNG m; m.s = *master; m.stride(total);
  o->reportCycleStart(admin, (double)n);
  int rc = o->transportBank(admin, bank, m.s, 1.0, next);
  m.stride(total);
  o->reportCycleEnd(admin, 0.0, 1.0);
  *master = m.s;
  if (st) { st->n_histories = n; st->n_events = o->nEvents; st->n_collisions = o->nColl; st->n_next = (int64_t)next.size(); }
  return rc;
}
int32_t or_fixed_source_cycle(or_handle h, int32_t admin, int32_t n, uint64_t* master, sg_cycle_stats* st) {
  return or_fixed_source_cycle_shard(h, admin, n, n, master, st);
}

// ---- unit-test probes
int32_t or_rng_draws(uint64_t* state, double* out, int32_t n) {
  orc::RNG r; r.s = *state;
  for (int i = 0; i < n; ++i) out[i] = r.get();
  *state = r.s;
  return SG_OK;
}
uint64_t or_rng_skip(uint64_t state, int64_t k) { orc::RNG r; r.s = state; r.skip(k); return r.s; }

int32_t or_surf_eval(int32_t type, const double* par, const int32_t* bc, const double* r, const double* u,
                     double* out /* [evaluate, distance, halfspace, going, tol] */) {
  orc::Surface s; s.build(type, par);
  if (bc) for (int i = 0; i < 6; ++i) s.bc[i] = bc[i];
  out[0] = s.evaluate(r); out[1] = s.distance(r, u); out[2] = s.halfspace(r, u) ? 1.0 : 0.0;
  out[3] = s.going(r, u) ? 1.0 : 0.0; out[4] = s.tol;
  return SG_OK;
}
int32_t or_surf_bc(int32_t type, const double* par, const int32_t* bc, int32_t transform, double* r, double* u) {
  orc::Surface s; s.build(type, par);
  for (int i = 0; i < 6; ++i) s.bc[i] = bc[i];
  if (transform) s.transformBC(r, u); else s.explicitBC(r, u);
  return SG_OK;
}
int32_t or_coords_init(or_handle h, const double* r, const double* u) {
  Oracle* o = O(h); o->probe = orc::CoordList(); o->probe.init(r, u); o->probeCache = orc::distCache(); return SG_OK;
}
int32_t or_coords_place(or_handle h) { O(h)->geom.placeCoord(O(h)->probe); return SG_OK; }
int32_t or_coords_move(or_handle h, int32_t mode, double* maxDist, int32_t* event) {
  // mode 0: move_noCache, 1: move_withCache, 2: geometry moveGlobal, 3: teleport
  Oracle* o = O(h); int ev = 0;
  if (mode == 0) o->geom.move(o->probe, *maxDist, ev, nullptr);
  else if (mode == 1) o->geom.move(o->probe, *maxDist, ev, &o->probeCache);
  else if (mode == 2) o->geom.moveGlobalGeom(o->probe, *maxDist, ev);
  else o->geom.teleport(o->probe, *maxDist);
  *event = ev;
  return SG_OK;
}
int32_t or_coords_get(or_handle h, int32_t level, double* r, double* u, int32_t* info /* nesting, matIdx, uniqueID, localID, uniIdx */) {
  Oracle* o = O(h);
  const orc::Coord& c = o->probe.lvl[level];
  for (int i = 0; i < 3; ++i) { r[i] = c.r[i]; u[i] = c.dir[i]; }
  info[0] = o->probe.nesting; info[1] = o->probe.matIdx; info[2] = o->probe.uniqueID; info[3] = c.localID; info[4] = c.uniIdx;
  return SG_OK;
}
int32_t or_what_is_at(or_handle h, const double* r, const double* u, int32_t* mat, int32_t* uid) {
  int m, id; O(h)->geom.whatIsAt(m, id, r, u); *mat = m; *uid = id; return SG_OK;
}
int32_t or_bounds(or_handle h, double* bb) { O(h)->geom.bounds(bb); return SG_OK; }
int32_t or_mg_info(or_handle h, int32_t mat, int32_t G, double* out /* total scatter capture fission nuFission majorant */) {
  Oracle* o = O(h);
  size_t k = (size_t)(mat - 1) * o->mg.nG + (G - 1);
  out[0] = o->mg.total[k]; out[1] = o->mg.scatter[k]; out[2] = o->mg.capture[k];
  out[3] = o->mg.fission[k]; out[4] = o->mg.nuFission[k]; out[5] = o->mg.majorant[G - 1];
  return SG_OK;
}
int32_t or_rotate_vector(const double* dir, double mu, double phi, double* out) { orc::rotateVector(dir, mu, phi, out); return SG_OK; }

// scoreMemory probe: replays the reference scoreMemory unit test pattern
int32_t or_scoremem_new(int64_t n, int32_t batch, or_handle* out) {
  orc::ScoreMemory* m = new orc::ScoreMemory(); m->init(n, batch); *out = reinterpret_cast<or_handle>(m); return SG_OK;
}
int32_t or_scoremem_free(or_handle h) { delete reinterpret_cast<orc::ScoreMemory*>(h); return SG_OK; }
int32_t or_scoremem_score(or_handle h, double s, int64_t idx) { reinterpret_cast<orc::ScoreMemory*>(h)->score(s, idx); return SG_OK; }
int32_t or_scoremem_accumulate(or_handle h, double s, int64_t idx) { reinterpret_cast<orc::ScoreMemory*>(h)->accumulate(s, idx); return SG_OK; }
int32_t or_scoremem_reduce(or_handle h) { reinterpret_cast<orc::ScoreMemory*>(h)->reduceBins(); return SG_OK; }
int32_t or_scoremem_closebin(or_handle h, double f, int64_t idx) { reinterpret_cast<orc::ScoreMemory*>(h)->closeBin(f, idx); return SG_OK; }
int32_t or_scoremem_closecycle(or_handle h, double f) { reinterpret_cast<orc::ScoreMemory*>(h)->closeCycle(f); return SG_OK; }
int32_t or_scoremem_close(or_handle h, double f) {
  orc::ScoreMemory* m = reinterpret_cast<orc::ScoreMemory*>(h); m->reduceBins(); m->closeCycle(f); return SG_OK;
}
int32_t or_scoremem_result(or_handle h, int64_t idx, int32_t samples, double* mean, double* sd) {
  reinterpret_cast<orc::ScoreMemory*>(h)->getResult(*mean, *sd, idx, samples); return SG_OK;
}

// CPU baseline: the gen loop with OpenMP over histories (thread-private tallies merged after the
// loop, sites concatenated in history order).  Returns histories processed; tallies discarded.
int64_t or_timed_gen_loop(or_handle h, int32_t admin, const sg_bank* in, int32_t n, uint64_t master,
                          double k, int32_t threads, int64_t* events) {
  Oracle* o = O(h);
  std::vector<orc::PState> v;
  bankToStates(in, n, v);
  int64_t ev = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel reduction(+:ev)
  {
    Oracle local = *o;   // thread-private operators, RNG and tallies (eigenPhysicsPackage :181)
    local.nEvents = 0;
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i) {
      std::vector<orc::PState> s;
      local.runHistory(v[i], i + 1, master, k, admin, &s, nullptr, nullptr);
    }
    ev += local.nEvents;
  }
#else
  (void)threads;
  for (int i = 0; i < n; ++i) { std::vector<orc::PState> s; o->runHistory(v[i], i + 1, master, k, admin, &s, nullptr, nullptr); }
  ev = o->nEvents;
#endif
  if (events) *events = ev;
  return n;
}

}  // extern "C"
