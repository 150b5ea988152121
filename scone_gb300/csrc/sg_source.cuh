// sg_source.cuh -- source sampling kernels (ParticleObjects/Source).
#pragma once
#include "sg_device.cuh"

namespace sg {

struct FissionSourceArgs {
  DGeom geom;
  DMG<double> mg;
  DBank out;
  int n;
  unsigned long long master;
  double bounds[6];
  int* err;
};

// fissionSource%sampleParticle (fissionSource_class.f90:149-271), MG data, G = 1, 10000 attempts.
// Particle i (1-based) uses master + stride(i) (source_inter.f90:98-119).
template <int MAXL>
__global__ void __launch_bounds__(128) k_fission_source(const __grid_constant__ FissionSourceArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  Rng<double> rng;
  rng.s = lcg_skip(a.master, RNG_STRIDE * (long long)(i + 1));
  Geom<double, MAXL> geom(a.geom);
  for (int att = 0; att < 10000; ++att) {
    double x0 = rng.get(), x1 = rng.get(), x2 = rng.get();
    Coords<double, MAXL> c;
    c.r0[0] = (a.bounds[3] - a.bounds[0]) * x0 + a.bounds[0];
    c.r0[1] = (a.bounds[4] - a.bounds[1]) * x1 + a.bounds[1];
    c.r0[2] = (a.bounds[5] - a.bounds[2]) * x2 + a.bounds[2];
    const double rs[3] = {c.r0[0], c.r0[1], c.r0[2]};
    c.u[0] = 1.0; c.u[1] = 0.0; c.u[2] = 0.0;
    geom.place(c);
    const int mat = c.mat;
    if (mat == SG_VOID_MAT || mat == 0) continue;
    if (mat == SG_UNDEF_MAT || mat == SG_OVERLAP_MAT) { atomicCAS(a.err, 0, SG_ERR_UNDEF_MAT); return; }
    if (!a.mg.fissile[mat - 1]) continue;
    double mu = 2.0 * rng.get() - 1.0;                  // fissionMG%sampleOut (fissionMG_class.f90:183-206)
    double sp, cp;
    sincos_phi<double>(rng.get(), sp, cp);
    double rem = rng.get();
    int g;
    for (g = 1; g <= a.mg.nG; ++g) {
      rem = rem - a.mg.chi[(mat - 1) * a.mg.nG + (g - 1)];
      if (rem < 0.0) break;
    }
    double d0 = 1.0, d1 = 0.0, d2 = 0.0;
    rotate_vector<double>(d0, d1, d2, mu, sp, cp);
    a.out.r[3 * i + 0] = rs[0]; a.out.r[3 * i + 1] = rs[1]; a.out.r[3 * i + 2] = rs[2];
    a.out.dir[3 * i + 0] = d0; a.out.dir[3 * i + 1] = d1; a.out.dir[3 * i + 2] = d2;
    a.out.wgt[i] = 1.0;
    a.out.G[i] = g;
    a.out.brood[i] = 0;
    a.out.time[i] = 0.0;
    return;
  }
  atomicCAS(a.err, 0, SG_ERR_STATE);
}

// fileSource%sampleParticle (fileSource_class.f90:146-190): particle i (1-based) takes entry
// int(xi N) + 1 of the table, xi the first draw of master + stride(i); the entry must lie inside the
// geometry (whatIsAt), as the reference checks.
struct FileSourceArgs {
  DGeom geom;
  const double* r;      // [N][3]
  const double* dir;    // [N][3]
  const double* wgt;    // [N]
  const double* E;      // [N] (CE) or null
  const int* G;         // [N] (MG) or null
  long long N;
  DBank out;
  int n;
  unsigned long long master;
  int* err;
};

template <int MAXL>
__global__ void __launch_bounds__(128) k_file_source(const __grid_constant__ FileSourceArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  Rng<double> rng;
  rng.s = lcg_skip(a.master, RNG_STRIDE * (long long)(i + 1));
  const long long idx = (long long)(rng.get() * (double)a.N) + 1;
  if (idx > a.N) { atomicCAS(a.err, 0, SG_ERR_STATE); return; }
  const long long j = idx - 1;
  Geom<double, MAXL> geom(a.geom);
  Coords<double, MAXL> c;
  for (int k = 0; k < 3; ++k) c.r0[k] = a.r[3 * j + k];
  c.u[0] = 1.0; c.u[1] = 0.0; c.u[2] = 0.0;          // whatIsAt without a direction (geometryStd :163-168)
  geom.place(c);
  if (c.mat == 0 || c.mat == SG_UNDEF_MAT) { atomicCAS(a.err, 0, SG_ERR_UNDEF_MAT); return; }
  for (int k = 0; k < 3; ++k) { a.out.r[3 * i + k] = a.r[3 * j + k]; a.out.dir[3 * i + k] = a.dir[3 * j + k]; }
  a.out.wgt[i] = a.wgt[j];
  a.out.G[i] = a.G ? a.G[j] : 0;
  if (a.out.E) a.out.E[i] = a.E ? a.E[j] : 0.0;
  a.out.brood[i] = 0;
  a.out.time[i] = 0.0;
}

}  // namespace sg
