// sg_internal.h -- device data records shared by the kernels and the host side of libsconegpu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/scone_gpu.h"

namespace sg {

// One surface: 64-bit params as uploaded (plane coefficients normalised), tolerance of the
// precision form the record was built for, boundary conditions (border surface only).
// The FP32 copies (pf, tolf) serve the mixed form at nesting levels below the root, where positions
// are local FP32 coordinates.
struct DSurf {
  int type;
  int axis;        // aPlane axis / cylinder axis
  int pl0, pl1;    // in-plane axes of cylinders and square cylinders
  int bc[6];
  int pad[2];
  double p[SG_SURF_NPAR];
  double tol;
  float pf[SG_SURF_NPAR];
  float tolf;
  float filt;      // mixed form, root border: |FP32 value| above this decides the halfspace (0: none)
};

// One universe.  i[] / d[] by type:
//   ROOT: i0 border surface
//   CELL: i0 first entry in uni_cells, i1 number of cells
//   PIN : i0 first annulus in pin_rsq/pin_tol, i1 number of annuli (last one has radius 1.1*INF)
//   LAT : i0..i2 sizeN, i3 outLocalID, i4 outline surface, i5 offset flag;
//         d0..2 pitch, d3..5 corner, d6..8 a_bar (half pitch reduced by the surface tolerance);
//         invf0..2 1 / pitch and invn0..1 1 / sizeN (FP32)
//   all : i6 = 1 when the origin is (0, 0, 0)
struct DUni {
  int type;
  int i[7];
  int rot;         // 1: rotated (universe `rotation`); its matrix is DGeom::rot[9 * index]
  double origin[3];
  double d[9];
  float originf[3];
  float f[9];      // FP32 copy of d
  float invf[3];   // lattice: 1 / pitch (mixed-form cell search)
  float invn[2];   // lattice: 1 / sizeN[0], 1 / sizeN[1] (local ID -> ijk)
};

struct DGeom {
  const DSurf* surfs;
  const DUni* unis;
  const int* uni_cells;
  const int* cell_ptr;
  const int* cell_surf;
  const double* pin_rsq;
  const double* pin_tol;
  const float* pin_rsqf;  // FP32 copies (mixed form)
  const float* pin_tolf;
  const int2* graph;    // geomGraph: x = matIdx (>= 0) or -(uniIdx), y = uniqueID or uniRootID (1-based)
  int root;             // root universe (0-based)
  int border;           // border surface (0-based)
  double nudge;         // cellUniverse crossing nudge of the precision form
  double tie_abs;       // absolute part of the tie rule between nesting levels (0 in the FP64 form)
  const int* cell_complex;  // [n_cell] 1: unionCell with unions (cell_surf holds its evaluation array)
  const double* rot;        // [n_uni][9] row-major rotation matrices; null when no universe is rotated
  const float* rotf;        // FP32 copy
};

// unionCell evaluation tokens in cell_surf (surfaces are signed 1-based indices); OPEN, CLOSE and
// UNION are the input codes, INTERSECT is inserted where SCONE's input leaves it implicit
static constexpr int CELL_OPEN = SG_CELL_OPEN, CELL_CLOSE = SG_CELL_CLOSE, CELL_UNION = SG_CELL_UNION;
static constexpr int CELL_INTERSECT = -2147483643;
__host__ __device__ inline bool cell_is_op(int t) { return t <= CELL_INTERSECT && t >= CELL_OPEN; }

// MG macroscopic data in the working precision R ([mat][G], P0/prod [mat][Gin][Gout])
template <class R>
struct DMG {
  int nMat, nG;
  const R* total;
  const R* scatter;
  const R* capture;
  const R* fission;
  const R* nuFission;
  const R* chi;
  const R* P0;
  const R* prod;
  const int* fissile;
  const R* majorant;
  R collisionXS;
  const R* P1n;         // [mat][Gin][Gout] 3 P1/P0 (multiScatterP1MG), null for P0 scattering
  const R* majInv;      // [G] 1 / max(majorant, collisionXS)
};

// Continuous-energy neutron data (aceNeutronNuclide mainData / eGrid, ceNeutronMaterial composition,
// aceNeutronDatabase unionised majorant).  Energy grids stay FP64 in both forms (the floor index is
// the reference's exactly); cross sections, densities, masses and temperatures are in R.
// Grid searches start from a hash over log(E): bin b of a nuclide (or of the union grid) holds the
// bracket (lo, hi) of grid indices that contains every energy of that bin, widened by a margin
// so that the FP32 log used to pick the bin cannot miss; a short binary search finishes it.
template <class R>
struct DCE {
  int nNuc, nMat;
  const double* e;          // all nuclide grids, concatenated
  const R* xs;              // [point][4] total, elastic, inelastic, capture
  const long long* off;     // [nNuc+1] first point of each nuclide
  const int2* hash;         // [nNuc][nHash] nuclide-relative brackets
  int nHash;
  float hLogMin, hInvStep;  // bin = floor((log E - hLogMin) * hInvStep), clamped
  const R* A;               // [nNuc] mass ratio
  const R* kT;              // [nNuc] nuclide temperature [MeV]
  const int* matPtr;        // [nMat+1]
  const int* matNuc;        // 0-based nuclide indices in composition order
  const R* matDens;         // atom densities
  // unionised majorant (aceNeutronDatabase%majorant) or the active materials (on-the-fly majorant)
  int hasMajorant;
  const double* ue;         // union grid
  const R* umaj;            // majorant values on it
  const int2* uhash;
  int nU, nUHash;
  float uLogMin, uInvStep;
  const int* act;           // active materials (1-based), for the on-the-fly majorant
  int nAct;
  // lookup acceleration: the union of every nuclide's grid and, per union point, each nuclide's
  // floor index there ([nLU][nNuc], -1 below the nuclide's grid); null when not built
  const double* lu;
  const int* lidx;
  const int* lmaj;          // [nLU] floor index of each union point in the majorant grid ue (-1 below)
  const int2* luhash;
  int nLU, nLUHash;
  float luLogMin, luInvStep;
  double minE;              // neutronCEstd minEnergy cut-off
  R threshE, threshA;       // free-gas thresholds
  R collisionXS;
};

// One tally clerk as the kernels see it (all admins of a launch flattened; acc offsets global).
struct DClerk {
  int type;
  int handle_virtual;
  int width;
  int resp[4];
  int n_axes;
  int ax_kind[3];
  int ax_n[3];
  int g_top, g_low;
  int pad;
  double ax_min[3];
  double ax_step[3];
  double ax_inv_step[3];
  float ax_minf[3];
  float ax_inv_stepf[3];
  long long multi[3];
  long long acc_off;     // offset (0-based) of this clerk's first bin in the launch's acc array
  long long nbins;       // map bins (surface-current clerks: per plane and direction)
  int cur_axis;          // surface-current clerk: 0..2 normal of the planes
  int n_planes;
  double planes[8];
  int ax_grid[3];        // SG_GRID_LIN / LOG / UNSTRUCT of space and energy axes
  const void* ax_tab[3]; // unstructured grid: n+1 bounds (double in the FP64 form, float in the mixed
                         // form); cell axis: int bin of every global cell index + 1 ([0]: no cell)
};

static constexpr int MAX_CLERKS = 8;

// SoA particle bank in device memory
struct DBank {
  double* r;       // [n][3]
  double* dir;     // [n][3]
  double* wgt;
  int* G;
  int* brood;
  double* time;
  double* E;       // CE energy (null for MG)
};

// Fission sites produced by one gen loop before they are ordered by brood ID.  The buffer is split
// into up to SITE_REGIONS regions, each filled through its own atomic cursor, so the append rate is
// not limited by one contended counter.  A warp appends to region (warp index & region_mask):
// region_mask = SITE_REGIONS - 1 spreads the appends over every region, 0 puts every site in
// region 0 (one cursor, the whole buffer as its capacity).
static constexpr int SITE_REGIONS = 64;
struct DSites {
  double* r;
  double* dir;
  double* wgt;
  int* G;
  int* brood;
  int* seq;
  double* time;
  int* cursor;          // [SITE_REGIONS]
  int region_cap;
  int region_mask;      // SITE_REGIONS - 1, or 0 for a single region
};

// Per-launch counters written by the transport kernel
struct DCounters {
  unsigned long long events;
  unsigned long long collisions;
  int work;             // next history to hand out
  int err_code;         // first error (SG_ERR_*), 0 if none
  int err_hist;         // history that raised it
  int pad;
};

// Particle state between the event kernels, component-major SoA of capacity `cap` (slot = bank index).
template <class R>
struct DPart {
  double* r0;      // [3][cap]  level-1 (global) position
  R* rl;           // [3*(MAXL-1)][cap] local positions below the root
  R* u;            // [3][cap]
  int* geo;        // [3*MAXL+3][cap] universe, graph base, local ID per level; nesting, material, unique ID
  unsigned long long* rng;
  R* w;
  R* w0;
  R* time;
  R* trackXS;
  int* ints;       // [5][cap] G, collisionN, history, sites written, segments
  double* E;       // [cap] CE energy
  int cap;
};

// Work queues of the event form: slots of particles awaiting transit or collision.
struct DQueues {
  const int* in;
  const int* n_in;
  int* out;
  int* n_out;
  int* work;       // next entry of `in` to hand out (persistent kernels)
};

// transport operators as compiled kernel variants
enum { OP_ST = 0, OP_DT = 1, OP_HT = 2 };
inline int transport_op(int transport) {
  if (transport == SG_TRANSPORT_DT) return OP_DT;
  if (transport == SG_TRANSPORT_HT || transport == SG_TRANSPORT_HT_NOCACHE) return OP_HT;
  return OP_ST;
}
inline bool transport_cache(int transport) {
  return transport != SG_TRANSPORT_ST_NOCACHE && transport != SG_TRANSPORT_HT_NOCACHE;
}

// neutronMGimp / neutronCEimp options and the weight-window field, in device memory (read at
// collisions only).  The split buffer holds `depth` particles per thread of the launch.
template <class R>
struct DColl {
  int imp_abs, roulette, split, ww, max_split;
  R min_wgt, max_wgt, av_wgt;
  DClerk ww_map;             // weightWindowsField map (axes only)
  const R* ww_lower;         // [bins]
  const R* ww_upper;
  R ww_cs;                   // constSurvival
  // split buffer: entry (thread, j) at thread * depth + j
  double* b_r;               // [3]
  R* b_u;                    // [3]
  R* b_w;
  double* b_E;
  int* b_G;
  R* b_time;
  int depth;
};

template <class R>
struct TransportArgs {
  DGeom geom;
  DMG<R> mg;
  DCE<R> ce;
  DBank in;
  int n;
  unsigned long long master;
  const double* k_eff;
  DClerk clerks[MAX_CLERKS];
  int n_clerks;
  int keff_clerk;       // index of the keff-implicit clerk (accumulated in registers), -1 if none
  int has_current;      // a surface-current clerk is present
  int has_cellmap;      // some clerk maps by cell
  double* acc;          // tally accumulators of the launch (global)
  int acc_n;
  int use_smem;         // accumulate map clerks in shared memory
  DSites sites;
  int* hist_nsites;     // [n] sites per history (0 when no fission)
  int* rec_coll;        // [n] or null
  unsigned long long* rec_rng;  // [n] or null
  DCounters* ctr;
  int use_cache;        // transportOperatorST cache flag
  int max_segments;     // safety limit per history
  R ht_cutoff;          // transportOperatorHT `cutoff`
  DPart<R> part;        // event form: particle state
  DQueues q;            // event form: queues of the launch
  int coll_imp;         // 1: neutronMGimp / neutronCEimp with *coll
  const DColl<R>* coll;
  int lean;             // 1: no rotated universe, cell map, current clerk, coll_imp or P1 scattering
                        // (multigroup): the history loop runs its lean instantiation
};

// Where the history loop scores map clerks.  Few bins: a block-local copy of score memory in shared
// memory, flushed once per block (global reductions on a handful of addresses serialise in L2:
// 2.5-6x slower on the 2-group infinite medium).  Many bins: straight into global memory (L2
// reductions spread over the bins cost less than shared-memory FP64 atomics: 7 % on the 2 023-bin
// lattice mesh).
inline bool scores_in_shared_memory(long long acc_n) { return acc_n > 0 && acc_n < 1024; }

}  // namespace sg
