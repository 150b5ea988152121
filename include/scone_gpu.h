/*
 * scone_gpu.h -- C ABI of libsconegpu, a GB300 (sm_103a) implementation of SCONE's
 * Monte Carlo particle-tracking cycle.
 *
 * The ABI is what a Fortran physicsPackage binds with ISO_C_BINDING: plain pointers,
 * sizes and int32 status codes, no C++ or torch types.  Every entry point returns
 * SG_OK (0) or a negative SG_ERR_* code; sg_last_error() gives the message.
 *
 * Conventions shared with SCONE (so arrays can be passed straight from the Fortran side):
 *   - material indices are 1-based (matIdx); 0 is OUTSIDE_MAT, 2147483647 is VOID_MAT
 *     (SharedModules/universalVariables.f90:45-48);
 *   - a cell/universe fill is matIdx (>= 0) or -uniIdx (1-based universe index)
 *     (Geometry/Universes/universe_inter.f90:477-507);
 *   - energy groups are 1-based; the MG scattering matrix P0 is stored with the incident
 *     group as the row, exactly as in an MG xsFile (multiScatterMG_class.f90:321-336);
 *   - bins of one tally admin are returned as SCONE's scoreMemory `bins(N,{BIN,CSUM,CSUM2})`,
 *     Fortran column-major (Tallies/scoreMemory_class.f90:16-18,87-97).
 *
 * The library is one handle per GPU stream; a handle is not thread-safe and is called from
 * the master thread (outside `!$omp parallel`).
 */
#ifndef SCONE_GPU_H
#define SCONE_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define SG_OK              0
#define SG_ERR_BAD_ARG    -1
#define SG_ERR_OOM        -2
#define SG_ERR_BANK_OVERFLOW -3
#define SG_ERR_UNDEF_MAT  -4
#define SG_ERR_OVERLAP    -5
#define SG_ERR_NAN        -6
#define SG_ERR_TIMEOUT    -7
#define SG_ERR_CUDA       -8
#define SG_ERR_STATE      -9
#define SG_ERR_LOST      -10

/* ---------------------------------------------------------------- constants */
#define SG_MAX_NEST       12      /* HARDCODED_MAX_NEST, universalVariables.f90:10 */
#define SG_SURF_NPAR       6
#define SG_VOID_MAT       2147483647
#define SG_UNDEF_MAT      2147483646
#define SG_OVERLAP_MAT    2147483645

/* surface types (Geometry/Surfaces) */
#define SG_SURF_XPLANE     1      /* aPlane_class.f90   par: a0                          */
#define SG_SURF_YPLANE     2
#define SG_SURF_ZPLANE     3
#define SG_SURF_PLANE      4      /* plane_class.f90    par: c1 c2 c3 c4 (normalised here) */
#define SG_SURF_XCYL       5      /* cylinder_class.f90 par: ox oy oz r                  */
#define SG_SURF_YCYL       6
#define SG_SURF_ZCYL       7
#define SG_SURF_SPHERE     8      /* sphere_class.f90   par: ox oy oz r                  */
#define SG_SURF_BOX        9      /* box_class.f90      par: ox oy oz hx hy hz           */
#define SG_SURF_XSQCYL    10      /* squareCylinder_class.f90 par: ox oy oz hx hy hz     */
#define SG_SURF_YSQCYL    11
#define SG_SURF_ZSQCYL    12

/* universe types (Geometry/Universes) */
#define SG_UNI_ROOT        1      /* ipar: border surface (0-based)        fills: [inside]        */
#define SG_UNI_CELL        2      /* ipar: cell indices (0-based)          fills: one per cell    */
#define SG_UNI_PIN         3      /* dpar: finite radii, ascending         fills: n_radii + 1     */
#define SG_UNI_LAT         4      /* ipar: nx ny nz(0 = 2D) offset(0/1)    dpar: px py pz
                                     fills: nx*ny*nz in local-ID order (x fastest, y, z) + pad   */

/* unionCell operators in a cell's surface list (Geometry/Cells/unionCell_class.f90:80-225): '<', '>',
 * ':' (union) and '#' (complement); intersections stay implicit, as in SCONE's input */
#define SG_CELL_OPEN       (-2147483647)
#define SG_CELL_CLOSE      (-2147483646)
#define SG_CELL_UNION      (-2147483645)
#define SG_CELL_COMPLEMENT (-2147483644)

/* boundary conditions (universalVariables.f90:57-59) */
#define SG_BC_VACUUM       0
#define SG_BC_REFLECTIVE   1
#define SG_BC_PERIODIC     2

/* precision forms */
#define SG_PREC_FP64       0      /* all-FP64 verification mode                                  */
#define SG_PREC_MIXED      1      /* FP32 XS/distances/sampling, FP64 positions and tally sums   */

/* execution forms of the gen loop */
#define SG_FORM_EVENT      0      /* event-based: transit / collision kernels over compacted queues */
#define SG_FORM_HISTORY    1      /* one persistent history-loop kernel                          */

/* transport operators (transportOperatorFactory_func.f90:48-60) */
#define SG_TRANSPORT_ST    1      /* transportOperatorST, distance cache on                      */
#define SG_TRANSPORT_DT    2      /* transportOperatorDT                                         */
#define SG_TRANSPORT_ST_NOCACHE 3 /* transportOperatorST { cache 0; }                           */
#define SG_TRANSPORT_HT    4      /* transportOperatorHT (hybrid: DT or ST chosen per transit)   */
#define SG_TRANSPORT_HT_NOCACHE 5 /* transportOperatorHT { cache 0; }                           */

/* tally clerks (Tallies/TallyClerks) */
#define SG_CLERK_COLLISION      1 /* collisionClerk_class.f90                                    */
#define SG_CLERK_TRACK          2 /* trackClerk_class.f90                                        */
#define SG_CLERK_KEFF_ANALOG    3 /* keffAnalogClerk_class.f90  (3 bins)                         */
#define SG_CLERK_KEFF_IMPLICIT  4 /* keffImplicitClerk_class.f90 (5 bins)                        */
#define SG_CLERK_SURFACE_CURRENT 5 /* no SCONE counterpart: weight crossing planes normal to an axis,
                                      bins [plane][map bin][direction -,+] (direction fastest)     */

/* tally map axes (Tallies/TallyMaps) */
#define SG_AXIS_X          1      /* spaceMap axis x, lin grid                                   */
#define SG_AXIS_Y          2
#define SG_AXIS_Z          3
#define SG_AXIS_GROUP      4      /* MG group axis (no SCONE counterpart: energyMap maps MG to 0) */
#define SG_AXIS_MATERIAL   5      /* materialMap over 1..n                                       */
#define SG_AXIS_ENERGY     6      /* energyMap, log grid over [min,max] (energyMap_class.f90:278-293,
                                     grid_class.f90:76-90,164-166); MG particles map to 0        */
#define SG_AXIS_CELL       7      /* cellMap (cellMap_class.f90:80-205): one bin per listed cell
                                     (the cell the particle is in at its lowest level); elsewhere
                                     bin n+1 with cell_rest (trackRest), else outside the map    */

/* grids of the space and energy axes (grid_class.f90:154-175): the default is lin for space axes and
 * log for the energy axis; unstructured grids take n+1 ascending bounds (a floor binary search) */
#define SG_GRID_DEFAULT    0
#define SG_GRID_LIN        1
#define SG_GRID_LOG        2
#define SG_GRID_UNSTRUCT   3

/* tally responses: 0 = fluxResponse, otherwise a macroResponse MT (endfConstants.f90:116-130) */
#define SG_RESP_FLUX       0

/* ---------------------------------------------------------------- descriptions */

typedef struct sg_geometry_desc {
  int32_t        n_surf;
  const int32_t* surf_type;     /* [n_surf]                     */
  const double*  surf_par;      /* [n_surf][SG_SURF_NPAR]       */
  int32_t        border_surf;   /* 0-based index of the root border surface  */
  int32_t        bc[6];         /* -x +x -y +y -z +z, applied to the border (geometryStd `boundary`) */
  int32_t        n_cell;
  const int32_t* cell_ptr;      /* [n_cell+1] into cell_surf    */
  const int32_t* cell_surf;     /* signed 1-based surface index (-k: -ve halfspace of surface k);
                                   a cell that also holds SG_CELL_* operator tokens is a unionCell */
  int32_t        n_uni;
  const int32_t* uni_type;      /* [n_uni]                      */
  const double*  uni_origin;    /* [n_uni][3]                   */
  const int32_t* uni_iptr;      /* [n_uni+1] into uni_ipar      */
  const int32_t* uni_ipar;
  const int32_t* uni_dptr;      /* [n_uni+1] into uni_dpar      */
  const double*  uni_dpar;
  const int32_t* uni_fptr;      /* [n_uni+1] into uni_fill      */
  const int32_t* uni_fill;      /* fills per local cell: matIdx or -uniIdx */
  int32_t        root_uni;      /* 0-based index of the root universe */
  const double*  uni_rot;       /* [n_uni][3] Euler angles (phi, theta, psi) in degrees, ZXZ convention
                                   (universe `rotation`); null: no universe is rotated */
} sg_geometry_desc;

typedef struct sg_mg_desc {     /* baseMgNeutronMaterial_class.f90:158-291, PN = P0 or P1 */
  int32_t        n_mat;
  int32_t        n_g;
  const double*  capture;       /* [n_mat][n_g]                 */
  const double*  fission;       /* [n_mat][n_g], read where fissile */
  const double*  nu;            /* [n_mat][n_g]                 */
  const double*  chi;           /* [n_mat][n_g]                 */
  const double*  p0;            /* [n_mat][n_g (in)][n_g (out)] */
  const double*  prod;          /* [n_mat][n_g (in)][n_g (out)] scatteringMultiplicity */
  const int32_t* fissile;       /* [n_mat] 0/1                  */
  double         avg_dist;      /* `avgDist`; <= 0 means none   */
  const double*  p1;            /* [n_mat][n_g (in)][n_g (out)] xsFile `P1` (baseMgNeutronMaterial
                                   `PN P1`, multiScatterP1MG_class.f90:96-128); NULL: P0 scattering */
} sg_mg_desc;

/* Continuous-energy neutron data: the part of aceNeutronDatabase / aceNeutronNuclide /
 * ceNeutronMaterial the tracking cycle reads (aceNeutronNuclide_class.f90:44-51,342-453,
 * aceNeutronDatabase_class.f90:346-808,1330-1621, ceNeutronMaterial_class.f90:338-455).
 * Nuclides are non-fissile with elastic scattering isotropic in the CM frame and no inelastic
 * channels (the ESZ-block data of an ACE card: energy grid, total, elastic, absorption). */
typedef struct sg_ce_desc {
  int32_t        n_nuc;
  const int64_t* nuc_ptr;       /* [n_nuc+1] offsets of each nuclide's points in e / xs           */
  const double*  e;             /* energy grids [MeV], ascending per nuclide                      */
  const double*  xs;            /* [point][4] mainData order: total, elastic, inelastic, capture [b] */
  const double*  A;             /* [n_nuc] mass ratio AW (neutron masses)                         */
  const double*  kT;            /* [n_nuc] nuclide temperature kT [MeV]                           */
  int32_t        n_mat;
  const int32_t* mat_ptr;       /* [n_mat+1] into mat_nuc / mat_dens                              */
  const int32_t* mat_nuc;       /* 0-based nuclide index, in composition order                    */
  const double*  mat_dens;      /* atom density [1/(barn cm)]                                     */
  int32_t        majorant;      /* 1: unionised majorant grid (aceNeutronDatabase `majorant`, default) */
  double         min_e, max_e;  /* neutronCEstd minEnergy / maxEnergy (1e-11, 20)                 */
  double         thresh_e;      /* neutronCEstd energyThreshold (400)                              */
  double         thresh_a;      /* neutronCEstd massThreshold (1)                                  */
  double         avg_dist;      /* `avgDist`; <= 0 means none                                     */
} sg_ce_desc;

typedef struct sg_axis_desc {
  int32_t kind;                 /* SG_AXIS_*                    */
  int32_t n;                    /* number of bins (cell axis: of listed cells) */
  double  min, max;             /* lin / log grid bounds        */
  int32_t grid;                 /* SG_GRID_* (space and energy axes) */
  int32_t cell_rest;            /* cell axis: 1 adds bin n+1 for every other place */
  const double*  bounds;        /* SG_GRID_UNSTRUCT: [n+1] ascending */
  const int32_t* cells;         /* SG_AXIS_CELL: [n] 0-based cell indices of the geometry */
} sg_axis_desc;

typedef struct sg_clerk_desc {
  int32_t      type;            /* SG_CLERK_*                   */
  int32_t      handle_virtual;  /* collision clerks: 1 (default) scores virtual collisions with Sigma_track */
  int32_t      n_resp;          /* 1..4                         */
  int32_t      resp[4];         /* SG_RESP_FLUX or macro MT     */
  int32_t      n_axes;          /* 0..3 (multiMap, first axis fastest) */
  sg_axis_desc axes[3];
  int32_t      filter_g_top;    /* energyFilter for MG: pass if g_top <= G <= g_low; 0 = no filter */
  int32_t      filter_g_low;
  int32_t      current_axis;    /* SG_CLERK_SURFACE_CURRENT: SG_AXIS_X/Y/Z normal of the planes */
  int32_t      n_planes;        /* SG_CLERK_SURFACE_CURRENT: 1..8 plane positions          */
  double       planes[8];
} sg_clerk_desc;

typedef struct sg_tally_desc {  /* tallyAdmin_class.f90:162-255 */
  int32_t              n_clerks;
  const sg_clerk_desc* clerks;
  int32_t              batch_size;    /* cycles per batch (>= 1) */
  int32_t              norm_clerk;    /* -1: no `norm`; else clerk index whose first bin normalises */
  double               norm_val;
} sg_tally_desc;

typedef struct sg_point_source_desc {  /* pointSource_class.f90:189-270, MG */
  double  r[3];
  double  dir[3];
  int32_t isotropic;
  int32_t G;                    /* used when n_prob_g == 0       */
  int32_t n_prob_g;
  const double* prob_g;         /* [n_prob_g]                    */
  double  E;                    /* CE source energy [MeV] (pointSource `E`), ignored for MG */
} sg_point_source_desc;

typedef struct sg_config {
  int32_t precision;            /* SG_PREC_*                     */
  int32_t transport;            /* SG_TRANSPORT_*                */
  int32_t device;               /* CUDA device ordinal           */
  int32_t max_bank;             /* capacity of each device bank (particles) */
  int32_t record_histories;     /* 1: keep per-history collision counts and end RNG states */
  int32_t form;                 /* SG_FORM_EVENT (default) or SG_FORM_HISTORY */
  double  ht_cutoff;            /* SG_TRANSPORT_HT* `cutoff`: delta tracking when Sigma_t/Sigma_maj >
                                   1 - cutoff (transportOperatorHT_class.f90:49-81); 0 = 0.9 (default) */
} sg_config;

/* A particle bank as SoA host arrays of SCONE's particleStateData (particle_class.f90:50-65).
 * Unused arrays may be NULL on input; on output every non-NULL array is written. */
typedef struct sg_bank {
  double*  wgt;                 /* [n]    */
  double*  r;                   /* [n][3] */
  double*  dir;                 /* [n][3] */
  int32_t* G;                   /* [n]    */
  double*  time;                /* [n]    */
  int32_t* brood_id;            /* [n]    */
  double*  E;                   /* [n] CE energy [MeV]; NULL for MG problems */
} sg_bank;

typedef struct sg_cycle_stats {
  int64_t n_histories;
  int64_t n_events;             /* flight segments incl. virtual collisions (device-counted) */
  int64_t n_collisions;         /* real collisions */
  int64_t n_next;               /* fission sites written to the next bank */
  double  start_weight;         /* popWeight of the transported bank */
  double  end_weight;           /* popWeight of the produced bank    */
  double  k_eff;                /* k used for this cycle              */
  double  k_new;                /* k estimate after the cycle (eigen device cycles) */
  double  transport_ms;         /* history-loop kernel time, CUDA events on the handle's stream */
  double  cycle_ms;             /* whole call, CUDA events on the handle's stream */
  int64_t n_kernels;            /* kernels launched by the call */
} sg_cycle_stats;

typedef struct sg_handle_t* sg_handle;

/* ---------------------------------------------------------------- lifetime */

/* new transportOperatorGPU: transportOperatorFactory_func.f90:36-60 + transportOperator%init */
int32_t sg_create(const sg_config* cfg, sg_handle* out);
int32_t sg_destroy(sg_handle h);
/* copies the last error message (NUL-terminated, truncated to len) */
int32_t sg_last_error(sg_handle h, char* buf, size_t len);

/* ---------------------------------------------------------------- uploads (host arrays copied) */

/* geometryStd%init: csg_class.f90:50-207 and geomGraph_class.f90:60-232 (shrunk graph) */
int32_t sg_upload_geometry(sg_handle h, const sg_geometry_desc* g);
/* baseMgNeutronDatabase%init + activate/initMajorant: baseMgNeutronDatabase_class.f90:340-503 */
int32_t sg_upload_mg(sg_handle h, const sg_mg_desc* mg);
/* aceNeutronDatabase%init + activate/initMajorant (aceNeutronDatabase_class.f90:873-1163,1291-1323): the
 * handle becomes a continuous-energy problem (replaces sg_upload_mg; banks carry E, not G). */
int32_t sg_upload_ce(sg_handle h, const sg_ce_desc* ce);
/* tallyAdmin%init: tallyAdmin_class.f90:162-255; returns an admin id */
int32_t sg_upload_tally(sg_handle h, const sg_tally_desc* t, int32_t* admin_out);
/* tallyAdmin%push: tallyAdmin_class.f90 (attachment receives every report first) */
int32_t sg_attach_tally(sg_handle h, int32_t admin, int32_t attachment);
/* pointSource%init for fixed-source runs: pointSource_class.f90 */
int32_t sg_set_point_source(sg_handle h, const sg_point_source_desc* src);

/* ---------------------------------------------------------------- cycle (host banks) */

/* source%generate (source_inter.f90:98-119): particle i uses master + stride(i), i = 1..n */
int32_t sg_generate_source(sg_handle h, uint64_t master_state, int32_t n, sg_bank* out);

/* The `gen:` history loop of fixedSource/eigenPhysicsPackage%cycles
 * (fixedSourcePhysicsPackage_class.f90:198-261, eigenPhysicsPackage_class.f90:211-252):
 * history n (1-based) of `in` starts with RNG master + stride(n), is placed, transported and
 * collided until death, scoring into tally admin `admin` (and its attachment).
 * Fission sites are returned in `next` sorted by brood ID (the order normSize_Repr sorts to);
 * `next_cap` is its capacity.  `k_eff` is the k used for fission-site weights.  An input bank in
 * page-locked host memory that the device can address is read in place by the kernels (no staging
 * copy); other host memory is copied first. */
int32_t sg_transport_bank(sg_handle h, int32_t admin, const sg_bank* in, int32_t n,
                          uint64_t master_state, double k_eff,
                          sg_bank* next, int32_t next_cap, sg_cycle_stats* stats);

/* tallyAdmin%reportCycleStart / reportCycleEnd (tallyAdmin_class.f90:672-788):
 * pop weights are popWeight() of the start and end dungeons, k_end is end%k_eff. */
int32_t sg_tally_cycle_start(sg_handle h, int32_t admin, double start_pop_weight);
int32_t sg_tally_cycle_end(sg_handle h, int32_t admin, double end_pop_weight, double k_end);

/* scoreMemory bins(N,3) column-major of one admin (N from sg_tally_size) */
int32_t sg_tally_size(sg_handle h, int32_t admin, int64_t* n_bins);
int32_t sg_get_bins(sg_handle h, int32_t admin, double* bins, int64_t n_bins);
/* keffResult of the first k clerk of an admin: mean and STD (keff clerks getResult) */
int32_t sg_get_keff(sg_handle h, int32_t admin, double* k, double* std);

/* ---------------------------------------------------------------- device-resident cycles */

/* ---------------------------------------------------------------- bank files and file sources */

/* particleDungeon%printToFile (particleDungeon_class.f90:1077-1112): particles 1..n of a bank to
 * `path` + ".bin" (binary: a stream of 10 doubles per particle: r(3), dir(3), E, G, broodID, wgt)
 * or `path` + ".txt" (the same ten numbers per line, as text).  NULL arrays write zeros (E for MG,
 * G for CE, broodID); a NULL wgt writes 1. */
int32_t sg_bank_write_file(const char* path, const sg_bank* bank, int32_t n, int32_t binary);
/* fileSource%init (fileSource_class.f90:47-144): the number of particles in such a file (`path` as
 * given, extension included), then the particles themselves into a bank of capacity cap */
int32_t sg_bank_count_file(const char* path, int32_t binary, int64_t* n);
int32_t sg_bank_read_file(const char* path, int32_t binary, sg_bank* bank, int32_t cap, int32_t* n);
/* fileSource as the source of fixed-source cycles (replaces the point source): particle i of a
 * cycle copies entry int(xi N) + 1 of these N particles, xi the first draw of master + stride(i)
 * (fileSource%sampleParticle, fileSource_class.f90:146-190); time 0; a particle outside the geometry
 * or in an undefined cell is an error.  MG problems read G, CE problems E. */
int32_t sg_set_file_source(sg_handle h, const sg_bank* particles, int32_t n);

/* fissionSource (fissionSource_class.f90:149-271) sampled on the device into the resident
 * bank: particle i uses master + stride(i); afterwards master is strided by pop
 * (eigenPhysicsPackage_class.f90:348-366). */
int32_t sg_eigen_init(sg_handle h, int32_t pop, uint64_t master_state, double k0);
/* One whole eigenvalue cycle on the resident banks: gen loop, cleanPop, stride(pop+1),
 * reportCycleEnd, normSize_Repr, stride(1), dungeon flip and k update
 * (eigenPhysicsPackage_class.f90:203-338).  `admin` is the cycle's tally admin; the
 * k estimate is read from attachment `atch`. */
int32_t sg_eigen_cycle(sg_handle h, int32_t admin, int32_t atch, sg_cycle_stats* stats);
/* The same whole cycle for a caller that keeps its dungeons in host memory: the body of
 * eigenPhysicsPackage%cycles (eigenPhysicsPackage_class.f90:203-338) with thisCycle in `in` (pop
 * particles), the package's pRNG in *master_state, thisCycle%k_eff in *k_eff and nextCycle%k_eff in
 * k_end.  The gen loop, cleanPop, stride(pop+1), reportCycleEnd, normSize_Repr to pop, stride(1) and
 * the k estimate of attachment `atch` run on the device; `out` receives the normalised next-cycle
 * bank (pop particles, in brood order), *master_state the strided pRNG and *k_eff the new k.  A bank
 * in page-locked host memory that the device can address (cudaHostAlloc, or cudaHostRegister with
 * mapping) is read by the kernels in place across the host link while they run; other host memory
 * is copied to the device first.  Replaces the resident run of sg_eigen_init. */
int32_t sg_eigen_cycle_bank(sg_handle h, int32_t admin, int32_t atch, const sg_bank* in, int32_t pop,
                            uint64_t* master_state, double* k_eff, double k_end, sg_bank* out,
                            sg_cycle_stats* stats);
/* current master RNG state and k of the resident eigen run */
int32_t sg_eigen_state(sg_handle h, uint64_t* master_state, double* k);
/* copy the resident "this cycle" bank to the host (pop particles) */
int32_t sg_eigen_get_bank(sg_handle h, sg_bank* out, int32_t cap, int32_t* pop);

/* fixedSourcePhysicsPackage%cycles, one batch, fully on the device: point source generation,
 * stride(n), gen loop, stride(n), reportCycleEnd.  master_state is updated in place. */
int32_t sg_fixed_source_cycle(sg_handle h, int32_t admin, int32_t n, uint64_t* master_state,
                              sg_cycle_stats* stats);
/* The same cycle for one process of a population split over processes (SCONE with MPI,
 * fixedSourcePhysicsPackage_class.f90:131,186-189,264 with getWorkshare/getOffset,
 * mpi_func.f90:133-159): `share` histories of `total`; master_state enters strided by this
 * process's offset and is strided by `total` after the source and after the gen loop, so the
 * union of all processes' histories is the single-process run's. */
int32_t sg_fixed_source_cycle_shard(sg_handle h, int32_t admin, int32_t share, int32_t total,
                                    uint64_t* master_state, sg_cycle_stats* stats);

/* One process's part of particleDungeon%normSize_Repr when the population is split over processes
 * (particleDungeon_class.f90:431-605, MPI branches).  `sites` holds this process's n fission sites
 * sorted by brood ID (as sg_transport_bank returns them); sites_before is the number of sites of the
 * processes before this one and tot_sites the number over all processes (the gathered popSizes);
 * master_state is the master process's RNG state at the call (:469-494: its draws number the sites
 * of all processes in process order).  Every process finds the same threshold (the heap threshold
 * over all tot_sites draws, computed on the device from master_state alone: there is nothing to
 * broadcast) and keeps, or duplicates, its own sites with the draws that fall to them (:500-586).
 * The result, sorted by brood ID, goes to `out` (capacity out_cap), its size to n_out.  The sizes
 * summed over processes equal tot_pop; loadBalancing (:593-700) is the caller's exchange. */
int32_t sg_normalise_shard(sg_handle h, const sg_bank* sites, int32_t n, int64_t sites_before,
                           int64_t tot_sites, int32_t tot_pop, uint64_t master_state,
                           sg_bank* out, int32_t out_cap, int32_t* n_out);

/* The running-batch scores of one admin (n_bins values, the sum over threads of scoreMemory's
 * parallelBins, scoreMemory_class.f90:215-233): read, and written back after a sum over processes.
 * That sum is the MPI reduction of a tally with mpiSync (scoreMemory%reduceBins, :403-432), which
 * the k attachment of an eigenvalue calculation uses (eigenPhysicsPackage_class.f90:607-630); call
 * both between sg_transport_bank and sg_tally_cycle_end of the batch's last cycle. */
int32_t sg_tally_get_scores(sg_handle h, int32_t admin, double* scores, int64_t n_bins);
int32_t sg_tally_set_scores(sg_handle h, int32_t admin, const double* scores, int64_t n_bins);

/* ---------------------------------------------------------------- gen loop without allocation */

/* No counterpart in SCONE.  The gen loop of sg_transport_bank for callers that cannot allocate
 * device memory when a cycle runs: programs whose device memory belongs to another allocator or
 * to a pool reserved up front (cudaMalloc would go around it or fail once the pool holds the GPU),
 * and real-time sections that must stay out of the driver's allocator, whose calls can block.  The banks are the
 * caller's device arrays (dev_in: r, dir, wgt, G, time; dev_next: every array, capacity next_cap);
 * the handle must already hold the geometry, multigroup data and tallies.  Multigroup handles only:
 * a continuous-energy handle is refused with SG_ERR_STATE.  It always runs the history-loop kernel,
 * whatever the handle's form.  It calls no cudaMalloc/cudaFree: its scratch (site staging,
 * per-history counts, scan sums, counters, k) is one static device array of 3 MiB that every GPU
 * loading the library holds until exit, which limits a call to SG_NOALLOC_MAX_HISTORIES histories
 * (larger n is rejected with SG_ERR_BAD_ARG before anything runs) and SG_NOALLOC_MAX_SITES fission
 * sites in total (a call that makes more fails with SG_ERR_BANK_OVERFLOW; the scores it made before
 * stopping stay in the tallies, as with sg_transport_bank).  The first call on a device looks up
 * that array's device address, so make it before any stream capture.  All calls share the array:
 * calls that overlap on the GPU race.  Returns the number of sites written in *n_next; the sites
 * and the scores are those of sg_transport_bank on the same bank (the fission bank identical, the
 * bins equal up to the order of the floating-point sums). */
#define SG_NOALLOC_MAX_HISTORIES 16384
#define SG_NOALLOC_MAX_SITES     32768
int32_t sg_transport_bank_noalloc(sg_handle h, int32_t admin, const sg_bank* dev_in, int32_t n,
                                  uint64_t master_state, double k_eff, sg_bank* dev_next,
                                  int32_t next_cap, int32_t* n_next);

/* ---------------------------------------------------------------- collision processor variants */

/* collisionProcessor choice (CollisionOperator/CollisionProcessors): neutronMGstd / neutronCEstd
 * (SG_COLL_STD, the default) or neutronMGimp / neutronCEimp (SG_COLL_IMP) with their options.
 * neutronMGimp acts through weight windows only (neutronMGimp_class.f90:319-351); neutronCEimp also
 * through implicit absorption, roulette and splitting (neutronCEimp_class.f90:160-232,406-424,
 * 633-734).  Split particles wait in a per-history buffer and are transported after the particle
 * that made them, last in first out, on the same RNG stream (the fixed-source and eigenvalue gen
 * loops' `buffer`); splitting and weight windows need the history-loop form. */
#define SG_COLL_STD 0
#define SG_COLL_IMP 1
typedef struct sg_collision_desc {
  int32_t kind;                 /* SG_COLL_*                                              */
  int32_t imp_abs;              /* `impAbs`: implicit absorption (needs roulette or windows) */
  int32_t roulette;             /* `roulette`                                             */
  int32_t split;                /* `split` (needs max_wgt >= 2 min_wgt)                   */
  int32_t weight_windows;       /* `weightWindows`: use the weightWindowsField below      */
  int32_t max_split;            /* `maxSplit` (SCONE default 1000)                        */
  double  min_wgt, max_wgt, av_wgt;   /* `minWgt` 0.25, `maxWgt` 1.25, `avWgt` 0.5        */
  int32_t ww_n_axes;            /* weightWindowsField (weightWindowsField_class.f90:75-111): */
  sg_axis_desc ww_axes[3];      /*   its `map` (multiMap order)                           */
  const double* ww_lower;       /*   `wLower`, one per map bin                            */
  const double* ww_upper;       /*   `wUpper`, one per map bin                            */
  double  ww_const_survival;    /*   `constSurvival` (> 1)                                */
  int32_t buffer_depth;         /* split particles one history may hold at once (0: 32)  */
} sg_collision_desc;
int32_t sg_set_collision(sg_handle h, const sg_collision_desc* d);

/* ---------------------------------------------------------------- event-form queue thresholds */

/* No SCONE counterpart (SCONE has no event form).  The event form (SG_FORM_EVENT) alternates
 * transit and collision kernels over compacted queues; the host checks the queue length every
 * `rounds_per_check` rounds and hands the rest to the history-loop tail kernel once it is at most
 * max(tail_min, n / tail_divisor).  Defaults 4, 4096, 64; sg_batch_autotune_plain picks them. */
typedef struct sg_event_tuning {
  int32_t rounds_per_check;
  int32_t tail_min;
  int32_t tail_divisor;
} sg_event_tuning;
int32_t sg_set_event_tuning(sg_handle h, const sg_event_tuning* t);
int32_t sg_get_event_tuning(sg_handle h, sg_event_tuning* t);

/* ---------------------------------------------------------------- batched solves */

/* No single SCONE counterpart: SCONE solves one problem per process
 * (fixedSourcePhysicsPackage%cycles, fixedSourcePhysicsPackage_class.f90:183-289).  A batch keeps
 * many independent fixed-source MG problems resident in one device arena (its HBM budget) and
 * transports every cycle of the problems it is given in ONE persistent launch fed from a device
 * work queue.  Each problem gives the results that sg_fixed_source_cycle, called `cycles` times on
 * a handle holding that problem alone, gives: the same RNG stream per history (bit-identical in
 * SG_PREC_FP64), the same per-cycle scoreMemory closes. */
typedef struct sg_batch_t* sg_batch;

typedef struct sg_batch_config {
  int32_t precision;            /* SG_PREC_*                               */
  int32_t transport;            /* SG_TRANSPORT_*                          */
  int32_t device;
  int32_t max_problems;         /* resident problem slots                  */
  int64_t arena_bytes;          /* device memory for problem data and score memory (admission budget) */
  int32_t max_work_items;       /* capacity of the device work queue       */
  int32_t reserved;
  double  ht_cutoff;            /* as sg_config.ht_cutoff                  */
} sg_batch_config;

/* one fixed-source problem: geometry, MG data, point source, one tally admin (batch_size 1: every
 * cycle closes a batch; k clerks are rejected), `cycles` cycles of `pop` histories from master_state */
typedef struct sg_problem_desc {
  const sg_geometry_desc*     geometry;
  const sg_mg_desc*           mg;
  const sg_point_source_desc* source;
  const sg_tally_desc*        tally;
  int32_t                     pop;
  int32_t                     cycles;
  uint64_t                    master_state;
} sg_problem_desc;

/* launch shape of the batched kernel, picked by sg_batch_autotune or set by hand */
typedef struct sg_batch_tuning {
  int32_t item_histories;       /* histories per work item                                      */
  int32_t blocks_per_sm;        /* persistent grid = SMs x blocks_per_sm (capped by occupancy)  */
  int32_t block_threads;        /* 32, 64, 96 or 128                                            */
  int32_t order;                /* 0: submission order; 1: largest problem first; 2: problems of
                                   one kind (nesting depth, group count) together, largest first */
} sg_batch_tuning;

typedef struct sg_batch_stats {
  int64_t n_histories;
  int64_t n_events;             /* flight segments (device-counted) */
  int64_t n_collisions;
  int32_t n_problems;
  int32_t n_items;              /* work items (batched) or 0 (plain) */
  double  kernel_ms;            /* transport time, CUDA events: the run graph (batched) or the sum of
                                   the transport kernels (plain) */
  double  run_ms;               /* the whole call, CUDA events on the batch stream */
  int64_t n_kernels;            /* kernels launched by the call */
} sg_batch_stats;

int32_t sg_batch_create(const sg_batch_config* cfg, sg_batch* out);
int32_t sg_batch_destroy(sg_batch b);
int32_t sg_batch_last_error(sg_batch b, char* buf, size_t len);
/* uploads a problem into a free slot; SG_ERR_OOM when the arena or the slots are full */
int32_t sg_batch_add(sg_batch b, const sg_problem_desc* p, int32_t* slot);
/* a new request on the data of resident problem `parent` (geometry, MG data, source and clerks shared,
 * nothing re-uploaded): its own pop, cycles, RNG seed and score memory, taken from the arena
 * (SG_ERR_OOM when full).  Does not wait for the device. */
int32_t sg_batch_instance(sg_batch b, int32_t parent, int32_t pop, int32_t cycles, uint64_t master_state,
                          int32_t* slot);
/* frees a slot and its arena memory (a parent only after its instances) */
int32_t sg_batch_remove(sg_batch b, int32_t slot);
/* arena bytes in use and capacity */
int32_t sg_batch_memory(sg_batch b, int64_t* used, int64_t* capacity);
int32_t sg_batch_set_tuning(sg_batch b, const sg_batch_tuning* t);
int32_t sg_batch_get_tuning(sg_batch b, sg_batch_tuning* t);
/* every cycle of the listed problems in one persistent launch, then the cycle closes (one CUDA
 * graph launch); slots must be distinct */
int32_t sg_batch_run(sg_batch b, const int32_t* slots, int32_t n, sg_batch_stats* stats);
/* the plain form: the listed problems one after another, each through sg_fixed_source_cycle's path
 * (one problem per launch sequence), `form` SG_FORM_EVENT or SG_FORM_HISTORY */
int32_t sg_batch_run_plain(sg_batch b, const int32_t* slots, int32_t n, int32_t form, sg_batch_stats* stats);
/* measures candidate launch shapes on the listed problems (their tallies are cleared afterwards),
 * keeps the fastest and returns it */
int32_t sg_batch_autotune(sg_batch b, const int32_t* slots, int32_t n, sg_batch_tuning* best);
/* the same for the plain event form: queue thresholds timed (wall clock) on the listed problems;
 * the best are kept for sg_batch_run_plain */
int32_t sg_batch_autotune_plain(sg_batch b, const int32_t* slots, int32_t n, sg_event_tuning* best);
/* scoreMemory bins(N,3) of a problem, as sg_get_bins; while serving, only for completed requests
 * (read beside the running waves) */
int32_t sg_batch_tally_size(sg_batch b, int32_t slot, int64_t* n_bins);
int32_t sg_batch_get_bins(sg_batch b, int32_t slot, double* bins, int64_t n_bins);
int32_t sg_batch_clear_tally(sg_batch b, int32_t slot);

/* ---------------------------------------------------------------- served solves (continuous batching) */

/* Requests are resident problems.  sg_serve_submit queues every cycle of a problem (its tally is
 * cleared); sg_serve_pump keeps up to two waves in flight on the device, each wave one launch of the
 * batched kernel over work drawn from ALL active requests (each gets an equal share of the wave's
 * `wave_histories`, so a request that arrives while others run joins the next wave), and retires
 * requests whose last history ran: their cycles are closed in that wave.  Latency is submit time to
 * the device completion of the request's last wave (CUDA event time mapped onto the host clock). */
/* wave_histories: histories per wave; item_histories: work-item size while serving (0: the tuning's) */
int32_t sg_serve_start(sg_batch b, int64_t wave_histories, int32_t item_histories);
int32_t sg_serve_submit(sg_batch b, int32_t slot);
/* launches/retires waves; wait != 0 blocks until at least one in-flight wave completes.
 * Completed requests since the last call are written to done_slots / latency_s (up to cap). */
int32_t sg_serve_pump(sg_batch b, int32_t wait, int32_t* done_slots, double* latency_s, int32_t cap,
                      int32_t* n_done);
/* waits for the waves in flight and leaves serving mode (completed requests not yet pumped are dropped) */
int32_t sg_serve_stop(sg_batch b);
/* histories queued but not yet launched, requests active, waves launched so far */
int32_t sg_serve_status(sg_batch b, int64_t* queued, int32_t* active, int64_t* waves);
/* while `on`, waves run with `blocks_per_sm` fewer resident blocks per SM than their tuning, so
 * kernels of other streams (eigenvalue requests on their own handles) find room on every SM */
int32_t sg_serve_share(sg_batch b, int32_t blocks_per_sm, int32_t on);
/* histories and flight events of the waves retired since sg_serve_start */
int32_t sg_serve_counts(sg_batch b, int64_t* histories, int64_t* events);
/* host clock (seconds, the one submit and latency use) */
double sg_serve_clock(void);

/* ---------------------------------------------------------------- verification records */

/* Per-history records of the last gen loop (needs cfg.record_histories): number of real
 * collisions (particle%collisionN increments) and the RNG state at history end. */
int32_t sg_get_history_records(sg_handle h, int32_t* collisions, uint64_t* rng_end, int32_t n);

/* ---------------------------------------------------------------- RNG (RNG_class.f90) */

/* n draws of `get` starting from *state (state advanced); writes xi in [0,1) */
int32_t sg_rng_draws(uint64_t* state, double* out, int32_t n);
/* skip(k) (RNG_class.f90:251-304), k may be negative */
uint64_t sg_rng_skip(uint64_t state, int64_t k);

#ifdef __cplusplus
}
#endif
#endif /* SCONE_GPU_H */
