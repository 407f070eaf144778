/*
 * nlmgpu.h -- C ABI of the GB300 peridynamics library (libnlmgpu.so).
 *
 * The library replaces the explicit-dynamics hot path of NLMech
 * (nonlocalmodels/NLMech): the horizon neighbour search, the RNPBond and
 * ElasticState bond-force loops, bond breaking / damage, and the
 * velocity-Verlet and central-difference integrators of FDModel.
 *
 * Conventions
 *  - Every array argument is a caller-owned HOST buffer.  Node vectors use the
 *    reference's util::Point3 layout: 3 doubles (x, y, z) per node, so a
 *    std::vector<util::Point3> can be passed as (const double*)&v[0].
 *  - Node and bond indices at the boundary are the caller's ("original")
 *    node ids.  Neighbour rows are returned in ascending id order, which is
 *    the order geometry::Neighbor builds them (src/geometry/neighbor.cpp:78).
 *  - Bond state is returned as one byte per CSR entry (0 = intact,
 *    1 = broken) in that same row order, i.e. the bit that
 *    geometry::Fracture::getBondState(i, j_local) returns
 *    (src/geometry/fracture.cpp:174-187).
 *  - Every call returns an int status (NLM_OK = 0).  Nothing calls exit();
 *    nlm_last_error() gives a message for the calling thread.
 *  - A handle owns one CUDA stream and its device memory.  A handle is not
 *    thread-safe; distinct handles are independent.
 */
#ifndef NLMGPU_H
#define NLMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NLM_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------- */
enum {
  NLM_OK = 0,
  NLM_ERR_INVALID = 1,     /* bad argument / inconsistent description   */
  NLM_ERR_CUDA = 2,        /* CUDA runtime error                        */
  NLM_ERR_OOM = 3,         /* device allocation failed                  */
  NLM_ERR_TIMEOUT = 4,     /* a bounded device wait gave up             */
  NLM_ERR_UNSUPPORTED = 5, /* option not implemented on this path       */
  NLM_ERR_STATE = 6,       /* call out of order for the handle          */
  NLM_ERR_NONFINITE = 7    /* NaN / Inf found in an input array         */
};

/* ---- enums mirroring the reference's deck strings ---------------------- */
enum nlm_material_kind {
  NLM_MAT_RNP_BOND = 0,      /* material::pd::RNPBond (rnpBond.cpp)        */
  NLM_MAT_ELASTIC_STATE = 1  /* material::pd::ElasticState (ElasticState.cpp) */
};

enum nlm_precision {
  NLM_PREC_FP64 = 0,  /* "plain": every bond in FP64, reference op order   */
  NLM_PREC_FP32C = 1  /* "compensated": FP32 bond math on split hi/lo
                         positions and displacements, FP64 state/update   */
};

enum nlm_scheme {
  NLM_VELOCITY_VERLET = 0,     /* "velocity_verlet"   fDModel.cpp:445-525 */
  NLM_CENTRAL_DIFFERENCE = 1   /* "central_difference" fDModel.cpp:376-443 */
};

enum nlm_decomposition {
  NLM_DECOMP_AUTO = 0,    /* pick by timing the candidates on the model    */
  NLM_DECOMP_THREAD = 1,  /* one thread per node, sliced-ELL bonds taken
                             four at a time                                */
  NLM_DECOMP_WARP = 2,    /* one warp per node, CSR bond storage           */
  NLM_DECOMP_THREAD1 = 3, /* one thread per node, one bond per iteration   */
  NLM_DECOMP_TILE = 4,    /* FP32C 2-D RNPBond: 256-node tiles with their
                             halo staged in shared memory, 16-bit
                             tile-local bond ids                           */
  NLM_DECOMP_TILE_LOCAL = 5 /* as TILE with the staged positions and
                             displacements in the tile's frame, one FP32
                             value per component: FP32C 2-D RNPBond (also
                             batched) and FP32C 2-D / 3-D ElasticState     */
};

/* Displacement_BC / Force_BC region types (loading/uLoading.cpp:38-46). */
enum nlm_region {
  NLM_REGION_RECTANGLE = 0, /* x in [x1,x2], y in [y1,y2] (utilGeom.cpp:43) */
  NLM_REGION_LINE = 1,      /* x1 < x < x2 (1-D)                          */
  NLM_REGION_CIRCLE = 2,    /* |x - (x1,y1)| < r1                          */
  NLM_REGION_TORUS = 3,     /* r2 <= |x - (x1,y1)| < r1                    */
  NLM_REGION_CUBOID = 4,    /* box [x1,x2]x[y1,y2]x[z1,z2] (Force_BC; a
                               Displacement_BC cuboid is an extension)     */
  NLM_REGION_ANGLED_RECTANGLE = 5 /* rectangle from (x1,y1) to (x2,y2) in axes
                               turned by theta (utilGeom.cpp:60-95)        */
};

enum nlm_time_fn { /* uLoading.cpp:210-236 */
  NLM_TFN_CONSTANT = 0,
  NLM_TFN_LINEAR = 1,
  NLM_TFN_QUADRATIC = 2,
  NLM_TFN_SIN = 3,
  NLM_TFN_LINEAR_STEP = 4,
  NLM_TFN_LINEAR_SLOW_FAST = 5
};

enum nlm_spatial_fn { /* uLoading.cpp:186-208, fLoading.cpp:124-238 */
  NLM_SFN_CONSTANT = 0,
  NLM_SFN_SIN_X = 1,
  NLM_SFN_SIN_Y = 2,
  NLM_SFN_SIN_Z = 3,
  NLM_SFN_LINEAR_X = 4,
  NLM_SFN_LINEAR_Y = 5,
  NLM_SFN_LINEAR_Z = 6,
  /* Force_BC only (refused in a Displacement_BC, as ULoading refuses them): */
  NLM_SFN_HAT_X = 7,      /* p0 * hat(x; x1, x2), util::function::hatFunction */
  NLM_SFN_HAT_Y = 8,      /* p0 * hat(y; y1, y2)                            */
  NLM_SFN_HAT_Z = 9,      /* p0 * hat(z; z1, z2)                            */
  NLM_SFN_LINE_LOAD = 10  /* per direction d: floor((x_d - min)/h) / floor(|max - min|/h),
                             from max when p0 == -1 (fLoading.cpp:171-232) */
};

enum nlm_crack_kind {
  NLM_CRACK_EDGE = 0,  /* inp::EdgeCrack, 2-D (fractureDeck.h:115-186)      */
  NLM_CRACK_PLANE = 1  /* planar patch z = z0 over [x0,x1]x[y0,y1] (3-D)    */
};

enum nlm_no_fail {
  NLM_NOFAIL_OFF = 0,     /* BaseInterior: every node interior            */
  NLM_NOFAIL_COMPUTE = 1, /* ComputeInterior: bbox minus tolerance        */
  NLM_NOFAIL_DATA = 2     /* DataInterior: the same flags, stored         */
};

/* ---- descriptions --------------------------------------------------- */

/* One Displacement_BC or Force_BC set (inp::BCData). */
typedef struct nlm_bc_set {
  int region;            /* enum nlm_region                              */
  double x1, x2, y1, y2; /* region box / centre                          */
  double z1, z2;         /* NLM_REGION_CUBOID only                       */
  double r1, r2;         /* circle / torus radii                         */
  int dir_mask;          /* bit d set = dof d (0:x 1:y 2:z), "Direction"  */
  int time_fn;           /* enum nlm_time_fn                             */
  double time_params[4];
  int spatial_fn;        /* enum nlm_spatial_fn                          */
  double spatial_params[2];
  double theta;          /* NLM_REGION_ANGLED_RECTANGLE: Location.Angle   */
} nlm_bc_set;

/* One crack (inp::EdgeCrack, or a 3-D plane).  timed = 0: a pre-crack, cut
 * at creation (an EdgeCrack with activation time < 0, fracture.cpp:20-43).
 * timed = 1: cut by the explicit model after the first step whose end time t
 * has activation_time definitely less than t (Fracture::addCrack,
 * fracture.cpp:45-70, called after every step at fDModel.cpp:366-373); at
 * most one timed crack is cut per step, in array order.  At most 32 timed
 * cracks per model; the batched and quasi-static models take pre-cracks
 * only. */
typedef struct nlm_crack {
  int kind;            /* enum nlm_crack_kind                              */
  int orientation;     /* EdgeCrack d_o: 1 = along x, -1 = along y, 0 = angle */
  double pb[2], pt[2]; /* EdgeCrack "Line": bottom/left and top/right ends */
  double theta;        /* EdgeCrack angle for orientation 0               */
  double z0;           /* plane kind: plane height                        */
  double lo[2], hi[2]; /* plane kind: patch [lo0,hi0] x [lo1,hi1]          */
  int timed;           /* 0: pre-crack; 1: cut at activation_time          */
  double activation_time; /* EdgeCrack "Activation_Time" (timed = 1)     */
} nlm_crack;

/* One No_Fail_Region "Region_k" (interiorFlagsDeck.h:38, interiorFlags.cpp:
 * 76-90): a node inside it is not interior, so its bonds never break.
 * Circle: params = centre x, y, z and radius r, inside when
 * |x - c| < r (definitelyLessThan).  Rectangle: params = x1, y1, x2, y2,
 * inside by util::geometry::isPointInsideRectangle.  Used when no_fail is on. */
enum nlm_nofail_region_kind { NLM_NOFAIL_CIRCLE = 0, NLM_NOFAIL_RECTANGLE = 1 };
typedef struct nlm_nofail_region {
  int kind;          /* enum nlm_nofail_region_kind */
  double params[4];
} nlm_nofail_region;

/* inp::MaterialDeck fields used on the hot path (materialDeck.h). */
typedef struct nlm_material {
  int kind;                 /* enum nlm_material_kind                      */
  double density;
  double E, G, K, Gc, KIc;  /* < 0 means "not given" (deck default -1)     */
  int plane_strain;         /* Is_Plane_Strain                             */
  int influence_type;       /* 0 const, 1 linear, 2 Gaussian (influenceFn.h) */
  int n_influence_params;
  double influence_params[2];
  int irreversible;         /* Irreversible_Bond_Fracture (default 1)      */
  double check_sc_factor;   /* Check_Sc_Factor (default 1)                 */
  int compute_from_classical; /* Compute_From_Classical (default 1)        */
  double bond_params[2];    /* C, beta when not computed from classical    */
  double es_sc;             /* ElasticState critical stretch; <= 0: no breaking */
  int es_ref_compat;        /* 1: keep the reference's 3-D e_d = 0          */
  int apply_contact;        /* No_Penetration: normal contact force between
                               the nodes of a broken bond (rnpBond.cpp:79-88,
                               :281-291); explicit single-model runs only    */
} nlm_material;

typedef struct nlm_fd_desc {
  int dim;                  /* 1, 2 or 3                                   */
  int64_t n_nodes;
  const double *x;          /* 3*n reference coordinates (Point3 layout)   */
  const double *volume;     /* n nodal volumes                             */
  double horizon;           /* Model.Horizon                               */
  double mesh_size;         /* h (Model.Mesh_Size or Horizon/Horizon_h_Ratio) */
  nlm_material material;
  int n_ubc;                /* Displacement_BC sets                        */
  const nlm_bc_set *ubc;
  int n_fbc;                /* Force_BC sets                               */
  const nlm_bc_set *fbc;
  int n_cracks;
  const nlm_crack *cracks;
  int no_fail;              /* enum nlm_no_fail                            */
  double no_fail_tol;       /* horizon * No_Fail_Region.Factor             */
  double dt;                /* Final_Time / Time_Steps                     */
  int scheme;               /* enum nlm_scheme                             */
  int precision;            /* enum nlm_precision                          */
  int decomposition;        /* enum nlm_decomposition                      */
  const double *u0;         /* optional 3*n initial displacement (or NULL) */
  const double *v0;         /* optional 3*n initial velocity (or NULL)     */
  int n_nofail_regions;     /* No_Fail_Region.Num_Regions                  */
  const nlm_nofail_region *nofail_regions;
} nlm_fd_desc;

/* ---- library ---------------------------------------------------------- */

/* Message of the last failed call on this thread ("" if none). */
const char *nlm_last_error(void);
int nlm_abi_version(void);
/* Number of CUDA devices visible (0 on a host without a GPU). */
int nlm_device_count(int *count);
/* Select the device used by handles created afterwards on this thread. */
int nlm_set_device(int device);

/* ---- neighbour search (replaces geometry::Neighbor, neighbor.cpp:24-92) --
 * Builds rows {j != i : definitelyLessThan(|x_i - x_j|, horizon + 1e-10)}
 * with a uniform cell list on the GPU.  Two calls: first with cols == NULL
 * to get rowptr (n+1 entries, rowptr[n] = nnz), then with cols of nnz. */
int nlm_neighbor_search(int dim, int64_t n, const double *x, double horizon,
                        int64_t *rowptr, int32_t *cols);

/* Same result as nlm_neighbor_search, with no device allocation.  No
 * counterpart in the reference (it allocates through its std::vector
 * neighbour lists); this entry serves callers that must not allocate device
 * memory: a host whose free HBM is already held by a pool allocator, or a run
 * that rebuilds neighbours while other streams work and cannot take the
 * device-wide synchronisation that cudaFree implies.  All intermediates live
 * in one file-scope __device__ array of 22,545,152 bytes; inputs above
 * n = 65,536 nodes, 262,144 grid cells, 4,194,304 bonds or 512 entries in a
 * row are rejected with NLM_ERR_INVALID.  The per-cell counters, scatter
 * cursors and error word of the scratch must start at zero; each call clears
 * them itself before its first kernel.  Calls that overlap in time on the
 * same device (two host threads) race on that one array: serialise them.
 * Every call looks up the array's address in the current context
 * (cudaGetSymbolAddress, with the device current), so a device reset or a
 * non-primary context between calls is safe; the first call on a device
 * also loads the module, so make it before any stream capture on that
 * device.  Works on the calling thread's current device and per-thread
 * default stream, and returns after the results are on the host. */
int nlm_neighbor_search_noalloc(int dim, int64_t n, const double *x, double horizon,
                                int64_t *rowptr, int32_t *cols);

/* ---- explicit finite-difference model (replaces model::FDModel<T>) ----- */
typedef struct nlm_fd nlm_fd;

/* Uploads the mesh, builds neighbours, applies pre-cracks and BC tables
 * (FDModel::initHObjects + init, fDModel.cpp:133-315). */
int nlm_fd_create(const nlm_fd_desc *desc, nlm_fd **out);
int nlm_fd_destroy(nlm_fd *h);

/* Number of directed bonds (sum of neighbour row lengths). */
int nlm_fd_num_bonds(const nlm_fd *h, int64_t *nnz);
/* Neighbour lists in original ids, rows ascending (rowptr n+1, cols nnz). */
int nlm_fd_get_neighbors(nlm_fd *h, int64_t *rowptr, int32_t *cols);

/* Advance nsteps time steps (FDModel::integrate, fDModel.cpp:317-374).  The
 * first call also performs the step-0 work: initial loads and forces. */
int nlm_fd_run(nlm_fd *h, int64_t nsteps);

/* Copy state out: u, v, f are 3*n (any may be NULL).  f is the force
 * density of the last force evaluation (external + internal). */
int nlm_fd_get_state(nlm_fd *h, double *u, double *v, double *f);
/* Overwrite u and v (3*n each, either may be NULL). */
int nlm_fd_set_state(nlm_fd *h, const double *u, const double *v);
/* Time and step counter (d_time, d_n). */
int nlm_fd_get_time(const nlm_fd *h, double *time, int64_t *step);
/* Bond state, one byte per CSR entry in nlm_fd_get_neighbors order. */
int nlm_fd_get_bond_state(nlm_fd *h, uint8_t *broken);
/* Damage fields of FDModel::computePostProcFields (fDModel.cpp:651-778):
 * phi_i = 1 - sum_unbroken V_j^c / sum V_j^c and Z_i = max_j |S|/S_c.
 * Either pointer may be NULL. */
int nlm_fd_damage(nlm_fd *h, float *phi, float *Z);
/* Number of broken bonds (directed). */
int nlm_fd_count_broken(nlm_fd *h, int64_t *count);
/* Fixity bits per node in the caller's order (bit d: dof d is prescribed by
 * a Displacement_BC; fe::Mesh::getFixity as ULoading sets it,
 * uLoading.cpp:99-102). */
int nlm_fd_get_fixity(nlm_fd *h, uint8_t *fixity);
/* Energies of computePostProcFields (fDModel.cpp:651-778), RNPBond, per node
 * in the caller's order (any may be NULL): strain energy (Strain_Energy),
 * work done u . f_ext (Work_Done), kinetic energy, and the strain energy of
 * nodes with Z > 1 (Fracture_Perienergy_Total); totals[4] their sums, in
 * FP64 (the reference sums the float arrays in float). */
int nlm_fd_energies(nlm_fd *h, float *strain, float *work, float *kinetic, float *fracture,
                    double *totals);
/* Reaction force of FDModel::computeForce (fDModel.cpp:543-580), 2-D RNPBond:
 * "Reaction_Force" R_i (reaction[3n], caller's order), "Total_Reaction_Force"
 * |R_i| (total[n]) and the sum of R_i over the nodes (sum[3]); any may be
 * NULL.  R_i sums V_i F_ij over the bonds that is_reaction_force (:582-605)
 * selects: node i in max_y - 1.5 delta < y < max_y - delta and the bond
 * meeting the line y = max_y - delta + 1e-6, with util::geometry's
 * doLinesIntersect as written (its orientation test truncates the cross
 * product to an int).  The bounding box is fe::Mesh::computeBBox's. */
int nlm_fd_reaction_force(nlm_fd *h, double *reaction, double *total, double *sum);
/* Start the run at this step and time (FDModel::restart sets
 * d_n = Restart.Step and d_time = d_n dt, fDModel.cpp:102-131); only before
 * the first step (NLM_ERR_STATE afterwards).  With nlm_fd_set_state this is
 * the reference's restart from a VTU file (which restores u and v only). */
int nlm_fd_set_time(nlm_fd *h, double time, int64_t step);
/* Overwrite the bond state (inverse of nlm_fd_get_bond_state). */
int nlm_fd_set_bond_state(nlm_fd *h, const uint8_t *broken);

/* ---- checkpoint / restart ----------------------------------------------
 * The reference's restart (fDModel.cpp:102-131, reader.cpp:149-173) reloads
 * u and v from a VTU file but not the bond state, so a restarted fracture
 * run heals its cracks.  A checkpoint here holds u, v, f, the bond state
 * (one byte per bond), the step counter and time in one binary file:
 *   "NLMCKPT" magic, int32 version, dim, precision, material, started,
 *   int64 n, nnz, step, double time, dt, then u, v, f (3n doubles each,
 *   caller's node order) and the bond bytes (nlm_fd_get_bond_state order).
 * Loading into a handle created from the same description continues the
 * run as if it had not stopped (bit for bit in FP64 plain). */
int nlm_fd_save(nlm_fd *h, const char *path);
int nlm_fd_load(nlm_fd *h, const char *path);
/* Work decomposition actually used (enum nlm_decomposition). */
int nlm_fd_decomposition(const nlm_fd *h, int *decomp);
/* Average device time of the bond-force kernel over the launches since the
 * last reset (milliseconds), measured with CUDA events on the handle's
 * stream; and the algorithmic bytes one launch moves. */
int nlm_fd_kernel_stats(nlm_fd *h, int reset, double *avg_ms,
                        int64_t *launches, double *bytes_per_launch);
/* Enable/disable per-launch event timing of the force kernel. */
int nlm_fd_set_timing(nlm_fd *h, int enable);
/* Synchronize the handle's stream. */
int nlm_fd_sync(nlm_fd *h);

/* Drop-in step for a host-resident state (the reference's DataManager keeps
 * u, v, f on the host, fDModel.cpp:200-206): copies u, v and f (3*n each) in,
 * advances nsteps from them, copies u, v and f out.  The first call on a
 * fresh handle performs the step-0 force evaluation (f is then output only).
 * Passing back unchanged the arrays of the previous call continues the run
 * exactly as nlm_fd_run would. */
int nlm_fd_step_host(nlm_fd *h, double *u, double *v, double *f,
                     int64_t nsteps);
/* How the last nlm_fd_step_host moved the arrays: 1 = read and written in
 * place by kernels (each of u, v, f lies inside one page-locked allocation
 * the device maps at the same address, e.g. from cudaHostAlloc or
 * cudaHostRegister), 0 = copied through device staging buffers, 2 = page-
 * locked arrays moved in caller-order bands whose copies in and out overlap
 * the step (one FP32C velocity-Verlet step of a 2-D model of at least 65536
 * nodes on a tile decomposition; same results as the other two).  On a
 * non-finite input every mode fails with the model unchanged; modes 1 and 2
 * also leave the caller's arrays as they were.  In 2-D the z entries of u
 * and v are left as the caller had them either way (the reference's 2-D
 * integrator never writes them) and f's z is written as 0. */
int nlm_fd_host_io(const nlm_fd *h, int *mode);
/* Cap the device memory the handle may allocate from this call on at
 * `bytes` (memory it frees again counts back; bytes < 0 removes the cap).
 * Buffers a path allocates lazily -- the banded host step's staging, the
 * in-place path's staging, post-processing outputs -- then fail with
 * NLM_ERR_OOM past the cap; the banded host step falls back to the in-place
 * path, with the same results.  No reference counterpart (the reference
 * allocates on the host only). */
int nlm_fd_set_alloc_limit(nlm_fd *h, int64_t bytes);
/* nlm_fd_run bracketed by CUDA events on the handle's stream; *ms is the
 * device time of the whole run (the stream is synchronized). */
int nlm_fd_run_timed(nlm_fd *h, int64_t nsteps, double *ms);

/* Replay the step loop from CUDA graphs of steps_per_graph steps (even,
 * >= 2; 0 = plain launches).  The step-0 evaluation and any remainder run as
 * plain launches, and so does a chunk in which a timed crack falls due.  A
 * graph step evaluates the Force_BC loads at its own time, which its launches
 * read from a device array. */
int nlm_fd_set_graph(nlm_fd *h, int steps_per_graph);

/* ---- batched specimens -------------------------------------------------
 * Many independent specimens (same dimension, dt, scheme and material kind;
 * FP32-compensated RNPBond) in one node space: each step is one launch per
 * node-count bucket over all specimens, each bucket with the decomposition
 * the autotuner picked for it (THREAD, THREAD1, WARP or, in 2-D,
 * TILE_LOCAL), or with the one every desc names when all name the same
 * (NLM_DECOMP_TILE is refused); when every bucket takes TILE_LOCAL a step
 * is a single launch.  Per-specimen constants live in a table in device
 * memory.  Specimen ids below are positions in the descs array. */
typedef struct nlm_batch nlm_batch;

int nlm_batch_create(const nlm_fd_desc *descs, int n_specimens, nlm_batch **out);
int nlm_batch_destroy(nlm_batch *b);
int nlm_batch_run(nlm_batch *b, int64_t nsteps);
/* nlm_batch_run bracketed by CUDA events on the batch's stream. */
int nlm_batch_run_timed(nlm_batch *b, int64_t nsteps, double *ms);
/* Bonds of one specimen, or of all specimens when specimen == -1. */
int nlm_batch_num_bonds(const nlm_batch *b, int specimen, int64_t *nnz);
int nlm_batch_get_state(nlm_batch *b, int specimen, double *u, double *v, double *f);
int nlm_batch_get_bond_state(nlm_batch *b, int specimen, uint8_t *broken);
int nlm_batch_get_time(const nlm_batch *b, double *time, int64_t *step);
/* Same meaning as nlm_fd_set_graph. */
int nlm_batch_set_graph(nlm_batch *b, int steps_per_graph);
/* Buckets (at most 8): node count and chosen decomposition of each. */
int nlm_batch_buckets(const nlm_batch *b, int *n_buckets, int64_t *bucket_nodes,
                      int *decomps);

/* ---- quasi-static Newton (replaces QuasiStaticModel<T>::solver) ---------
 * RNPBond plates: load step k sets the Displacement_BC values at time k*dt
 * (QuasiStaticModel.cpp:537-549), then Newton iterations on the free dofs
 * with the analytic sparse tangent and preconditioned CG until
 * ||r|| <= tol * ||r(plain guess)||, where the plain guess is the previous
 * load step's solution with the new boundary values.  Bonds over the
 * critical strain break after convergence and the step is solved again. */
typedef struct nlm_qs_params {
  int max_newton;      /* Newton iterations per solve (Solver.Max_Iteration) */
  double tol;          /* relative residual tolerance (default 1e-8)         */
  int lin_max_iters;   /* CG iterations per Newton step                      */
  double lin_tol;      /* CG relative tolerance (inexact Newton)             */
  int break_bonds;     /* 1: bonds past the critical strain break during
                          every residual evaluation (RNPBond::getBondEF)    */
  int max_break_rounds;  /* unused (kept for layout compatibility)          */
  double guess_accept; /* a guess is used only if its linearised residual is
                          at most guess_accept times that of the plain
                          start (<= 0: 0.1)                                  */
  int krylov_launch;   /* 0: the FP32 Krylov solve runs two launches per
                          iteration (default; 46.6 us per iteration with the
                          Newton work around it on the 200 x 200 plate);
                          1: one cooperative launch per solve with grid
                          barriers between its phases where the device
                          allows it (50.2 us per iteration there)          */
  double wait_limit_s; /* bound of each grid-barrier wait of that launch
                          (<= 0: 1 s); a wait that runs out ends the solve
                          with NLM_ERR_TIMEOUT and the handle stays usable   */
  int barrier_extra;   /* testing the bound only: arrivals each barrier waits
                          for beyond the launched blocks (0 in use; > 0 makes
                          every wait run out)                                */
  double lin_tol_gamma; /* > 0: a Newton iteration whose residual is already
                          near the target solves to the looser relative
                          tolerance min(0.1, gamma * target / ||r||), never
                          tighter than lin_tol (a forcing term after
                          Eisenstat and Walker); 0: lin_tol throughout      */
} nlm_qs_params;

typedef struct nlm_qs_stats {
  int newton_iters;    /* all Newton iterations of the load step             */
  int lin_iters;       /* all CG iterations                                   */
  int break_rounds;    /* re-solves after bond breaking                       */
  int used_guess;      /* 1 if the caller's guess was used (not the fallback) */
  int64_t broken;      /* bonds broken in this step                           */
  double res_plain;    /* ||r|| at the plain previous-step guess              */
  double res_start;    /* ||r|| at the start point actually used             */
  double res_final;
  double ms;           /* wall time of the load step                         */
} nlm_qs_stats;

typedef struct nlm_qs nlm_qs;
int nlm_qs_create(const nlm_fd_desc *desc, const nlm_qs_params *prm, nlm_qs **out);
int nlm_qs_destroy(nlm_qs *q);
/* One load step.  guess: 3*n displacement (original order) to start Newton
 * from, or NULL for the plain previous-step guess; a guess whose residual
 * exceeds the plain guess's is replaced by the plain guess. */
int nlm_qs_load_step(nlm_qs *q, const double *guess, nlm_qs_stats *stats);
/* Same with n_cand candidate starts (n_cand x 3n, Point3 layout): each is
 * judged by the linear model of the residual at the previous converged
 * state and the best is used if its linearised residual is at most
 * guess_accept times that of the plain start; stats->used_guess is then the
 * 1-based index of the chosen candidate (0: plain start). */
int nlm_qs_load_step_candidates(nlm_qs *q, const double *guesses, int n_cand,
                                nlm_qs_stats *stats);
int nlm_qs_get_state(nlm_qs *q, double *u);
int nlm_qs_get_bond_state(nlm_qs *q, uint8_t *broken);
int nlm_qs_damage(nlm_qs *q, float *phi, float *Z);
int nlm_qs_num_bonds(const nlm_qs *q, int64_t *nnz);

/* ---- quasi-static ElasticState (the reference's QuasiStaticModel) -------
 * QuasiStaticModel<ElasticState> (src/model/quasistatic/QuasiStaticModel.cpp,
 * the reference's only quasi-static instantiation, :648): per load step n the
 * force loading is added to the body force at time n dt, the displacement
 * loading is applied, and Newton iterates while ||f + b|| >= tol (free dofs)
 * and fewer than max_iters iterations ran (solver, :526-594).  The Jacobian is
 * assembly_jacobian_matrix_part's (:361-454): central differences of f_i with
 * u_j moved by +-perturbation * mesh size, for j = i and its neighbours,
 * keeping the (i, r; j, r) entries (jacobian = 0, as the reference) or whole
 * blocks (jacobian = 1).  The linear solve is BiCGSTAB to lin_tol relative
 * (the reference asks BlazeIterative for a CG solve, :486-489).  Differences:
 * the first residual of a load step uses the force at the new boundary
 * values, and a node with only some components prescribed keeps rows for its
 * free ones.  dim 1, 2 or 3 (desc->dim); 1-D needs material.E. */
typedef struct nlm_esqs nlm_esqs;
typedef struct nlm_esqs_params {
  int jacobian;        /* 0: (i, r; j, r) entries (reference); 1: full blocks */
  int max_iters;       /* Newton iterations per load step (Solver.Max_Iteration) */
  double tol;          /* Solver.Tolerance on ||f + b||                     */
  int tol_relative;    /* 1: ||r|| / ||r_0|| < tol instead                   */
  double perturbation; /* Solver.Perturbation                               */
  int lin_max_iters;   /* BiCGSTAB iteration cap                            */
  double lin_tol;      /* BiCGSTAB relative residual                        */
  double dt;           /* load-step time increment (Final_Time / Time_Steps) */
} nlm_esqs_params;
int nlm_esqs_create(const nlm_fd_desc *desc, const nlm_esqs_params *params, nlm_esqs **out);
int nlm_esqs_destroy(nlm_esqs *q);
/* nsteps load steps; newton_iters[k], lin_iters[k] per step (may be NULL);
 * final_res = ||f + b|| after the last one. */
int nlm_esqs_solve(nlm_esqs *q, int nsteps, int *newton_iters, int *lin_iters,
                   double *final_res);
/* u (3 per node) and the output's "Force" f_i V_i (3 per node), caller's
 * order; either may be NULL. */
int nlm_esqs_get_state(nlm_esqs *q, double *u, double *force);

/* ---- learned warm start of the quasi-static solver --------------------
 * No counterpart in the reference (its QuasiStaticModel starts every load
 * step from the previous displacement).  A per-node MLP
 *   n_in -> n_hidden (ReLU) x n_layers -> n_out (linear)
 * predicts the start displacement that nlm_qs_load_step receives as its
 * guess.  Parameters are FP32 (Adam master copy); every GEMM rounds its
 * operands to BF16 and accumulates in FP32 on the tensor cores.
 *
 * Parameter layout (nlm_mlp_get_params / set_params), for layer l = 0..n_layers
 * with padded widths d_0 = roundup(n_in, 16), d_1..d_n_layers =
 * roundup(n_hidden, 16), d_{n_layers+1} = roundup(n_out, 8):
 *   W_l[d_l][d_{l+1}] row-major (input index major), then b_l[d_{l+1}].
 * Padding rows and columns are zero and stay zero under training.
 * x: rows x n_in, y and targets t: rows x n_out, float, host memory. */
typedef struct nlm_mlp nlm_mlp;
int nlm_mlp_create(int n_in, int n_hidden, int n_layers, int n_out, uint64_t seed,
                   nlm_mlp **out);
int nlm_mlp_destroy(nlm_mlp *h);
int nlm_mlp_num_params(const nlm_mlp *h, int64_t *count);
int nlm_mlp_get_params(nlm_mlp *h, float *params);
int nlm_mlp_set_params(nlm_mlp *h, const float *params);
/* Inference: y = net(x). */
int nlm_mlp_forward(nlm_mlp *h, const float *x, int64_t rows, float *y);
/* Mean squared error over rows x n_out and its gradient (params layout);
 * loss and grads may be NULL. */
int nlm_mlp_grad(nlm_mlp *h, const float *x, const float *t, int64_t rows, float *loss,
                 float *grads);
/* Upload a training set (kept on the device). */
int nlm_mlp_set_data(nlm_mlp *h, const float *x, const float *t, int64_t rows);
/* Minibatch Adam over the uploaded set (reshuffled each epoch from seed);
 * losses[e] = mean batch loss of epoch e (NULL to skip the readback). */
int nlm_mlp_train(nlm_mlp *h, int epochs, int batch, float lr, uint64_t seed, float *losses);

#ifdef __cplusplus
}
#endif

#endif /* NLMGPU_H */
