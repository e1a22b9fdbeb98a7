/*
 * sps.h -- C-ABI of the GB300 stress-particle SPH step library (libsps_gb300.so).
 *
 * The reference (CaitlinChalk/Stress-Particle-SPH, Fortran 90) advances one time
 * step with `time_integration` (code/2_SPH_main_2018.f90:78, public at :22), called
 * once per step by the driver (code/1_SPH_2018.f90:82).  All state lives in module
 * globals (code/5_SPH_global_vars_2018.f90, code/6_SPH_time_vars_2018.f90,
 * code/4_SPH_material_vars_2018.f90).  This header is the drop-in seam for that call:
 * the caller keeps its arrays, copies them in once (`sps_upload`), replaces every
 * `call time_integration` + `time_sph = time_sph + dt_sph` pair with `sps_step`, and
 * copies fields back (`sps_download`) before it writes output.
 *
 * Conventions
 *   - plain C types only: int32 counts, double / float / int32 arrays;
 *   - arrays use the reference's Fortran layout: x(2,N) is interleaved (x1,y1,x2,y2,..),
 *     stress(4,N) is (sxx,syy,sxy,szz) per particle, bc_info(8,N) column-major;
 *   - particle order is the reference's: nodes 1..nnode, stress-points
 *     nnode+1..ntotal, dummy wall particles ntotal+1..ntotal2 (0-based here);
 *   - every function returns an int status: SPS_OK (0) or a negative SPS_ERR_*;
 *     no C++ exception crosses the boundary; the message of the last failure on a
 *     context is available from sps_last_error;
 *   - a context owns one CUDA stream and its device buffers; it is used from one
 *     host thread at a time and is not re-entrant.
 */
#ifndef SPS_GB300_H
#define SPS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPS_OK 0
#define SPS_ERR_ARG (-1)         /* bad argument / inconsistent sizes              */
#define SPS_ERR_UNSUPPORTED (-2) /* option outside the implemented hot path        */
#define SPS_ERR_CUDA (-3)        /* CUDA runtime failure (no device, launch error) */
#define SPS_ERR_CAPACITY (-4)    /* neighbour / pair capacity exceeded             */
#define SPS_ERR_NONFINITE (-5)   /* NaN/Inf found in the state after a step        */
#define SPS_ERR_STATE (-6)       /* call out of order (e.g. step before upload)    */

/* arithmetic of the step */
#define SPS_PREC_FP64_PLAIN 0 /* FP64 with the reference's FP32 roundings (oracle-exact) */
#define SPS_PREC_FP32_FAST 1  /* FP32 pair arithmetic, compensated neighbour sums       */

/*
 * Problem description: the module variables that `time_integration` reads but never
 * writes.  Field names follow the reference's variable names.  Pointers are only read
 * during sps_create (the context keeps its own copies).
 */
typedef struct sps_params {
  /* counts (code/3_SPH_material_2018.f90 Read_2DMesh / set_up_dummy_nodes) */
  int32_t nnode;   /* velocity particles ("nodes")                            */
  int32_t nstress; /* stress-points                                           */
  int32_t ndummy;  /* all dummy wall particles (nrow * ndummy2)               */
  int32_t ndummy2; /* dummies of the innermost layer (ids ntotal+1..+ndummy2) */
  int32_t ndimn;   /* must be 2                                               */
  int32_t nstre;   /* must be 4                                               */
  int32_t ntype_solid; /* 1 plane stress (szz = nu (sxx+syy) in the return), 2 plane strain */

  /* solver flags (.dat `pa_sph nnps sle skf CSPM update_x XSPH`, input.txt) */
  int32_t sp_sph, inside_approach, cspm, xsph, update_x, cont_density, sle, skf;
  int32_t art_stress; /* Monaghan's artificial stress (artificial_force)              */

  /* material props(1,1..20): 1 ntype_eco, 2 ncrit, 3 E, 4 nu, 6 rho, 13 tan(phi), 14 c */
  double props[20];
  /* elastic constants exactly as the caller's module holds them
     (code/3_SPH_material_2018.f90:738-749: D11 = (4./3.)G + K with FP32 literals) */
  double D11, D12, D22, D33, D41, D42;
  double pi; /* module `pi` = 4*atan(1.0) evaluated in FP32 (:163) */
  double dx, dy;
  double dt_sph;
  double alpha, beta; /* artificial viscosity                        */
  double damping;     /* DampingTG                                   */

  /* gravity: cgrav * ft_grav * timecurve(tcurve_grav)(time_sph) */
  int32_t ic_grav, tcurve_grav;
  double cgrav[2];
  double ft_grav;

  /* time curves ttcurves(ntcurves,mptstcurves) (FP64), ftcurves(...) (FP32),
     column-major exactly as allocated by the reference */
  int32_t ntcurves, mptstcurves;
  const int32_t* nptstcurves;
  const double* ttcurves;
  const float* ftcurves;

  /* boundary conditions: bc_list(8,no_bcs) as read (column 7 already x twopi) */
  int32_t no_bcs, ifsigman;
  const double* bc_list;

  double xmin_domain[2], xmax_domain[2];

  /* dummy wall tables, length ntotal2 (entries below ntotal unused), FP32 like the reference */
  const float* wall_position;
  const float* horizontal_or_not;

  int32_t precision;      /* SPS_PREC_*                                      */
  int32_t max_neighbours; /* neighbour capacity per particle (two lists of half this size);
                             0 = sized from the kernel support at upload */

  /* outside approach (inside_approach = 0): input.txt `SPH_shifting vel_vector
     shift_update rx_factor ry_factor disp_tol` (code/3_SPH_material_2018.f90:388-396);
     stress-point j of node i is particle nnode + npoints*(i-1) + j */
  int32_t npoints;      /* stress-points per node (2 with vel_vector)                  */
  int32_t sph_shift;    /* SPH_shift: re-interpolate the step after a shift            */
  int32_t vel_vector;   /* orient the two stress-points along the node velocity        */
  int32_t shift_update; /* reposition the stress-points every shift_update steps (>= 1) */
  double r_x, r_y;      /* shift distances dx*rx_factor, dx*ry_factor                  */
  double disp_tol;      /* vel_vector: node displacement since the last shift, in dx,
                           above which its stress-points are repositioned              */

  /* Two constants that differ between the reference's source copies and that no input
     file carries; a caller passes the values of the copy it replaces.
     cspm_det_min: the CSPM determinant below which get_derivatives skips the correction,
       the default-real literal 1e-07 of the Drucker-Prager example's copy
       (example_problems/soil_failure_bui_et_al_2008/2_SPH_main_2018.f90:599) or 1e-03 of
       code/, the strain-localisation and the vertical-slope copies (same line), widened to
       double: (double)1e-07f or (double)1e-03f.
     bc_nodes_only: 1 when Normal_BCs applies the boundary conditions to the nodes only
       (`do ipoin = 1,nnode`: code/3_SPH_material_2018.f90:1664 and the strain-localisation
       copy), 0 when it applies them to nodes and stress-points (`1,ntotal`: the
       Drucker-Prager copy's 3_SPH_material_2018.f90:1683, the vertical-slope copy's :1664). */
  double cspm_det_min;
  int32_t bc_nodes_only;
} sps_params;

typedef struct sps_ctx sps_ctx;

/* Allocate a context on the current CUDA device.  Replaces the allocation part of
   Setup_Global_Arrays (code/3_SPH_material_2018.f90:883) for the hot-path arrays. */
int sps_create(const sps_params* p, sps_ctx** out);

/* Copy the dynamic state in (all arrays length ntotal2 unless noted):
   x(2,.), vel(2,.), stress(4,.), mass, rho, hsml, itype (1 SP, 2 node, 25 dummy),
   intvars1 = Internal_Vars(1,.) (length ntotal), f_drucker (length ntotal),
   x00(2,.) initial positions (displacement origin). */
int sps_upload(sps_ctx* ctx, const double* x, const double* vel, const double* stress,
               const double* mass, const double* rho, const double* hsml, const int32_t* itype,
               const double* intvars1, const double* f_drucker, const double* x00);

/* Boundary-condition bookkeeping of Get_BCs_on_node (code/3_SPH_material_2018.f90:1049):
   bc_or_not(ntotal), bc_info(8,ntotal). Optional when no_bcs == 0. */
int sps_upload_bcs(sps_ctx* ctx, const int32_t* bc_or_not, const int32_t* bc_info);

/* Advance nsteps steps.  Each step is `call time_integration` followed by
   `time_sph = time_sph + dt_sph` (code/1_SPH_2018.f90:82-83); *time_sph is read on entry
   and holds the advanced time on return (for a batch: time_sph[r] per realisation, each
   advanced by its own dt_sph).  Itimestep bookkeeping of the pair list (grid_find_NEW's
   linked-list reuse) is carried by the context across calls. */
int sps_step(sps_ctx* ctx, int32_t nsteps, double* time_sph);

/* Copy fields back; any pointer may be NULL to skip that field.
   x, vel: (2,ntotal2); stress: (4,ntotal2); rho: ntotal2; intvars1: ntotal;
   displ: (2,nnode); bc_or_not: ntotal; f_drucker: ntotal.  The stress of dummy particles
   is returned as 0: the reference only writes it as pair-local scratch inside
   get_derivatives (node--dummy pairs, 2_SPH_main_2018.f90:577-588) and never reads it
   outside that pair. */
int sps_download(sps_ctx* ctx, double* x, double* vel, double* stress, double* rho,
                 double* intvars1, double* displ, int32_t* bc_or_not, double* f_drucker);

/* The module arrays of get_nodes_on_free_surface (code/3_SPH_material_2018.f90:1135),
   which every step with update_x recomputes after the position update, for realisation r
   (0 for a single problem): normal(2,ntotal) (unit outward normal on surface particles, 0
   inside) and subset(ntotal) (1 on the free surface, 2 inside).  The routine's
   bc_or_not update (2 on the surface) is returned by sps_download. */
int sps_download_surface(sps_ctx* ctx, int32_t r, double* normal, int32_t* subset);

/* Test hook: the pair list of the last step in the reference's traversal order (the
   order its linked list `last -> next` is walked), after Pint_Update
   (code/3_SPH_material_2018.f90:1574): 1-based pair_i, pair_j, pint_type, and the FP32
   w, dwdx, dwdy.  Call with NULL arrays to get the count in *npairs; otherwise *npairs
   holds the capacity on entry and the count on return. */
int sps_dump_pairs(sps_ctx* ctx, int32_t* pair_i, int32_t* pair_j, int32_t* pint_type,
                   float* w, float* dwdx, float* dwdy, int64_t* npairs);

/* Which free-surface detection the FP32 form runs when a download or snapshot needs the
   surface of the last step (no reference counterpart: the reference has one precision).
   exact = 0 (the default): FP32 arithmetic, lists walked without the walk-order merge, so
   bc_or_not, subset and normals can differ from get_nodes_on_free_surface
   (code/3_SPH_material_2018.f90:1135) for particles at the scan region's edge; exact = 1:
   the reference's rounding and order, as in the FP64 plain form.  A detection that a later
   step reads (the traction-free BC, XSPH with BCs, the outside approach) is always exact.
   Takes effect from the next detection; the plain form ignores it. */
int sps_set_surface_detection(sps_ctx* ctx, int32_t exact);

/* The CUDA stream (a cudaStream_t) every launch of this context is issued on, so that a
   caller can order its own work or record CUDA events against it.  No reference
   counterpart (the reference has no device). */
int sps_get_stream(sps_ctx* ctx, void** stream);

/* Self-test (no reference counterpart): compare, on the device, the reciprocal-corrected
   division the step uses for quotients by a particle's density or smoothing length with
   the IEEE division, on n pseudo-random operand pairs; *mismatches counts results that
   differ in any bit. */
int sps_selftest_division(sps_ctx* ctx, int64_t n, uint64_t seed, int64_t* mismatches);

/* Self-test (no reference counterpart): compare, on the device, the FP64 <-> FP32
   conversions the FP32 form does on the integer pipe (round-to-nearest double -> float,
   the hi/lo split of a double into two floats, float -> double, and int -> float for
   the remainders below 2^29 that the split converts) with the hardware
   conversions, on n pseudo-random values; *mismatches counts results that differ in any
   bit. */
int sps_selftest_convert(sps_ctx* ctx, int64_t n, uint64_t seed, int64_t* mismatches);

/* Self-test (no reference counterpart): the stress return of both forms first certifies
   in FP32 that a stress lies inside the Drucker-Prager cone with a margin covering its
   roundings, and then skips the FP64 adapt_stress2.  On n pseudo-random materials and
   stresses (a quarter of them within a relative 1e-3 .. 1e-9 of the cone), *mismatches
   counts certified stresses that the FP64 return of either form would change in any bit
   (must be 0) and *certified the stresses certified. */
int sps_selftest_cone(sps_ctx* ctx, int64_t n, uint64_t seed, int64_t* mismatches,
                      int64_t* certified);

/* Launch-shape autotuner (no reference counterpart): time each tunable kernel (the pair
   search and lists, the interpolation, the derivative sums, the stress-return and RK
   kernels, XSPH) at block sizes 64, 128, 256 and 512 over nsteps profiled steps of the
   uploaded state, keep the fastest size per kernel, and restore the state, so the results
   of later steps are the same as without tuning.  blocks (may be NULL) receives the 8
   chosen sizes in that order.  The FP32 form then tunes its neighbour sums' look-ahead
   the same way (sps_tuned_lookahead), then their L2 prefetch (sps_tuned_prefetch).  The cell size is not tuned: the reference's pair
   order depends on it. */
int sps_autotune(sps_ctx* ctx, int32_t nsteps, int32_t* blocks);

/* The look-ahead of the FP32 form's neighbour sums that sps_autotune chose after the
   block sizes (no reference counterpart): ahead[0] neighbours a pass in the interpolation
   (2, 4 or 8), ahead[1] in the node derivative sums (1, 2 or 4); a pass loads its
   neighbours' list entries and records before it sums any of them, in the same order, so
   the results do not depend on these.  Defaults before tuning: 4 and 2. */
int sps_tuned_lookahead(sps_ctx* ctx, int32_t* ahead);

/* Whether the FP32 form's neighbour sums request their list entries into L2 ahead of use
   (no reference counterpart): *flags bit 0 for the interpolation, bit 1 for the
   derivative sums.  One lane of each warp issues a bulk L2 prefetch of the warp's entries;
   a hint that changes no result.  sps_autotune times both settings after the look-ahead
   and keeps the faster per group; the default before tuning is 0 (off). */
int sps_tuned_prefetch(sps_ctx* ctx, int32_t* flags);

/* Sets those flags directly (0 .. 3). */
int sps_set_prefetch(sps_ctx* ctx, int32_t flags);

/* Sets that look-ahead directly (interp 2, 4 or 8; derivs 1, 2 or 4), e.g. to reuse the
   values tuned on one context in another of the same workload. */
int sps_set_lookahead(sps_ctx* ctx, int32_t interp, int32_t derivs);

/* Number of this library's kernels one step launches (no reference counterpart). */
int sps_kernels_per_step(sps_ctx* ctx, int32_t* n);

/* Profiling hook (no reference counterpart): run nsteps steps launching each kernel with
   CUDA events around it on the context stream, and return the per-kernel totals.  names
   receives up to cap NUL-separated kernel names (names_len bytes), ms[k] the summed
   milliseconds and launches[k] the launch count of kernel k; *nkernels the number of
   distinct kernels.  The state advances exactly as with sps_step. */
int sps_profile_step(sps_ctx* ctx, int32_t nsteps, double* time_sph, char* names,
                     int32_t names_len, double* ms, int32_t* launches, int32_t cap,
                     int32_t* nkernels);

/* ---- batches (no reference counterpart: the reference runs one problem per process) ----
   A batch packs nreal independent problems (realisations) into one context: one launch per
   kernel and stage advances all of them, each with its own particle counts, material,
   dt_sph, gravity curve and domain.  Every realisation keeps its own cell grid and its own
   pair-list bookkeeping, so its results are bit-identical to a context holding it alone.
   The realisations must share the solver flags (sp_sph, inside_approach, cspm, xsph,
   update_x, cont_density, sle, skf, ntype_solid, precision, pi); boundary conditions
   (no_bcs > 0) need a batch of one.  sps_create(p) is sps_create_batch(1, p). */
int sps_create_batch(int32_t nreal, const sps_params* params, sps_ctx** out);
/* sps_upload / sps_download / sps_dump_pairs for realisation r, with r's arrays in the
   reference's layout and 1-based ids local to r. */
int sps_upload_real(sps_ctx* ctx, int32_t r, const double* x, const double* vel,
                    const double* stress, const double* mass, const double* rho,
                    const double* hsml, const int32_t* itype, const double* intvars1,
                    const double* f_drucker, const double* x00);
int sps_download_real(sps_ctx* ctx, int32_t r, double* x, double* vel, double* stress,
                      double* rho, double* intvars1, double* displ, int32_t* bc_or_not,
                      double* f_drucker);
int sps_dump_pairs_real(sps_ctx* ctx, int32_t r, int32_t* pair_i, int32_t* pair_j,
                        int32_t* pint_type, float* w, float* dwdx, float* dwdy,
                        int64_t* npairs);

/* Output staging without a host stall (no reference counterpart: the reference writes
   its output files from host arrays between steps: out_plot -> OutputRes,
   code/1_SPH_2018.f90:90-93,117-121 and code/3_SPH_material_2018.f90:2919).  sps_snapshot enqueues on
   the context stream a device-to-device copy of the fields sps_download returns (for every
   realisation; the free surface is refreshed first when it was left for the download),
   then copies that buffer to pinned host memory on a second stream, so that the
   sps_step calls that follow run while the copy is in flight.  sps_snapshot_wait blocks
   until the copy has finished and returns realisation r's fields exactly as
   sps_download_real would have at the snapshot (same arguments, any may be NULL);
   *step (may be NULL) receives the number of steps the context had taken then.  One
   snapshot is held: waiting again returns the same one, a new sps_snapshot replaces it. */
int sps_snapshot(sps_ctx* ctx);
int sps_snapshot_wait(sps_ctx* ctx, int32_t r, double* x, double* vel, double* stress,
                      double* rho, double* intvars1, double* displ, int32_t* bc_or_not,
                      double* f_drucker, int64_t* step);
/* sps_snapshot_wait without the copy: blocks the same way, then points each non-NULL
   argument at realisation r's field inside the snapshot's pinned host buffer (same layout
   as sps_download).  The pointers stay valid until the next sps_snapshot or
   sps_destroy. */
int sps_snapshot_view(sps_ctx* ctx, int32_t r, const double** x, const double** vel,
                      const double** stress, const double** rho, const double** intvars1,
                      const double** displ, const int32_t** bc_or_not, const double** f_drucker,
                      int64_t* step);

/* Copy the last error message of this context (or of the last failed sps_create when
   ctx is NULL) into buf (NUL-terminated, truncated to len). Returns its length. */
int sps_last_error(sps_ctx* ctx, char* buf, int32_t len);

void sps_destroy(sps_ctx* ctx);

/* ---- allocation-free neighbour statistics (no counterpart in the reference) -----------
   For callers that cannot call cudaMalloc -- hosts whose device memory is all reserved by
   their own pool allocator, so that a further cudaMalloc fails although the pool has room,
   and loops with a latency bound that may not take the device-wide synchronisation that
   cudaMalloc and cudaFree can imply.  No context is needed and no device memory is
   allocated: all device scratch is one fixed array of SPS_STATIC_SCRATCH_BYTES inside
   this library's device code, which limits a call to SPS_STATIC_MAX_PARTICLES particles.

   For the n particles x(2,n), hsml(n), on the current device: degree[a] = the number of
   particles b != a the step's pair test accepts (r < scale_k (h_a + h_b) / 2, scale_k = 2
   for skf 1 and 3 otherwise, the test of grid_find_NEW, code/2_SPH_main_2018.f90:1345-1353),
   wsum[a] = the sum over those b of the kernel value W_ab rounded to FP32 as the step
   stores it (kernel of code/2_SPH_main_2018.f90:1458-1560 with the caller's pi), and
   *npairs = the number of accepted pairs.  As in the step, b is looked for only in the
   3 x 3 cells (2 hmax wide) of the step's grid around a, so with skf 2 or 3 partners more
   than one cell away are not counted; the pair set is the one the step builds when every
   particle lies inside the domain.  The sums run in an unspecified order (rounding at the
   1e-16 relative level may differ between calls).
   stream: a cudaStream_t to run on, or NULL for the default stream; the call
   synchronises it before returning.  msg (msg_len bytes, may be NULL) receives a
   NUL-terminated message when the call fails.
   Returns SPS_ERR_CAPACITY when n > SPS_STATIC_MAX_PARTICLES or the particles span more
   than SPS_STATIC_MAX_CELLS cells of the grid, SPS_ERR_ARG for bad
   arguments (NULL pointers, skf outside 1..3, a non-finite position or a non-positive
   smoothing length), SPS_ERR_CUDA for a runtime failure.
   Every call looks the scratch array's address up in the current device's context
   (cudaGetSymbolAddress); the first call on a device, and the first after its context was
   reset, may load this library's device code there: make that call before any stream
   capture begins.  Every call on a device shares
   the one scratch array, so calls that overlapped would race on it: each call holds a
   process-wide lock and synchronises its stream before it returns, so calls from several
   host threads run one after another. */
#define SPS_STATIC_MAX_PARTICLES 65536
#define SPS_STATIC_MAX_CELLS 65536
#define SPS_STATIC_SCRATCH_BYTES 3670016 /* 3.5 MiB */
int sps_neighbour_stats_static(int32_t n, const double* x, const double* hsml, int32_t skf,
                               double pi, void* stream, int32_t* degree, double* wsum,
                               int64_t* npairs, char* msg, int32_t msg_len);

#ifdef __cplusplus
}
#endif
#endif /* SPS_GB300_H */
