/*
 * sps_oracle.h -- CPU oracle for the stress-particle SPH step (TEST INFRASTRUCTURE).
 *
 * This is a plain-C restatement of the reference's per-step hot path
 * (example_problems/soil_failure_bui_et_al_2008/2_SPH_main_2018.f90 time_integration and
 * the routines it calls, plus the constitutive routines of
 * example_problems/soil_failure_bui_et_al_2008/3_SPH_material_2018.f90).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and only as the
 * checker or the timed CPU baseline -- never as the product path.
 *
 * PARITY UNPINNED: the reference is Fortran and no Fortran compiler exists on either
 * machine of this build, and the reference ships no golden outputs or tests.  The oracle
 * is therefore pinned by its own known-answer and invariant tests, not by reference runs.
 *
 * The entry points mirror include/sps.h one for one (orc_* <-> sps_*), so a test can feed
 * both the same inputs and compare.
 */
#ifndef SPS_ORACLE_H
#define SPS_ORACLE_H
#include "../include/sps.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

int orc_create(const sps_params* p, orc_ctx** out);
int orc_upload(orc_ctx* c, const double* x, const double* vel, const double* stress,
               const double* mass, const double* rho, const double* hsml, const int32_t* itype,
               const double* intvars1, const double* f_drucker, const double* x00);
int orc_upload_bcs(orc_ctx* c, const int32_t* bc_or_not, const int32_t* bc_info);
int orc_step(orc_ctx* c, int32_t nsteps, double* time_sph);
int orc_download(orc_ctx* c, double* x, double* vel, double* stress, double* rho,
                 double* intvars1, double* displ, int32_t* bc_or_not, double* f_drucker);
/* the module arrays of get_nodes_on_free_surface after the last step: normal(2,ntotal),
   subset(ntotal) (1 = on the free surface, 2 = inside) */
int orc_download_surface(orc_ctx* c, double* normal, int32_t* subset);
int orc_dump_pairs(orc_ctx* c, int32_t* pair_i, int32_t* pair_j, int32_t* pint_type, float* w,
                   float* dwdx, float* dwdy, int64_t* npairs);
void orc_destroy(orc_ctx* c);

/* kernel() (2_SPH_main_2018.f90:1440) exposed for known-answer tests */
void orc_kernel(int32_t skf, double pi, double r, const double* dx2, double hsml, double* w,
                double* dwdx);
/* adapt_stress2 (3_SPH_material_2018.f90:2087) on one stress vector, for invariant tests */
void orc_adapt_stress(double tanfi, double coh, double* stress4);
/* artificial_force over the current pair list and state: art_force (2,nnode) */
void orc_artificial_force(orc_ctx* c, double* out);
/* the viscoplastic laws of plastic_terms (ncrit 1-4): vivel and Gs = -Dmatx vivel */
void orc_viscoplastic(const double* props, int ntype_solid, const double* stress4, double iv1,
                      double* vivel, double* Gs);
/* drucker_prager (3_SPH_material_2018.f90:1958) on one stress-point, for tests.
   f_drucker is read and updated; G and vivel receive 4 values. */
void orc_drucker_prager(const double* props, double time_sph, const double* stress4,
                        const double* grad_u4, double* f_drucker, double* G, double* vivel);

#ifdef __cplusplus
}
#endif
#endif
