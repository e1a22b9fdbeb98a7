/*
 * sph_host.h -- host side above the step C-ABI (libsph_host.so).
 *
 * The reference's set-up path (problem_input_data, setup_particles, Read_2DMesh,
 * set_up_dummy_nodes, Setup_Global_Arrays, Get_BCs_on_node, Initial_conditions in
 * example_problems/soil_failure_bui_et_al_2008/3_SPH_material_2018.f90:37-1569) stays
 * outside the GPU hot path.  Because no Fortran compiler is available to build it, this
 * library restates it in C++ so that a caller without the Fortran driver can produce the
 * exact module state that `time_integration` starts from, and hands it to sps_upload.
 *
 * It also holds the synthetic workload generators used by the benchmark (granular column
 * with a K0 geostatic stress, vertical slope on a foundation).  These go beyond what the
 * reference's rectangle-only generator and zero/constant initial conditions can express.
 */
#ifndef SPH_HOST_H
#define SPH_HOST_H
#include <stdint.h>

#include "sps.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sph_problem sph_problem;

/* pointers into the problem's own arrays (valid until sph_problem_free) */
typedef struct sph_problem_arrays {
  int32_t ntotal2;
  double *x, *vel, *stress, *mass, *rho, *hsml, *intvars1, *f_drucker, *x00;
  int32_t *itype, *bc_or_not, *bc_info;
  float *wall_position, *horizontal_or_not;
} sph_problem_arrays;

/* run control read by the driver loop (code/1_SPH_2018.f90:50-106) */
typedef struct sph_run_block {
  double dt, time_end;
  int32_t maxtimestep, print_step, save_step, plot_step;
} sph_run_block;

/* Read a problem directory holding input.txt, <name>.dat and <name>.pts in the
   Drucker-Prager example's format (`ntype_solid nstre nmats` on the material header line;
   the two-value `nstre nmats` form of the other examples is accepted too). */
int sph_problem_read(const char* dir, sph_problem** out, char* err, int32_t errlen);

/* Same reader on in-memory file contents. */
int sph_problem_parse(const char* input_txt, const char* dat, const char* pts, sph_problem** out,
                      char* err, int32_t errlen);

/* Granular column collapse: a width x height block of cohesionless Drucker-Prager soil on
   a floor with a left wall (3 dummy rows each), inside approach, one stress-point per
   cell, cubic kernel h = sml*dx, gravity, and a K0 geostatic initial stress
   (syy = -rho g depth, sxx = szz = K0 syy) on nodes and stress-points. The
   reference-format text is generated and parsed by sph_problem_parse, then the K0 stress
   is applied. */
typedef struct sph_column_spec {
  double width, height, dx, sml;
  double young, poiss, rho, phi_deg, cohesion, k0;
  double floor_length; /* floor wall extent to the right of x = 0 */
  double dt;           /* 0 -> 0.1 h / sqrt(E/rho) */
  double alpha, beta, damping;
  int32_t xsph, cspm;
} sph_column_spec;
int sph_problem_column(const sph_column_spec* spec, sph_problem** out);

/* Biaxial compression sample [0,width]x[0,height], no walls or gravity: the top and bottom
   node rows are rough platens (vx = 0, vy = -/+ platen_v ramped in linearly over t_ramp),
   the side columns carry the normal stress sxx = -confining and sxy = 0, all as the
   reference's segment BCs (Normal_BCs, 3_SPH_material_2018.f90:1666), the layout of its
   strain-localisation example.  Initial stress sxx = szz = -confining, syy = -confining -
   q_ratio * q_y, with q_y the axial excess that puts the state on the Drucker-Prager cone
   (0 <= q_ratio < 1).  A stress BC sets the boundary nodes' stress; it does not add the
   traction to their momentum balance, whose neighbour sums stay one-sided, so a compressive
   confining value pushes the sides outwards instead of confining the sample: the
   localisation example uses 0, as do the defaults of the bindings. */
typedef struct sph_biaxial_spec {
  double width, height, dx, sml;
  double young, poiss, rho, phi_deg, cohesion;
  double confining;  /* Pa, > 0 in compression */
  double platen_v;   /* m/s, each platen towards the middle */
  double t_ramp;     /* s, > 0 */
  double q_ratio;
  double dt;         /* 0 -> 0.1 h / sqrt(E/rho) */
} sph_biaxial_spec;
int sph_problem_biaxial(const sph_biaxial_spec* spec, sph_problem** out);

/* Vertical slope: a foundation [0,Lf]x[0,Hf] with a block [0,Ls]x[Hf,Hf+Hs] on top (vertical
   face at x = Ls), floor and side walls around the foundation, K0 stress, gravity ramped
   from 0 to 1 over t_ramp by a time curve. Masses follow the reference's rule (each node
   carries a quarter cell per adjacent cell, stress-points one cell). */
typedef struct sph_slope_spec {
  double Lf, Hf, Ls, Hs, dx, sml;
  double young, poiss, rho, phi_deg, cohesion, k0;
  double t_ramp;
  double dt; /* 0 -> 0.1 h / sqrt(E/rho) */
  double alpha, beta, damping;
  int32_t xsph;
  double face_deg; /* angle of the slope face from the horizontal; 0 or 90: vertical face
                      at x = Ls, else the face runs from the crest (Ls, Hf + Hs) down to
                      the toe (Ls + Hs / tan(face), Hf), which must lie on the foundation */
} sph_slope_spec;
int sph_problem_slope(const sph_slope_spec* spec, sph_problem** out);

const sps_params* sph_problem_params(const sph_problem* p);

/* sizeof(sps_params) as this library was compiled, for bindings that mirror the struct */
int32_t sph_sizeof_params(void);

/* The output flags read by problem_input_data (code/3_SPH_material_2018.f90:333-336):
   stress_out(1:4), vel_out(1:2), strain_out, rho_out, sml_out, disp_out. */
int sph_problem_output_flags(const sph_problem* p, int32_t* flags);

/* OutputRes (code/3_SPH_material_2018.f90:2750-3010) for a driver without the Fortran
   writers.  In directory dir: nodes.csv.NNNNNN, stress_points.csv.NNNNNN and
   surface_points.csv.NNNNNN (NNNNNN = itimestep) with the columns the output flags select,
   F16.8 fields, separators and headers as the reference writes them; and the step's GiD
   result blocks (displacement, velocity, sxx/syy/sxy, plastic strain) appended to
   <name>.post.res.  Arrays in the reference layout as sps_download returns them: x, vel
   (2,ntotal2), stress (4,ntotal2), intvars1, rho, hsml, bc_or_not (ntotal), displ
   (2,nnode); intvars1, rho, hsml, bc_or_not and displ may be NULL (written as 0).  The
   list-directed lines (surface points, GiD) have compiler-specific spacing in the
   reference; here each value is one blank-separated field with 17 significant digits. */
int sph_write_output(sph_problem* p, const char* dir, int32_t itimestep, double time_sph,
                     const double* x, const double* vel, const double* stress,
                     const double* intvars1, const double* rho, const double* hsml,
                     const int32_t* bc_or_not, const double* displ);

/* OutputMesh (code/3_SPH_material_2018.f90:2707-2744): <name>.post.msh with the initial
   node coordinates and, for problems built by the rectangle generator, its quadrilateral
   cells numbered as Read_2DMesh numbers them (code/3_SPH_material_2018.f90:515-532); then
   starts <name>.post.res with the GiD header. */
int sph_write_mesh(sph_problem* p, const char* dir);
int sph_problem_get_arrays(sph_problem* p, sph_problem_arrays* out);
int32_t sph_problem_nblocks(const sph_problem* p);
int sph_problem_block(const sph_problem* p, int32_t i, sph_run_block* out);
const char* sph_problem_name(const sph_problem* p);
void sph_problem_free(sph_problem* p);

#ifdef __cplusplus
}
#endif
#endif
