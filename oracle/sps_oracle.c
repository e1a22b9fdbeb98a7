/*
 * sps_oracle.c -- CPU oracle of the stress-particle SPH step.  TEST INFRASTRUCTURE ONLY:
 * loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the
 * product path.
 *
 * PARITY UNPINNED: the reference is Fortran 90; no Fortran compiler exists on either
 * machine of this build and the reference ships no golden outputs, so this restatement is
 * pinned only by its own known-answer and invariant tests (tests/test_oracle_*.py).
 *
 * It restates, routine by routine and in the same floating-point operation order, the
 * Drucker-Prager example's copy of the reference (paths below are relative to
 * example_problems/soil_failure_bui_et_al_2008/):
 *   2_SPH_main_2018.f90   time_integration :78, XSPH_update :189, stress_point_update :403,
 *                         get_derivatives :487, RK4 :653, density_update :807,
 *                         artificial_viscosity :826, get_spin_rate_tensor :1021,
 *                         boundary_forces :1039, Check_Out_Domain :1170,
 *                         grid_find_NEW :1199, kernel :1440
 *   3_SPH_material_2018.f90  Pint_Update :1574, BCs/Normal_BCs :1641/:1665,
 *                         update_strain :1864, plastic_terms :1884, drucker_prager :1958,
 *                         adapt_stress2 :2087, Get_derivative_intvars :2697,
 *                         gravity_force :2809
 * Mixed precision is reproduced: FP32 `real` locals become `float`, FP32 literals such as
 * 2./3. stay float, pair kernel values are stored as float (5_SPH_global_vars_2018.f90:19-21).
 * Build with -ffp-contract=off so no multiply-add is fused (gfortran -O3 on x86-64 has no
 * FMA instructions available).
 *
 * Pair order: grid_find_NEW keeps its pairs in a linked list that is walked from `last`;
 * new nodes are prepended and old nodes are refilled in list order
 * (2_SPH_main_2018.f90:1309-1401).  Every scatter loop of the reference accumulates in
 * that walk order, so the oracle keeps the pairs in creation order and walks them through
 * the permutation `order[]` that the linked list produces (see build_walk_order).
 */
#include "sps_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct orc_ctx {
  sps_params p;
  int NN, NT, N2; /* nnode, ntotal, ntotal2 */
  int32_t *nptstcurves;
  double *ttcurves;
  float *ftcurves;
  double *bc_list;
  float *wall_position, *horizontal_or_not;
  /* state (Fortran layouts) */
  double *x, *vel, *stress, *mass, *rho, *hsml, *x00, *x0, *vx0, *displ;
  int32_t *itype, *out_domain, *bc_or_not, *bc_info, *bc_int;
  double *intvars1, *f_drucker, *grad_u, *Ddev;
  double *f_bound, *art_visc, *art_force;
  /* outside approach: itimestep_sph of the step being taken (0 before the first step after
     an upload), and the velocity-vector variant's x_10(2,nnode), disp_10(nnode) */
  int64_t itimestep;
  double *x10, *disp10;
  double *normal, *subset; /* module arrays of get_nodes_on_free_surface, (2,ntotal), (ntotal) */
  /* pair list, creation order */
  int64_t npairs, cap, m_pairs;
  int32_t *pi, *pj, *ptype;
  float *pw, *pdx, *pdy;
  int64_t *order; /* walk position -> creation index */
  /* scratch */
  int32_t *which_cell, *cell_cnt, *cell_start, *cell_list;
  int64_t cell_cap;
  double time_sph;
  int uploaded;
  int step_count;
};

#define X(c, d, i) ((c)->x[(d) + 2 * (size_t)(i)])
#define V(c, d, i) ((c)->vel[(d) + 2 * (size_t)(i)])
#define S(c, k, i) ((c)->stress[(k) + 4 * (size_t)(i)])

static void* xcalloc(size_t n, size_t sz) {
  void* p = calloc(n ? n : 1, sz);
  return p;
}

/* ------------------------------------------------------------------------------------
 * kernel (2_SPH_main_2018.f90:1440-1538).  FP64 except the FP32 literal 2./3. (:1480).
 * x**n with a constant n is expanded by gfortran into multiplications: x**2 = x*x,
 * x**3 = (x*x)*x, x**4 = (x*x)*(x*x), x**5 = ((x*x)*x)*(x*x).
 * ---------------------------------------------------------------------------------- */
void orc_kernel(int32_t skf, double pi, double r, const double* dx2, double hsml, double* w,
                double* dwdx) {
  double q = r / hsml;
  double factor;
  *w = 0.0;
  dwdx[0] = 0.0;
  dwdx[1] = 0.0;
  if (skf == 1) {
    factor = 15.0 / (7.0 * pi * hsml * hsml);
    if (q >= 0 && q <= 1.0) {
      const double two_thirds = (double)(2.0f / 3.0f);
      *w = factor * ((two_thirds - q * q) + (q * q * q) / 2.0);
      for (int d = 0; d < 2; d++) dwdx[d] = ((factor * (-2.0 + 1.5 * q)) / (hsml * hsml)) * dx2[d];
    } else if (q > 1.0 && q <= 2.0) {
      double t = 2.0 - q;
      *w = (factor / 6.0) * ((t * t) * t);
      for (int d = 0; d < 2; d++)
        dwdx[d] = -(((((factor / 6.0) * 3.0) * (t * t)) / hsml) * (dx2[d] / r));
    }
  } else if (skf == 2) {
    factor = 1.0 / ((hsml * hsml) * pi);
    if (q >= 0 && q <= 3.0) {
      *w = factor * exp(-(q * q));
      for (int d = 0; d < 2; d++) dwdx[d] = *w * (((-2.0 * dx2[d]) / hsml) / hsml);
    }
  } else if (skf == 3) {
    factor = 7.0 / (478.0 * pi * hsml * hsml);
    double a = 3.0 - q, b = 2.0 - q, c1 = 1.0 - q;
    double a2 = a * a, b2 = b * b, c2 = c1 * c1;
    double a4 = a2 * a2, b4 = b2 * b2;
    double a5 = (a2 * a) * a2, b5 = (b2 * b) * b2, c5 = (c2 * c1) * c2;
    if (q >= 0 && q <= 1.0) {
      *w = factor * ((a5 - 6.0 * b5) + 15.0 * c5);
      for (int d = 0; d < 2; d++)
        dwdx[d] = factor * ((((-120.0 + 120.0 * q) - 50.0 * (q * q)) / (hsml * hsml)) * dx2[d]);
    } else if (q > 1.0 && q <= 2.0) {
      *w = factor * (a5 - 6.0 * b5);
      for (int d = 0; d < 2; d++)
        dwdx[d] = ((factor * (-5.0 * a4 + 30.0 * b4)) / hsml) * (dx2[d] / r);
    } else if (q > 2.0 && q <= 3.0) {
      *w = factor * a5;
      for (int d = 0; d < 2; d++) dwdx[d] = ((factor * (-5.0 * a4)) / hsml) * (dx2[d] / r);
    }
  }
}

/* adapt_stress2 body for one particle (3_SPH_material_2018.f90:2087-2161), FP64 */
static void adapt_one(double alpha2, double kc, double* s) {
  double smean = ((s[0] + s[1]) + s[3]) / 3.0;
  double d0 = s[0] - smean, d1 = s[1] - smean, d2 = s[2], d3 = s[3] - smean;
  double varj2 = d2 * d2 + 0.5 * ((d0 * d0 + d1 * d1) + d3 * d3);
  double yield = -((alpha2 * 3.0) * smean) + kc;
  if (yield < 0) {
    double shift = kc / (3.0 * alpha2);
    s[0] = (s[0] - smean) + shift;
    s[1] = (s[1] - smean) + shift;
    s[3] = (s[3] - smean) + shift;
    smean = ((s[0] + s[1]) + s[3]) / 3.0;
    d0 = s[0] - smean;
    d1 = s[1] - smean;
    d2 = s[2];
    d3 = s[3] - smean;
    varj2 = d2 * d2 + 0.5 * ((d0 * d0 + d1 * d1) + d3 * d3);
    yield = -((alpha2 * 3.0) * smean) + kc;
  }
  double sj = sqrt(varj2);
  if (yield < sj) {
    double rn = (-((3.0 * alpha2) * smean) + kc) / sj;
    if (sj <= (double)1e-5f) rn = 0.0;
    s[0] = rn * d0 + smean;
    s[1] = rn * d1 + smean;
    s[3] = rn * d3 + smean;
    s[2] = rn * d2;
  }
}

static void dp_constants(double tanfi, double coh, double* alpha2, double* kc) {
  double den = sqrt(9.0 + 12.0 * (tanfi * tanfi));
  *alpha2 = tanfi / den;
  *kc = (3.0 * coh) / den;
}

void orc_adapt_stress(double tanfi, double coh, double* stress4) {
  double a2, kc;
  dp_constants(tanfi, coh, &a2, &kc);
  adapt_one(a2, kc, stress4);
}

/* drucker_prager (3_SPH_material_2018.f90:1958-2083): FP32 body, FP64 interface */
static void drucker_prager(const double* props, double time_sph, const double* s,
                           const double* gu /* grad_u(2,2) of this SP */, double* f_dp,
                           double* G, double* vivel) {
  double f0 = *f_dp;
  float tanfi = (float)props[12], coh = (float)props[13];
  float young = (float)props[2], poiss = (float)props[3];
  float smean = (float)(((s[0] + s[1]) + s[3]) / 3.0);
  float devia[4];
  devia[0] = (float)(s[0] - (double)smean);
  devia[1] = (float)(s[1] - (double)smean);
  devia[2] = (float)s[2];
  devia[3] = (float)(s[3] - (double)smean);
  float varj2 = devia[2] * devia[2] +
                0.5f * ((devia[0] * devia[0] + devia[1] * devia[1]) + devia[3] * devia[3]);
  float vari1 = 3.0f * smean;
  float eps11 = (float)gu[0];                      /* grad_u(1,1) */
  float eps12 = (float)(0.5 * (gu[2] + gu[1]));    /* 0.5*(grad_u(1,2)+grad_u(2,1)) */
  float eps22 = (float)gu[3];                      /* grad_u(2,2) */
  float emean = eps11 + eps22;
  float alpha2 = tanfi / sqrtf(9.0f + 12.0f * (tanfi * tanfi));
  float kc = (3.0f * coh) / sqrtf(9.0f + 12.0f * (tanfi * tanfi));
  float yield = -(alpha2 * vari1) + kc;
  float sj = sqrtf(varj2);
  *f_dp = (double)(sj - yield);
  float f1 = (float)(*f_dp);
  double df = (double)f1 - f0;
  float G_mod = young / (2.0f * (1.0f + poiss));
  float K_mod = young / (3.0f * (1.0f - 2.0f * poiss));
  float s_eps = (devia[0] * eps11 + (2.0f * devia[2]) * eps12) + devia[1] * eps22;
  if (time_sph > 0 && f1 >= 0 && df >= 0 && sj >= 1e-5f) {
    float G1[4];
    for (int i = 0; i < 4; i++) G1[i] = (G_mod / sj) * devia[i];
    float lambda_1 = ((3.0f * alpha2) * K_mod) * emean;
    float lambda_2 = (G_mod / sj) * s_eps;
    float lambda_3 = G_mod;
    float G2 = (lambda_1 + lambda_2) / lambda_3;
    for (int i = 0; i < 4; i++) G[i] = (double)(G1[i] * G2);
    const float sixth = 1.0f / 6.0f;
    float rs = 1.0f / sj;
    vivel[0] = (double)((sixth * rs) * ((2.0f * devia[0] - devia[1]) - devia[3]));
    vivel[1] = (double)((sixth * rs) * ((2.0f * devia[1] - devia[0]) - devia[3]));
    vivel[2] = (double)(rs * devia[2]);
    vivel[3] = (double)((sixth * rs) * ((2.0f * devia[3] - devia[0]) - devia[1]));
    for (int i = 0; i < 4; i++) vivel[i] = vivel[i] * (double)G2;
  } else {
    for (int i = 0; i < 4; i++) {
      G[i] = 0.0;
      vivel[i] = 0.0;
    }
  }
}

void orc_drucker_prager(const double* props, double time_sph, const double* stress4,
                        const double* grad_u4, double* f_drucker, double* G, double* vivel) {
  drucker_prager(props, time_sph, stress4, grad_u4, f_drucker, G, vivel);
}

/* The viscoplastic laws (ncrit 1 Tresca, 2 von Mises, 3 Mohr-Coulomb, 4 Drucker-Prager;
   Perzyna flow), 2D branches (ntype_solid 1-3), in the reference's operation order:
     Get_Vivel :2165-2228, invar09 :2233-2377, yieldf09 :2381-2556, flowvp09 :2560-2609,
     Get_Dmatx :2614-2691 (3_SPH_material_2018.f90).
   The same routines, with the same 2D arithmetic, are in the strain-localisation and
   vertical-slope examples' copies, whose inputs use them.  FP32 literals are kept as
   floats: root3 = sqrt(3.00) is an FP32 square root, the degree factor 0.017453292, the
   radian factor 57.29577951308, the flow rule's root3 = 1.73205080757 and allow = 0.01 are
   FP32 constants widened to FP64.  props: 3 E, 4 nu, 7 yield stress, 8 hardening modulus,
   9 friction angle (degrees), 10 gamma, 11 delta, 12 n (1-based as in the .dat file). */
#define VP_RAD ((double)0.017453292f)
static double vp_root3(void) { return (double)sqrtf(3.0f); }

/* invar09 (2D): invariants, the yield function value and the current yield-surface size */
static void vp_invar(const double* props, const double* s, double iv1, double* devia,
                     double* smean, double* varj2, double* sint3, double* theta, double* steff,
                     double* yield, double* fdatm) {
  const double root3 = vp_root3();
  const int ncrit = (int)props[1];
  *smean = ((s[0] + s[1]) + s[3]) / 3.0;
  devia[0] = s[0] - *smean;
  devia[1] = s[1] - *smean;
  devia[2] = s[2];
  devia[3] = s[3] - *smean;
  *varj2 = devia[2] * devia[2] +
           0.5 * ((devia[0] * devia[0] + devia[1] * devia[1]) + devia[3] * devia[3]);
  const double varj3 = devia[3] * (devia[3] * devia[3] - *varj2);
  *steff = sqrt(*varj2);
  if (*steff != 0.0) {
    *sint3 = -(((3.0 * root3) * varj3) / ((2.0 * *varj2) * *steff));
    if (*sint3 > 1.0) *sint3 = 1.0;
  } else {
    *sint3 = 0.0;
  }
  if (*sint3 < -1.0) *sint3 = -1.0;
  if (*sint3 > 1.0) *sint3 = 1.0;
  *theta = asin(*sint3) / 3.0;
  double snphi;
  switch (ncrit) {
    case 1:
      *yield = (2.0 * cos(*theta)) * *steff;
      break;
    case 2:
      *yield = root3 * *steff;
      break;
    case 3:
      snphi = sin(props[8] * VP_RAD);
      *yield = *smean * snphi + *steff * (cos(*theta) - (sin(*theta) * snphi) / root3);
      break;
    default: /* 4 */
      snphi = sin(props[8] * VP_RAD);
      *yield = ((6.0 * *smean) * snphi) / (root3 * (3.0 - snphi)) + *steff;
      break;
  }
  /* linear hardening, limited to a tenth of the initial size (the reference stops the run
     when the initial size is not above 0.001; sps_create rejects such materials) */
  const double fdatm0 = props[6], hards = props[7];
  double f = fdatm0 + hards * iv1;
  double fact = fabs(f) / fabs(fdatm0);
  if (fact < (double)0.1f) fact = (double)0.1f;
  *fdatm = fdatm0 * fact;
}

/* yieldf09 (2D): the flow vector df/ds */
static void vp_avect(const double* props, const double* devia, double varj2, double theta,
                     double steff, double* avect) {
  const double root3 = vp_root3();
  const int ncrit = (int)props[1];
  const double frict = props[8];
  const double tanth = tan(theta), tant3 = tan(3.0 * theta), sinth = sin(theta),
               costh = cos(theta), cost3 = cos(3.0 * theta);
  const double veca1[4] = {1.0, 1.0, 0.0, 1.0};
  double veca2[4] = {0.0, 0.0, 0.0, 0.0}, veca3[4];
  if (steff > 0) {
    for (int i = 0; i < 4; i++) veca2[i] = devia[i] / (2.0 * steff);
    veca2[2] = devia[2] / steff;
  }
  veca3[0] = devia[1] * devia[3] + varj2 / 3.0;
  veca3[1] = devia[0] * devia[3] + varj2 / 3.0;
  veca3[2] = -((2.0 * devia[2]) * devia[3]);
  veca3[3] = (devia[0] * devia[1] - devia[2] * devia[2]) + varj2 / 3.0;
  double cons1 = 0.0, cons2 = 0.0, cons3 = 0.0;
  const double abthe = fabs(theta * (double)57.29577951308f);
  if (ncrit == 1) {
    if (abthe >= 29.0) {
      cons2 = root3;
      cons3 = 0.0;
    } else {
      cons2 = 2.0 * (costh + sinth * tant3);
      cons3 = (root3 * sinth) / (varj2 * cost3);
    }
  } else if (ncrit == 2) {
    cons2 = root3;
  } else if (ncrit == 3) {
    cons1 = sin(frict * VP_RAD) / 3.0;
    if (abthe >= 29.0) {
      double plumi = 1.0;
      if (theta > 0.0) plumi = -1.0;
      cons2 = 0.5 * (root3 + (plumi * cons1) * root3);
      cons3 = 0.0;
    } else {
      cons2 = costh * ((1.0 + tanth * tant3) + (cons1 * (tant3 - tanth)) * root3);
      cons3 = (root3 * sinth + (3.0 * cons1) * costh) / ((2.0 * varj2) * cost3);
    }
  } else { /* 4 */
    const double snphi = sin(frict * VP_RAD);
    cons1 = (2.0 * snphi) / (root3 * (3.0 - snphi));
    cons2 = 1.0;
  }
  for (int i = 0; i < 4; i++) avect[i] = (cons1 * veca1[i] + cons2 * veca2[i]) + cons3 * veca3[i];
}

/* Get_Vivel (2D) with flowvp09: the viscoplastic strain rate */
static void vp_vivel(const double* props, const double* s, double iv1, double* vivel) {
  double devia[4], smean, varj2, sint3, theta, steff, yield, fdatm;
  for (int i = 0; i < 4; i++) vivel[i] = 0.0;
  vp_invar(props, s, iv1, devia, &smean, &varj2, &sint3, &theta, &steff, &yield, &fdatm);
  if (!(yield > fdatm)) return;
  double avect[4];
  vp_avect(props, devia, varj2, theta, steff, avect);
  const double gamma = props[9], delta = props[10], nflow = props[11];
  const double fnorm = (yield - fdatm) / fdatm;
  if (fnorm >= (double)0.01f) {
    double cmult;
    if (nflow != 1) cmult = gamma * (exp(delta * fnorm) - 1.0);
    else cmult = gamma * pow(fnorm, delta);
    for (int i = 0; i < 4; i++) vivel[i] = cmult * avect[i];
  }
}

/* Get_Dmatx (2D): the isotropic elastic matrix */
static void vp_dmatx(const double* props, int ntype_solid, double D[4][4]) {
  const double young = props[2], poiss = props[3];
  memset(D, 0, sizeof(double) * 16);
  if (ntype_solid == 1) {
    const double c = young / (1.0 - poiss * poiss);
    D[0][0] = c;
    D[1][1] = c;
    D[0][1] = c * poiss;
    D[1][0] = c * poiss;
    D[2][2] = ((1.0 - poiss) * c) / 2.0;
  } else {
    const double c = (young * (1.0 - poiss)) / ((1.0 + poiss) * (1.0 - 2.0 * poiss));
    const double cp = (c * poiss) / (1.0 - poiss);
    D[0][0] = c;
    D[1][1] = c;
    D[0][1] = cp;
    D[1][0] = cp;
    D[0][3] = cp;
    D[1][3] = cp;
    D[3][0] = cp;
    D[3][1] = cp;
    D[3][3] = c;
    if (ntype_solid == 2) D[2][2] = ((1.0 - 2.0 * poiss) * c) / (2.0 * (1.0 - poiss));
    else D[2][2] = (c * (1.0 - 2.0 * poiss)) / (2.0 * (1.0 - poiss));
  }
}

void orc_viscoplastic(const double* props, int ntype_solid, const double* stress4, double iv1,
                      double* vivel, double* Gs) {
  double D[4][4];
  vp_vivel(props, stress4, iv1, vivel);
  vp_dmatx(props, ntype_solid, D);
  for (int i = 0; i < 4; i++) {
    Gs[i] = 0.0;
    for (int j = 0; j < 4; j++) Gs[i] = Gs[i] - D[i][j] * vivel[j];
  }
}

/* plastic_terms (3_SPH_material_2018.f90:1884-1954) + Get_derivative_intvars 2D branch
   (:2767-2775).  Returns Gs (= -G) and der_intvars(1). */
static void plastic_terms(orc_ctx* c, int ie, const double* fi, double* Gs, double* der1) {
  const double* props = c->p.props;
  int ntype_eco = (int)props[0];
  int ncrit = (int)props[1];
  double vivel[4] = {0, 0, 0, 0}, G2[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; k++) Gs[k] = 0.0;
  if (ntype_eco > 1) {
    double poiss = props[3];
    double s2[4] = {fi[0], fi[1], fi[2], fi[3]};
    if (c->p.ntype_solid == 1) s2[3] = poiss * (s2[0] + s2[1]);
    if (ncrit <= 5) {
      orc_viscoplastic(props, c->p.ntype_solid, s2, c->intvars1[ie], vivel, Gs);
    } else if (ncrit == 12) {
      drucker_prager(props, c->time_sph, s2, &c->grad_u[4 * (size_t)ie], &c->f_drucker[ie], G2,
                     vivel);
      for (int k = 0; k < 4; k++) Gs[k] = -G2[k];
    }
    *der1 = sqrt((2.0 * ((vivel[0] * vivel[0] + vivel[1] * vivel[1]) + vivel[3] * vivel[3]) +
                  vivel[2] * vivel[2]) /
                 3.0);
  } else {
    *der1 = 0.0;
  }
}

/* Check_Out_Domain (2_SPH_main_2018.f90:1170-1194) */
static void check_out_domain(orc_ctx* c) {
  for (int i = 0; i < c->N2; i++)
    for (int d = 0; d < 2; d++) {
      double dxx = (X(c, d, i) - c->p.xmin_domain[d]) * (X(c, d, i) - c->p.xmax_domain[d]);
      if (dxx > 0.0) c->out_domain[i] = 1;
    }
}

static int ensure_pair_cap(orc_ctx* c, int64_t need) {
  if (need <= c->cap) return 0;
  int64_t nc = c->cap ? c->cap : 1024;
  while (nc < need) nc *= 2;
  int32_t* a = realloc(c->pi, nc * sizeof(int32_t));
  if (!a) return -1;
  c->pi = a;
  a = realloc(c->pj, nc * sizeof(int32_t));
  if (!a) return -1;
  c->pj = a;
  a = realloc(c->ptype, nc * sizeof(int32_t));
  if (!a) return -1;
  c->ptype = a;
  float* f = realloc(c->pw, nc * sizeof(float));
  if (!f) return -1;
  c->pw = f;
  f = realloc(c->pdx, nc * sizeof(float));
  if (!f) return -1;
  c->pdx = f;
  f = realloc(c->pdy, nc * sizeof(float));
  if (!f) return -1;
  c->pdy = f;
  int64_t* o = realloc(c->order, nc * sizeof(int64_t));
  if (!o) return -1;
  c->order = o;
  c->cap = nc;
  return 0;
}

/* Walk order of grid_find_NEW's linked list (2_SPH_main_2018.f90:1309-1401).  With m the
   number of list nodes before this step and n the pairs found now, pair k (creation order)
   refills the k-th node from `last` when k < m; pairs k >= m get new nodes prepended, so the
   walk is pairs n-1, n-2, ..., m followed by 0, 1, ..., min(n,m)-1. */
static void build_walk_order(orc_ctx* c) {
  int64_t n = c->npairs, m = c->m_pairs, k = 0;
  for (int64_t a = n - 1; a >= m; a--) c->order[k++] = a;
  for (int64_t a = 0; a < (n < m ? n : m); a++) c->order[k++] = a;
  if (n > c->m_pairs) c->m_pairs = n;
}

/* grid_find_NEW (2_SPH_main_2018.f90:1199-1435) with kernel() and the FP32 store */
static int grid_find_new(orc_ctx* c) {
  double xmin[2], xmax[2], deltx[2];
  int ndivx[2];
  int scale_k = (c->p.skf == 1) ? 2 : 3;
  for (int d = 0; d < 2; d++) {
    xmin[d] = (double)1.e10f;
    xmax[d] = -xmin[d];
    deltx[d] = 0.0;
  }
  for (int d = 0; d < 2; d++) {
    for (int i = 0; i < c->N2; i++) {
      if (c->out_domain[i] == 1) continue;
      if (X(c, d, i) < xmin[d]) xmin[d] = X(c, d, i);
      if (X(c, d, i) > xmax[d]) xmax[d] = X(c, d, i);
      if (deltx[d] < c->hsml[i]) deltx[d] = c->hsml[i];
    }
    deltx[d] = deltx[d] * 2.0;
    double length = xmax[d] - xmin[d];
    ndivx[d] = (int)(length / deltx[d] + 1.0);
    double length_new = (double)ndivx[d] * deltx[d];
    xmin[d] = (xmin[d] - (length_new - length) / 2.0) - (double)0.001f * length;
    xmax[d] = (xmax[d] + (length_new - length) / 2.0) + (double)0.001f * length;
  }
  int64_t ndivt = (int64_t)ndivx[0] * ndivx[1];
  if (ndivt > c->cell_cap) {
    free(c->cell_cnt);
    free(c->cell_start);
    c->cell_cnt = xcalloc(ndivt, sizeof(int32_t));
    c->cell_start = xcalloc(ndivt, sizeof(int32_t));
    if (!c->cell_cnt || !c->cell_start) return -1;
    c->cell_cap = ndivt;
  }
  memset(c->cell_cnt, 0, ndivt * sizeof(int32_t));
  for (int i = 0; i < c->N2; i++) {
    c->which_cell[i] = -1;
    if (c->out_domain[i] == 1) continue;
    int idv[2];
    for (int d = 0; d < 2; d++) {
      idv[d] = (int)((X(c, d, i) - xmin[d]) / deltx[d] + 1.0);
      if (idv[d] > ndivx[d]) idv[d] = ndivx[d];
    }
    int64_t idivt = (int64_t)ndivx[0] * (idv[1] - 1) + idv[0]; /* 1-based */
    c->which_cell[i] = (int32_t)(idivt - 1);
    c->cell_cnt[idivt - 1]++;
  }
  int32_t pos = 0;
  for (int64_t t = 0; t < ndivt; t++) {
    c->cell_start[t] = pos;
    pos += c->cell_cnt[t];
  }
  {
    /* fill in ascending particle id within each cell (:1297-1305) */
    int32_t* cur = xcalloc(ndivt, sizeof(int32_t));
    if (!cur) return -1;
    for (int i = 0; i < c->N2; i++) {
      int32_t t = c->which_cell[i];
      if (t < 0) continue;
      c->cell_list[c->cell_start[t] + cur[t]++] = i;
    }
    free(cur);
  }
  c->npairs = 0;
  for (int idy = 1; idy <= ndivx[1]; idy++)
    for (int idx = 1; idx <= ndivx[0]; idx++) {
      int64_t idivt = (int64_t)ndivx[0] * (idy - 1) + idx;
      int npicsi = c->cell_cnt[idivt - 1];
      for (int ii = 1; ii <= npicsi; ii++) {
        int it = c->cell_list[c->cell_start[idivt - 1] + ii - 1];
        int idx0 = idx - 1 > 1 ? idx - 1 : 1;
        int idx1 = idx + 1 < ndivx[0] ? idx + 1 : ndivx[0];
        int idy1 = idy + 1 < ndivx[1] ? idy + 1 : ndivx[1];
        for (int jdy = idy; jdy <= idy1; jdy++)
          for (int jdx = idx0; jdx <= idx1; jdx++) {
            int64_t jdivt = (int64_t)ndivx[0] * (jdy - 1) + jdx;
            if (jdivt < idivt) continue;
            int jj = (idivt == jdivt) ? ii + 1 : 1;
            int npicsj = c->cell_cnt[jdivt - 1];
            for (int j = jj; j <= npicsj; j++) {
              int jt = c->cell_list[c->cell_start[jdivt - 1] + j - 1];
              double dxiac[2];
              dxiac[0] = X(c, 0, it) - X(c, 0, jt);
              double driac = dxiac[0] * dxiac[0];
              dxiac[1] = X(c, 1, it) - X(c, 1, jt);
              driac = driac + dxiac[1] * dxiac[1];
              double mhsml = (c->hsml[it] + c->hsml[jt]) / 2.0;
              double r = sqrt(driac);
              if (r < (double)scale_k * mhsml) {
                if (ensure_pair_cap(c, c->npairs + 1)) return -1;
                double w, dw[2];
                orc_kernel(c->p.skf, c->p.pi, r, dxiac, mhsml, &w, dw);
                int64_t k = c->npairs++;
                c->pi[k] = it;
                c->pj[k] = jt;
                c->ptype[k] = 0;
                c->pw[k] = (float)w;
                c->pdx[k] = (float)dw[0];
                c->pdy[k] = (float)dw[1];
              }
            }
          }
      }
    }
  build_walk_order(c);
  return 0;
}

/* Pint_Update (3_SPH_material_2018.f90:1574-1634): orientation and pair type */
static void pint_update(orc_ctx* c) {
  for (int64_t k = 0; k < c->npairs; k++) {
    int i = c->pi[k], j = c->pj[k];
    int ti = c->itype[i], tj = c->itype[j];
    int ii = abs(ti), jj = abs(tj), isumm = ti + tj;
    if ((ii == 2 && jj == 1) || (ii == 2 && jj == 25) || (ii == 1 && jj == 25)) {
      c->pi[k] = j;
      c->pj[k] = i;
      c->pdx[k] = -c->pdx[k];
      c->pdy[k] = -c->pdy[k];
    }
    int t = 0;
    if (isumm == 3) t = 1;
    else if (isumm == 2) t = 2;
    else if (isumm == 4) t = 3;
    else if (isumm == 27) t = 6;
    else if (isumm == 26) t = 9;
    c->ptype[k] = t;
  }
}

/* stress_point_update (2_SPH_main_2018.f90:403-482) */
static void stress_point_update(orc_ctx* c) {
  const int NN = c->NN, NT = c->NT;
  if (!c->p.sp_sph) {
    for (int i = 0; i < NN; i++) {
      for (int d = 0; d < 2; d++) V(c, d, NN + i) = V(c, d, i);
      for (int k = 0; k < 4; k++) S(c, k, i) = S(c, k, NN + i);
      c->intvars1[i] = c->intvars1[NN + i];
      if (c->p.cont_density) c->rho[i] = c->rho[NN + i];
    }
    return;
  }
  double* vel_t = xcalloc(2 * (size_t)NT, sizeof(double));
  double* st_t = xcalloc(4 * (size_t)NT, sizeof(double));
  double* iv_t = xcalloc(NT, sizeof(double));
  double* rho_t = xcalloc(NT, sizeof(double));
  double* norm = xcalloc(NT, sizeof(double));
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    if (c->ptype[q] != 1) continue;
    int j = c->pi[q]; /* stress point */
    int i = c->pj[q]; /* node */
    double w = (double)c->pw[q];
    double h1 = (c->mass[j] / c->rho[j]) * w;
    double h2 = (c->mass[i] / c->rho[i]) * w;
    for (int d = 0; d < 2; d++) vel_t[d + 2 * (size_t)j] = vel_t[d + 2 * (size_t)j] + V(c, d, i) * h2;
    for (int s = 0; s < 4; s++)
      st_t[s + 4 * (size_t)i] = st_t[s + 4 * (size_t)i] + S(c, s, j) * h1;
    iv_t[i] = iv_t[i] + c->intvars1[j] * h1;
    if (c->p.cont_density) rho_t[i] = rho_t[i] + c->rho[j] * h1;
    norm[j] = norm[j] + (w * c->mass[i]) / c->rho[i];
    norm[i] = norm[i] + (w * c->mass[j]) / c->rho[j];
  }
  for (int i = NN; i < NT; i++) {
    if (norm[i] == 0) continue;
    V(c, 0, i) = vel_t[0 + 2 * (size_t)i] / norm[i];
    V(c, 1, i) = vel_t[1 + 2 * (size_t)i] / norm[i];
  }
  for (int i = 0; i < NN; i++) {
    if (norm[i] != 0) {
      for (int s = 0; s < 4; s++) S(c, s, i) = st_t[s + 4 * (size_t)i] / norm[i];
      c->intvars1[i] = iv_t[i] / norm[i];
    } else {
      V(c, 0, i) = 0.0;
      V(c, 1, i) = 0.0;
    }
  }
  if (c->p.cont_density)
    for (int i = 0; i < NN; i++) c->rho[i] = rho_t[i] / norm[i];
  free(vel_t);
  free(st_t);
  free(iv_t);
  free(rho_t);
  free(norm);
}

/* get_derivatives (2_SPH_main_2018.f90:487-648); div1(4,NT), div2(2,NT) */
static void get_derivatives(orc_ctx* c, double* div1, double* div2) {
  const int NN = c->NN, NT = c->NT;
  double* g1 = xcalloc(4 * (size_t)NT, sizeof(double)); /* grad1(a,b,i) -> a + 2b + 4i */
  double* g2 = xcalloc(6 * (size_t)NT, sizeof(double)); /* grad2(s,b,i) -> s + 3b + 6i */
  double* AE = xcalloc(5 * (size_t)NT, sizeof(double));
  memset(div1, 0, 4 * (size_t)NT * sizeof(double));
  memset(div2, 0, 2 * (size_t)NT * sizeof(double));
  for (int i = 0; i < NN; i++) c->bc_int[i] = 0;
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    int j = c->pi[q];
    int i = c->pj[q];
    double dwx = (double)c->pdx[q], dwy = (double)c->pdy[q];
    double h1 = (dwx * c->mass[i]) / c->rho[i];
    int t = c->ptype[q];
    if (t == 1) {
      double h2 = 0.0;
      for (int d = 0; d < 2; d++) {
        g1[d + 0 + 4 * (size_t)j] = g1[d + 0 + 4 * (size_t)j] + (V(c, d, i) - V(c, d, j)) * h1;
        h2 = (dwy * c->mass[i]) / c->rho[i];
        g1[d + 2 + 4 * (size_t)j] = g1[d + 2 + 4 * (size_t)j] + (V(c, d, i) - V(c, d, j)) * h2;
      }
      for (int s = 0; s < 3; s++) {
        double ai = S(c, s, i) / (c->rho[i] * c->rho[i]);
        double aj = S(c, s, j) / (c->rho[j] * c->rho[j]);
        double gg1 = dwx * (ai + aj);
        g2[s + 0 + 6 * (size_t)i] = g2[s + 0 + 6 * (size_t)i] - c->mass[j] * gg1;
        double gg2 = dwy * (ai + aj);
        g2[s + 3 + 6 * (size_t)i] = g2[s + 3 + 6 * (size_t)i] - c->mass[j] * gg2;
      }
      if (c->p.cspm) {
        double h1b = -((dwx * c->mass[j]) / c->rho[j]);
        double h2b = -((dwy * c->mass[j]) / c->rho[j]);
        double* Aj = &AE[5 * (size_t)j];
        double* Ai = &AE[5 * (size_t)i];
        Aj[0] = Aj[0] + (X(c, 0, i) - X(c, 0, j)) * h1;
        Aj[1] = Aj[1] + (X(c, 1, i) - X(c, 1, j)) * h1;
        Aj[2] = Aj[2] + (X(c, 0, i) - X(c, 0, j)) * h2;
        Aj[3] = Aj[3] + (X(c, 1, i) - X(c, 1, j)) * h2;
        Ai[0] = Ai[0] + (X(c, 0, j) - X(c, 0, i)) * h1b;
        Ai[1] = Ai[1] + (X(c, 1, j) - X(c, 1, i)) * h1b;
        Ai[2] = Ai[2] + (X(c, 0, j) - X(c, 0, i)) * h2b;
        Ai[3] = Ai[3] + (X(c, 1, j) - X(c, 1, i)) * h2b;
      }
    } else if (t == 9) {
      /* i is the stress point, j the dummy */
      const double beta_max = 1.5, vel_wall = 0.0;
      double wall = (double)c->wall_position[j];
      double da, db;
      if (c->horizontal_or_not[j] == 1.0f) {
        da = fabs(X(c, 1, i) - wall);
        db = fabs(X(c, 1, j) - wall);
      } else {
        da = fabs(X(c, 0, i) - wall);
        db = fabs(X(c, 0, j) - wall);
      }
      double bq = 1.0 + db / da;
      double beta = beta_max < bq ? beta_max : bq;
      double dv[2];
      for (int d = 0; d < 2; d++) dv[d] = V(c, d, i) * (1.0 - beta) + beta * vel_wall;
      double hh1 = (dwx * c->mass[j]) / c->rho[j];
      for (int d = 0; d < 2; d++) {
        g1[d + 0 + 4 * (size_t)i] = g1[d + 0 + 4 * (size_t)i] + (V(c, d, i) - dv[d]) * hh1;
        double hh2 = (dwy * c->mass[j]) / c->rho[j];
        g1[d + 2 + 4 * (size_t)i] = g1[d + 2 + 4 * (size_t)i] + (V(c, d, i) - dv[d]) * hh2;
      }
    } else if (t == 6) {
      /* i is the node, j the dummy: stress(:,j) = stress(:,i) (pair-local) */
      c->bc_int[i] = 1;
      for (int s = 0; s < 4; s++) S(c, s, j) = S(c, s, i);
      for (int s = 0; s < 3; s++) {
        double ai = S(c, s, i) / (c->rho[i] * c->rho[i]);
        double aj = S(c, s, j) / (c->rho[j] * c->rho[j]);
        double hh1 = dwx * (ai + aj);
        g2[s + 0 + 6 * (size_t)i] = g2[s + 0 + 6 * (size_t)i] - c->mass[j] * hh1;
        double hh2 = dwy * (ai + aj);
        g2[s + 3 + 6 * (size_t)i] = g2[s + 3 + 6 * (size_t)i] - c->mass[j] * hh2;
      }
    }
  }
  if (c->p.cspm) {
    for (int i = 0; i < NT; i++) {
      double* A = &AE[5 * (size_t)i];
      A[4] = A[0] * A[3] - A[1] * A[2];
      /* the copy's threshold: (double)1e-07f (2_SPH_main_2018.f90:599 of the
         Drucker-Prager example) or (double)1e-03f (code/ and the other copies) */
      if (fabs(A[4]) < c->p.cspm_det_min) {
        A[4] = 1;
        A[0] = 1;
        A[1] = 0;
        A[2] = 0;
        A[3] = 1;
      } else {
        A[4] = 1.0 / A[4];
      }
    }
    for (int d = 0; d < 2; d++) {
      for (int i = NN; i < NT; i++) {
        double* A = &AE[5 * (size_t)i];
        double* g = &g1[4 * (size_t)i];
        g[d + 0] = A[4] * (A[0] * g[d + 0] + A[1] * g[d + 2]);
      }
      for (int i = NN; i < NT; i++) {
        double* A = &AE[5 * (size_t)i];
        double* g = &g1[4 * (size_t)i];
        g[d + 2] = A[4] * (A[2] * g[d + 0] + A[3] * g[d + 2]);
      }
      for (int i = 0; i < NN; i++) {
        double* A = &AE[5 * (size_t)i];
        double* g = &g2[6 * (size_t)i];
        g[d + 0] = A[4] * (A[0] * g[d + 0] + A[1] * g[d + 3]);
      }
      for (int i = 0; i < NN; i++) {
        double* A = &AE[5 * (size_t)i];
        double* g = &g2[6 * (size_t)i];
        g[d + 3] = A[4] * (A[2] * g[d + 0] + A[3] * g[d + 3]);
      }
    }
  }
  const double D11 = c->p.D11, D12 = c->p.D12, D22 = c->p.D22, D33 = c->p.D33, D41 = c->p.D41,
               D42 = c->p.D42;
  for (int i = NN; i < NT; i++) {
    double* g = &g1[4 * (size_t)i];
    double g11 = g[0], g21 = g[1], g12 = g[2], g22 = g[3];
    div1[0 + 4 * (size_t)i] = -(D11 * g11 + D12 * g22);
    div1[1 + 4 * (size_t)i] = -(D12 * g11 + D22 * g22);
    div1[2 + 4 * (size_t)i] = -(D33 * g21 + D33 * g12);
    div1[3 + 4 * (size_t)i] = -(D41 * g11 + D42 * g22);
  }
  for (int i = 0; i < NN; i++) {
    double* g = &g2[6 * (size_t)i];
    div2[0 + 2 * (size_t)i] = -(g[0] + g[2 + 3]);
    div2[1 + 2 * (size_t)i] = -(g[2] + g[1 + 3]);
  }
  memcpy(c->grad_u, g1, 4 * (size_t)NT * sizeof(double));
  free(g1);
  free(g2);
  free(AE);
}

/* time-curve factor used by gravity_force (3_SPH_material_2018.f90:2830-2848) and the
   time-curve BC branch of Normal_BCs (:1707-1722) */
static double tcurve_value(const orc_ctx* c, int it, double t) {
  int nc = c->p.ntcurves;
  int npts = c->nptstcurves[it - 1];
  double tt0 = 0, tt1 = 0;
  int ip;
  for (ip = 1; ip <= npts - 1; ip++) {
    tt0 = c->ttcurves[(it - 1) + (size_t)(ip - 1) * nc];
    tt1 = c->ttcurves[(it - 1) + (size_t)ip * nc];
    if (t >= tt0 && t <= tt1) break;
    tt0 = -1000.0;
  }
  if (tt0 >= 0.0) {
    double xi = (t - tt0) / (tt1 - tt0);
    return (1.0 - xi) * (double)c->ftcurves[(it - 1) + (size_t)(ip - 1) * nc] +
           xi * (double)c->ftcurves[(it - 1) + (size_t)ip * nc];
  }
  return 0.0;
}

/* gravity_force (3_SPH_material_2018.f90:2809-2871) over the nodes */
static void gravity_force(const orc_ctx* c, double* Gs /* (2,NN) */) {
  double factg = 0.0;
  for (size_t k = 0; k < 2 * (size_t)c->NN; k++) Gs[k] = 0.0;
  if (c->p.ic_grav != 0) {
    factg = tcurve_value(c, c->p.tcurve_grav, c->time_sph);
    factg = factg * c->p.ft_grav;
    if (c->p.ic_grav == 1)
      for (int i = 0; i < c->NN; i++)
        for (int d = 0; d < 2; d++) Gs[d + 2 * (size_t)i] = factg * c->p.cgrav[d];
  }
  for (int i = 0; i < c->NN; i++)
    for (int d = 0; d < 2; d++)
      Gs[d + 2 * (size_t)i] = Gs[d + 2 * (size_t)i] - c->p.damping * V(c, d, i);
}

/* boundary_forces, test == 2 branch (2_SPH_main_2018.f90:1117-1161): FP32 locals */
static void boundary_forces(orc_ctx* c) {
  const int NN = c->NN;
  for (size_t k = 0; k < 2 * (size_t)NN; k++) c->f_bound[k] = 0.0;
  const float cc = 20.0f;
  const float d0 = (float)(c->p.dx / 2.0);
  for (int j = c->NT; j < c->NT + c->p.ndummy2; j++) {
    for (int i = 0; i < NN; i++) {
      float r[2];
      r[0] = (float)(X(c, 0, i) - X(c, 0, j));
      r[1] = (float)(X(c, 1, i) - X(c, 1, j));
      float r2 = sqrtf(r[0] * r[0] + r[1] * r[1]);
      float f2;
      float h = (float)(0.5 * (c->hsml[i] + c->hsml[j]));
      float r_bound = r2 / (0.75f * h);
      if (r2 > 0 && r2 < 1.5f * d0) f2 = 1.0f - (r2 / (1.5f * d0));
      else f2 = 0.0f;
      float f;
      if (0 < r_bound && r_bound <= 2.0f / 3.0f) f = 2.0f / 3.0f;
      else if (2.0f / 3.0f < r_bound && r_bound <= 1) f = 2.0f * r_bound - 1.5f * (r_bound * r_bound);
      else if (1 < r_bound && r_bound < 2) f = 0.5f * ((2.0f - r_bound) * (2.0f - r_bound));
      else f = 0.0f;
      for (int d = 0; d < 2; d++)
        c->f_bound[d + 2 * (size_t)i] =
            c->f_bound[d + 2 * (size_t)i] +
            (double)((((0.01f * (cc * cc)) * f2) * f) * (r[d] / (r2 * r2)));
    }
  }
}

/* artificial_force (2_SPH_main_2018.f90:908-1016): Monaghan's artificial stress over the
   node-node pairs in walk order.  Per particle, the principal stresses of the in-plane
   stress (angle 0.5 atan(2 s12 / (s11 - s22)), 0 unless s11 - s22 >= 1e-8), their tensile
   parts scaled by -eps / rho^2, and the reference's rotation back (whose second component
   is R2(1) (cos^2 + sin^2)); per pair, f = W / W(dx, h0) with h0 = 1.2 dx and the power
   n = 2.55.  eps, n, 1.2 and 1e-8 are FP32 literals. */
static void art_R(const orc_ctx* c, int i, double* R) {
  const double eps = (double)0.1f;
  const double s12 = S(c, 0, i) - S(c, 1, i);
  double th = 0.0;
  if (s12 >= (double)1e-08f) th = 0.5 * atan((2.0 * S(c, 2, i)) / s12);
  const double co = cos(th), si = sin(th), cc = co * co, ss = si * si;
  const double cs2 = (2.0 * co) * si;
  double sig[2], R2[2];
  sig[0] = (cc * S(c, 0, i) + cs2 * S(c, 2, i)) + ss * S(c, 1, i);
  sig[1] = (ss * S(c, 0, i) - cs2 * S(c, 2, i)) + cc * S(c, 1, i);
  for (int k = 0; k < 2; k++)
    R2[k] = sig[k] > 0 ? -(eps * (sig[k] / (c->rho[i] * c->rho[i]))) : 0.0;
  R[0] = R2[0] * cc + R2[1] * ss;
  R[1] = R2[0] * (cc + ss);
  R[2] = (R2[0] - R2[1]) * (co * si);
}

static void artificial_force(orc_ctx* c) {
  const int NN = c->NN;
  const double n = (double)2.55f;
  const double hsml0 = (double)1.2f * c->p.dx;
  const double dx2[2] = {c->p.dx, c->p.dy};
  double w2, g2[2];
  orc_kernel(c->p.skf, c->p.pi, c->p.dx, dx2, hsml0, &w2, g2);
  double* tmp = xcalloc(6 * (size_t)NN, sizeof(double)); /* (istre, d, i) */
#define T(k, d, i) tmp[(k) + 3 * ((d) + 2 * (size_t)(i))]
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    if (c->ptype[q] != 3) continue;
    const int i = c->pi[q], j = c->pj[q];
    double Ri[3], Rj[3];
    art_R(c, i, Ri);
    art_R(c, j, Rj);
    const double fn = pow((double)c->pw[q] / w2, n);
    for (int st = 0; st < 3; st++) {
      const double h1 = ((double)c->pdx[q] * fn) * (Ri[st] + Rj[st]);
      T(st, 0, i) = T(st, 0, i) + c->mass[j] * h1;
      T(st, 0, j) = T(st, 0, j) - c->mass[i] * h1;
      const double h2 = ((double)c->pdy[q] * fn) * (Ri[st] + Rj[st]);
      T(st, 1, i) = T(st, 1, i) + c->mass[j] * h2;
      T(st, 1, j) = T(st, 1, j) - c->mass[i] * h2;
    }
  }
  for (int i = 0; i < NN; i++) {
    c->art_force[0 + 2 * (size_t)i] = T(0, 0, i) + T(2, 1, i);
    c->art_force[1 + 2 * (size_t)i] = T(2, 0, i) + T(1, 1, i);
  }
#undef T
  free(tmp);
}

void orc_artificial_force(orc_ctx* c, double* out) {
  artificial_force(c);
  memcpy(out, c->art_force, sizeof(double) * 2 * (size_t)c->NN);
}

/* artificial_viscosity (2_SPH_main_2018.f90:826-904): FP32 accumulators */
static void artificial_viscosity(orc_ctx* c) {
  const int NN = c->NN;
  float* avt = xcalloc(2 * (size_t)NN, sizeof(float));
  float visc = 0.0f;
  const float cs = 600.0f;
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    if (c->ptype[q] != 3) continue;
    int i = c->pi[q], j = c->pj[q];
    float xij = (float)(X(c, 0, i) - X(c, 0, j));
    float yij = (float)(X(c, 1, i) - X(c, 1, j));
    float h = (float)(0.5 * (c->hsml[i] + c->hsml[j]));
    float rho2 = (float)(0.5 * (c->rho[i] + c->rho[j]));
    float div_u = (float)((double)xij * (V(c, 0, i) - V(c, 0, j)));
    div_u = (float)((double)div_u + (double)yij * (V(c, 1, i) - V(c, 1, j)));
    float sq = sqrtf(xij * xij + yij * yij);
    float theta = (h * div_u) / (sq * sq + 0.01f * (h * h));
    if (div_u < 0)
      visc = (float)((-((c->p.alpha * (double)cs) * (double)theta) +
                      c->p.beta * (double)(theta * theta)) /
                     (double)rho2);
    else if (div_u >= 0)
      visc = 0.0f;
    float px = visc * c->pdx[q], py = visc * c->pdy[q];
    avt[0 + 2 * (size_t)i] = (float)((double)avt[0 + 2 * (size_t)i] + (double)px * c->mass[j]);
    avt[0 + 2 * (size_t)j] = (float)((double)avt[0 + 2 * (size_t)j] - (double)px * c->mass[i]);
    avt[1 + 2 * (size_t)i] = (float)((double)avt[1 + 2 * (size_t)i] + (double)py * c->mass[j]);
    avt[1 + 2 * (size_t)j] = (float)((double)avt[1 + 2 * (size_t)j] - (double)py * c->mass[i]);
  }
  for (size_t k = 0; k < 2 * (size_t)NN; k++) c->art_visc[k] = -(double)avt[k];
  free(avt);
}

/* Normal_BCs (3_SPH_material_2018.f90:1665-1770); ic_time is an uninitialised local in the
   reference and is taken as 0, so t_actual = time_sph.  The loop runs over 1..ntotal
   (:1683) or, with bc_nodes_only, over the nodes 1..nnode as in code/ and the
   strain-localisation copy (code/3_SPH_material_2018.f90:1664). */
static void normal_bcs(orc_ctx* c) {
  if (c->p.no_bcs <= 0) return;
  double t = c->time_sph;
  const int nloop = c->p.bc_nodes_only ? c->NN : c->NT;
  for (int ip = 0; ip < nloop; ip++) {
    int nber = c->bc_info[1 + 8 * (size_t)ip];
    if (c->bc_or_not[ip] != 1) continue;
    if (nber == 0) continue;
    for (int r = 0; r < 5; r++) {
      int bt = c->bc_info[r + 2 + 8 * (size_t)ip];
      if (bt == 0) continue;
      const double* b = &c->bc_list[8 * (size_t)(bt - 1)];
      int itc = (int)b[2];
      double val = 0.0;
      if (itc == 0) {
        double a0 = b[4], a1 = b[3], w = b[5], phi = b[6], tt = b[7];
        double fact = 1.0 - exp(-t / tt);
        double argum = w * t - phi;
        val = (a0 + a1 * sin(argum)) * fact;
      } else if (itc > 0) {
        val = tcurve_value(c, itc, t) * b[3];
      }
      int var = (int)b[1];
      if (var == 5) V(c, 0, ip) = val;
      else if (var == 6) V(c, 1, ip) = val;
      else if (var == 1) S(c, 0, ip) = val;
      else if (var == 3) S(c, 2, ip) = val;
      else if (var == 2) S(c, 1, ip) = val;
    }
  }
}

/* BCs (3_SPH_material_2018.f90:1640-1660) */
static void apply_stress_free(orc_ctx* c);
static void bcs(orc_ctx* c) {
  normal_bcs(c);
  if (c->p.ifsigman == 1) apply_stress_free(c);
}

static void adapt_all(orc_ctx* c) {
  double a2, kc;
  dp_constants(c->p.props[12], c->p.props[13], &a2, &kc);
  for (int i = 0; i < c->NT; i++) adapt_one(a2, kc, &c->stress[4 * (size_t)i]);
}

/* RK4 (2_SPH_main_2018.f90:653-802) */
static void rk4(orc_ctx* c) {
  const int NN = c->NN, NT = c->NT;
  const double f1rk[4] = {0.0, 0.5, 0.5, 1.0}, f2rk[4] = {1.0, 2.0, 2.0, 1.0};
  const int ncrit = (int)c->p.props[1];
  const double dt = c->p.dt_sph;
  size_t n2 = 2 * (size_t)NT, n4 = 4 * (size_t)NT;
  double* vel0 = xcalloc(n2, sizeof(double));
  double* st0 = xcalloc(n4, sizeof(double));
  double* rho0 = xcalloc(NT, sizeof(double));
  double* hsml0 = xcalloc(NT, sizeof(double));
  double* RKv = xcalloc(n2, sizeof(double));
  double* RKs = xcalloc(n4, sizeof(double));
  double* RKr = xcalloc(NT, sizeof(double));
  double* RKh = xcalloc(NT, sizeof(double));
  double* RKd = xcalloc(NT, sizeof(double));
  double* RHS1 = xcalloc(n4, sizeof(double));
  double* RHS2 = xcalloc(n2, sizeof(double));
  double* RHSr = xcalloc(NT, sizeof(double));
  double* RHSh = xcalloc(NT, sizeof(double));
  double* div1 = xcalloc(n4, sizeof(double));
  double* div2 = xcalloc(n2, sizeof(double));
  double* src = xcalloc(n4, sizeof(double));
  double* spin = xcalloc(n4, sizeof(double));
  double* grav = xcalloc(2 * (size_t)NN, sizeof(double));
  memcpy(vel0, c->vel, n2 * sizeof(double));
  memcpy(st0, c->stress, n4 * sizeof(double));
  memcpy(rho0, c->rho, NT * sizeof(double));
  memcpy(hsml0, c->hsml, NT * sizeof(double));
  for (size_t k = 0; k < 2 * (size_t)NN; k++) c->art_visc[k] = 0.0;
  memset(c->vel, 0, 2 * (size_t)c->N2 * sizeof(double));
  memset(c->stress, 0, 4 * (size_t)c->N2 * sizeof(double));
  for (int st = 0; st < 4; st++) {
    for (int i = 0; i < NN; i++)
      for (int d = 0; d < 2; d++)
        V(c, d, i) = vel0[d + 2 * (size_t)i] + (f1rk[st] * dt) * RHS2[d + 2 * (size_t)i];
    for (int i = NN; i < NT; i++)
      for (int s = 0; s < 4; s++)
        S(c, s, i) = st0[s + 4 * (size_t)i] + (f1rk[st] * dt) * RHS1[s + 4 * (size_t)i];
    if (c->p.cont_density) {
      for (int i = NN; i < NT; i++)
        RHSr[i] = -c->rho[i] * (c->grad_u[0 + 4 * (size_t)i] + c->grad_u[3 + 4 * (size_t)i]);
      for (int i = NN; i < NT; i++) c->rho[i] = rho0[i] + (f1rk[st] * dt) * RHSr[i];
      if (c->p.sle == 2) {
        for (int i = NN; i < NT; i++) RHSh[i] = -(hsml0[i] / (c->rho[i] * 2.0)) * RHSr[i];
        for (int i = NN; i < NT; i++) c->hsml[i] = hsml0[i] + (f1rk[st] * dt) * RHSh[i];
      }
    }
    if (ncrit == 12) adapt_all(c);
    if (c->p.no_bcs > 0) bcs(c);
    stress_point_update(c);
    if (c->p.sp_sph) {
      if (ncrit == 12) adapt_all(c);
      if (c->p.no_bcs > 0) bcs(c);
    }
    get_derivatives(c, div1, div2);
    for (int j = NN; j < NT; j++) {
      double G[4], der1;
      plastic_terms(c, j, &c->stress[4 * (size_t)j], G, &der1);
      for (int s = 0; s < 4; s++) src[s + 4 * (size_t)j] = G[s];
      RKd[j] = RKd[j] + der1 * f2rk[st];
    }
    gravity_force(c, grav);
    if (c->p.inside_approach) boundary_forces(c);
    if (c->p.alpha > 0 || c->p.beta > 0) artificial_viscosity(c);
    if (c->p.art_stress) artificial_force(c);
    if (c->p.update_x) {
      for (int i = NN; i < NT; i++) {
        const double* g = &c->grad_u[4 * (size_t)i];
        double om1 = 0.5 * (g[2] - g[1]);
        double om2 = -0.5 * (g[2] - g[1]);
        spin[0 + 4 * (size_t)i] = 2.0 * om1 * S(c, 2, i);
        spin[1 + 4 * (size_t)i] = 2.0 * om2 * S(c, 2, i);
        spin[2 + 4 * (size_t)i] = om2 * S(c, 0, i) + om1 * S(c, 1, i);
      }
    }
    for (int i = NN; i < NT; i++)
      for (int s = 0; s < 4; s++) {
        size_t o = s + 4 * (size_t)i;
        RHS1[o] = (-div1[o] + spin[o]) + src[o];
      }
    for (int i = 0; i < NN; i++)
      for (int d = 0; d < 2; d++) {
        size_t o = d + 2 * (size_t)i;
        RHS2[o] = (((-div2[o] + grav[o]) + c->art_visc[o]) + c->f_bound[o]) + c->art_force[o];
      }
    for (int i = 0; i < NN; i++)
      for (int d = 0; d < 2; d++) RKv[d + 2 * (size_t)i] += f2rk[st] * RHS2[d + 2 * (size_t)i];
    for (int i = NN; i < NT; i++)
      for (int s = 0; s < 4; s++) RKs[s + 4 * (size_t)i] += f2rk[st] * RHS1[s + 4 * (size_t)i];
    if (c->p.cont_density) {
      for (int i = 0; i < NT; i++) RKr[i] = RKr[i] + f2rk[st] * RHSr[i];
      if (c->p.sle == 2)
        for (int i = 0; i < NT; i++) RKh[i] = RKh[i] + f2rk[st] * RHSh[i];
    }
  }
  for (int i = 0; i < NN; i++)
    for (int d = 0; d < 2; d++)
      V(c, d, i) = vel0[d + 2 * (size_t)i] + (dt / 6.0) * RKv[d + 2 * (size_t)i];
  for (int i = NN; i < NT; i++)
    for (int s = 0; s < 4; s++)
      S(c, s, i) = st0[s + 4 * (size_t)i] + (dt / 6.0) * RKs[s + 4 * (size_t)i];
  if (ncrit == 12) adapt_all(c);
  if (c->p.no_bcs > 0) bcs(c);
  if (c->p.cont_density) {
    for (int i = NN; i < NT; i++) c->rho[i] = rho0[i] + (dt / 6.0) * RKr[i];
    if (c->p.sle == 2)
      for (int i = NN; i < NT; i++) c->hsml[i] = hsml0[i] + (dt / 6.0) * RKh[i];
  }
  for (int i = 0; i < NT; i++) c->Ddev[i] = RKd[i] / 6.0;
  free(vel0);
  free(st0);
  free(rho0);
  free(hsml0);
  free(RKv);
  free(RKs);
  free(RKr);
  free(RKh);
  free(RKd);
  free(RHS1);
  free(RHS2);
  free(RHSr);
  free(RHSh);
  free(div1);
  free(div2);
  free(src);
  free(spin);
  free(grav);
}

/* get_nodes_on_free_surface (3_SPH_material_2018.f90:1135-1430).  Its locals are `real`
   (FP32); the module arrays normal and subset are FP64.  An FP32 accumulation with an FP64
   operand is evaluated in FP64 and rounded once, as Fortran's mixed-kind expressions are.
   `x**0.5` is taken as the square root. */
static void free_surface(orc_ctx* c) {
  const int NT = c->NT;
  float* A = xcalloc(4 * (size_t)NT, sizeof(float));
  float* ff = xcalloc(2 * (size_t)NT, sizeof(float));
  float* f_int = xcalloc((size_t)NT, sizeof(float));
  float* gf = xcalloc(2 * (size_t)NT, sizeof(float));
  float* nb = xcalloc((size_t)NT, sizeof(float));
  float* tt = xcalloc(2 * (size_t)NT, sizeof(float));
  float* tau = xcalloc(2 * (size_t)NT, sizeof(float));
  double* nrm = c->normal;
  for (int i = 0; i < NT; i++) c->subset[i] = 0.0;
  /* step 1: renormalisation matrix and kernel-gradient sums over types 1, 2, 3 */
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    int t = c->ptype[q];
    if (t != 1 && t != 2 && t != 3) continue;
    int i = c->pi[q], j = c->pj[q];
    float gx = c->pdx[q], gy = c->pdy[q];
    float hf1i = (float)(c->mass[j] * (double)gx / c->rho[j]);
    float hf1j = (float)(-(c->mass[i] * (double)gx / c->rho[i]));
    float hf2i = (float)(c->mass[j] * (double)gy / c->rho[j]);
    float hf2j = (float)(-(c->mass[i] * (double)gy / c->rho[i]));
    double dxij = X(c, 0, j) - X(c, 0, i), dyij = X(c, 1, j) - X(c, 1, i);
    double dxji = X(c, 0, i) - X(c, 0, j), dyji = X(c, 1, i) - X(c, 1, j);
    A[0 + 4 * (size_t)i] = (float)((double)A[0 + 4 * (size_t)i] + dxij * (double)hf1i);
    A[0 + 4 * (size_t)j] = (float)((double)A[0 + 4 * (size_t)j] + dxji * (double)hf1j);
    ff[0 + 2 * (size_t)i] = ff[0 + 2 * (size_t)i] + hf1i;
    ff[0 + 2 * (size_t)j] = ff[0 + 2 * (size_t)j] + hf1j;
    A[1 + 4 * (size_t)i] = (float)((double)A[1 + 4 * (size_t)i] + dyij * (double)hf1i);
    A[2 + 4 * (size_t)i] = (float)((double)A[2 + 4 * (size_t)i] + dxij * (double)hf2i);
    A[3 + 4 * (size_t)i] = (float)((double)A[3 + 4 * (size_t)i] + dyij * (double)hf2i);
    A[1 + 4 * (size_t)j] = (float)((double)A[1 + 4 * (size_t)j] + dyji * (double)hf1j);
    A[2 + 4 * (size_t)j] = (float)((double)A[2 + 4 * (size_t)j] + dxji * (double)hf2j);
    A[3 + 4 * (size_t)j] = (float)((double)A[3 + 4 * (size_t)j] + dyji * (double)hf2j);
    ff[1 + 2 * (size_t)i] = ff[1 + 2 * (size_t)i] + hf2i;
    ff[1 + 2 * (size_t)j] = ff[1 + 2 * (size_t)j] + hf2j;
  }
  /* step 2: first normal estimate; step 3 set-up: scan point and tangent */
  for (int i = 0; i < NT; i++) {
    float* a = &A[4 * (size_t)i];
    for (int r = 0; r < 4; r++)
      if (fabsf(a[r]) <= 1.e-8f) a[r] = 0.0f;
    float f0 = ff[2 * (size_t)i], f1 = ff[2 * (size_t)i + 1];
    float v0 = -(a[0] * f0 + a[1] * f1);
    float v1 = -(a[2] * f0 + a[3] * f1);
    float v2 = sqrtf(v0 * v0 + v1 * v1);
    nrm[2 * (size_t)i] = (double)(v0 / v2);
    nrm[2 * (size_t)i + 1] = (double)(v1 / v2);
    tt[2 * (size_t)i] = (float)(X(c, 0, i) + c->hsml[i] * nrm[2 * (size_t)i]);
    tt[2 * (size_t)i + 1] = (float)(X(c, 1, i) + c->hsml[i] * nrm[2 * (size_t)i + 1]);
    tau[2 * (size_t)i] = (float)(-nrm[2 * (size_t)i + 1]);
    tau[2 * (size_t)i + 1] = (float)nrm[2 * (size_t)i];
  }
  /* step 3: a particle with a neighbour in its scan region is inside */
  const float sqrt2 = sqrtf(2.0f);
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    int t = c->ptype[q];
    int i = c->pi[q], j = c->pj[q];
    int side[2] = {0, 0}; /* check i against j, check j against i */
    if (t == 2 || t == 3) side[0] = side[1] = 1;
    else if (t == 6 || t == 9) side[1] = 1;
    for (int sdx = 0; sdx < 2; sdx++) {
      if (!side[sdx]) continue;
      int a = sdx == 0 ? i : j, b = sdx == 0 ? j : i;
      if (c->subset[a] != 0.0) continue;
      double ddx = X(c, 0, b) - X(c, 0, a), ddy = X(c, 1, b) - X(c, 1, a);
      float xba = (float)sqrt(ddx * ddx + ddy * ddy);
      float xbt0 = (float)(X(c, 0, b) - (double)tt[2 * (size_t)a]);
      float xbt1 = (float)(X(c, 1, b) - (double)tt[2 * (size_t)a + 1]);
      float xbt_norm = sqrtf(xbt0 * xbt0 + xbt1 * xbt1);
      float prod = (float)(fabs(nrm[2 * (size_t)a] * (double)xbt0 + nrm[2 * (size_t)a + 1] * (double)xbt1) +
                           (double)fabsf(tau[2 * (size_t)a] * xbt0 + tau[2 * (size_t)a + 1] * xbt1));
      float limit = (float)((double)sqrt2 * c->hsml[a]);
      if (xba >= limit && (double)xbt_norm < c->hsml[a]) {
        c->subset[a] = 2.0;
        f_int[a] = -1.0f;
      } else if (xba < limit && (double)prod < c->hsml[a]) {
        c->subset[a] = 2.0;
        f_int[a] = -1.0f;
      }
    }
  }
  for (int i = 0; i < NT; i++)
    if (c->subset[i] == 0.0) c->subset[i] = 1.0;
  for (int i = 0; i < NT; i++)
    if (c->bc_or_not[i] != 1) c->bc_or_not[i] = 0;
  for (int i = 0; i < NT; i++) {
    if (c->subset[i] == 2.0 && c->bc_or_not[i] != 1) c->bc_or_not[i] = 0;
    else if (c->subset[i] == 1.0 && c->bc_or_not[i] != 1) c->bc_or_not[i] = 2;
    else if (c->subset[i] == 1.0 && c->bc_or_not[i] == 1) c->subset[i] = 2.0;
  }
  /* step 4: normals of the surface particles from their surface neighbours */
  for (int i = 0; i < 2 * NT; i++) nrm[i] = 0.0;
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    int t = c->ptype[q];
    if (t != 1 && t != 2 && t != 3) continue;
    int i = c->pi[q], j = c->pj[q];
    if (c->subset[i] == 1.0 && c->subset[j] == 1.0) {
      float x1 = (float)X(c, 0, i), y1 = (float)X(c, 1, i);
      float x2 = (float)X(c, 0, j), y2 = (float)X(c, 1, j);
      float xv = x2 - x1, yv = y2 - y1;
      nrm[2 * (size_t)i] = nrm[2 * (size_t)i] - (double)yv;
      nrm[2 * (size_t)i + 1] = nrm[2 * (size_t)i + 1] + (double)xv;
      nrm[2 * (size_t)j] = nrm[2 * (size_t)j] - (double)yv;
      nrm[2 * (size_t)j + 1] = nrm[2 * (size_t)j + 1] + (double)xv;
      nb[i] = nb[i] + 1.0f;
      nb[j] = nb[j] + 1.0f;
    }
    float gx = c->pdx[q], gy = c->pdy[q];
    float hf1i = (float)(c->mass[j] * (double)gx / c->rho[j]);
    float hf1j = (float)(-(c->mass[i] * (double)gx / c->rho[i]));
    float hf2i = (float)(c->mass[j] * (double)gy / c->rho[j]);
    float hf2j = (float)(-(c->mass[i] * (double)gy / c->rho[i]));
    gf[2 * (size_t)i] = gf[2 * (size_t)i] + (f_int[j] - f_int[i]) * hf1i;
    gf[2 * (size_t)j] = gf[2 * (size_t)j] + (f_int[i] - f_int[j]) * hf1j;
    gf[2 * (size_t)i + 1] = gf[2 * (size_t)i + 1] + (f_int[j] - f_int[i]) * hf2i;
    gf[2 * (size_t)j + 1] = gf[2 * (size_t)j + 1] + (f_int[i] - f_int[j]) * hf2j;
  }
  for (int i = 0; i < NT; i++) {
    if (c->subset[i] != 1.0) continue;
    double* n = &nrm[2 * (size_t)i];
    n[0] = n[0] / (double)nb[i];
    n[1] = n[1] / (double)nb[i];
    float norm_vect = (float)sqrt(n[0] * n[0] + n[1] * n[1]);
    n[0] = n[0] / (double)norm_vect;
    n[1] = n[1] / (double)norm_vect;
    float p_scal = (float)((double)gf[2 * (size_t)i] * n[0] + (double)gf[2 * (size_t)i + 1] * n[1]);
    if (p_scal < 0) {
      n[0] = -n[0];
      n[1] = -n[1];
    }
  }
  free(A);
  free(ff);
  free(f_int);
  free(gf);
  free(nb);
  free(tt);
  free(tau);
}

/* apply_stress_free (3_SPH_material_2018.f90:1775-1858): zero normal and shear traction
   on free-surface nodes away from walls (called inside BCs when ifsigman = 1) */
static void apply_stress_free(orc_ctx* c) {
  for (int ip = 0; ip < c->NN; ip++) {
    if (!(c->bc_or_not[ip] == 2 && c->bc_int[ip] != 1)) continue;
    double costh = c->normal[2 * (size_t)ip], sinth = c->normal[2 * (size_t)ip + 1];
    if (isnan(costh) || isnan(sinth)) continue;
    double s2 = sinth * sinth, c2 = costh * costh, sc = sinth * costh;
    double sxx0 = S(c, 0, ip), syy0 = S(c, 1, ip), sxy0 = S(c, 2, ip);
    double stt = (s2 * sxx0 - (2.0 * sc) * sxy0) + c2 * syy0;
    S(c, 0, ip) = s2 * stt;
    S(c, 1, ip) = c2 * stt;
    S(c, 2, ip) = -(sc * stt);
    S(c, 3, ip) = c2 * stt;
  }
}

/* XSPH_update (2_SPH_main_2018.f90:189-239) */
static void xsph_update(orc_ctx* c) {
  const int NT = c->NT;
  double* vs = xcalloc(2 * (size_t)NT, sizeof(double));
  double* xl = xcalloc(2 * (size_t)NT, sizeof(double));
  memcpy(xl, c->x, 2 * (size_t)NT * sizeof(double));
  const double eps = 0.5;
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    int t = c->ptype[q];
    if (t != 2 && t != 3) continue;
    int i = c->pi[q], j = c->pj[q];
    double w = (double)c->pw[q];
    if (t == 2) {
      for (int d = 0; d < 2; d++)
        vs[d + 2 * (size_t)i] += ((c->mass[j] / c->rho[j]) * (V(c, d, j) - V(c, d, i))) * w;
      for (int d = 0; d < 2; d++)
        vs[d + 2 * (size_t)j] += ((c->mass[i] / c->rho[i]) * (V(c, d, i) - V(c, d, j))) * w;
    } else {
      for (int d = 0; d < 2; d++)
        vs[d + 2 * (size_t)j] += ((c->mass[i] / c->rho[i]) * (V(c, d, i) - V(c, d, j))) * w;
      for (int d = 0; d < 2; d++)
        vs[d + 2 * (size_t)i] += ((c->mass[j] / c->rho[j]) * (V(c, d, j) - V(c, d, i))) * w;
      if (c->bc_or_not[i] == 2 && c->bc_or_not[j] != 2) c->bc_or_not[j] = 3;
      if (c->bc_or_not[j] == 2 && c->bc_or_not[i] != 2) c->bc_or_not[i] = 3;
    }
  }
  const double dt = c->p.dt_sph;
  for (int i = 0; i < NT; i++)
    for (int d = 0; d < 2; d++)
      X(c, d, i) = xl[d + 2 * (size_t)i] + dt * (V(c, d, i) + eps * vs[d + 2 * (size_t)i]);
  free(vs);
  free(xl);
}

/* shift_stress_points (2_SPH_main_2018.f90:244-368) with isolated_nodes (:373-398): every
   shift_update steps the stress-points are placed again around their nodes (fixed offsets
   r_x, r_y, or along the node velocity with the velocity-vector variant); then, every step,
   the stress-points of nodes next to a wall moving faster than 0.4 and of nodes with fewer
   than two node neighbours are put on their node.  cos_theta, sin_theta, r_x2 and abs_vel
   are FP32 in the reference. */
static void shift_stress_points(orc_ctx* c) {
  const int NN = c->NN, np = c->p.npoints;
  const double dx = c->p.dx, rx = c->p.r_x, ry = c->p.r_y;
  if (c->itimestep % c->p.shift_update == 0) {
    if (c->p.vel_vector) {
      for (int i = 0; i < NN; i++) {
        const double ex = X(c, 0, i) - c->x10[2 * (size_t)i];
        const double ey = X(c, 1, i) - c->x10[2 * (size_t)i + 1];
        c->disp10[i] = sqrt(ex * ex + ey * ey) / dx;
      }
      for (int i = 0; i < NN; i++) {
        c->x10[2 * (size_t)i] = X(c, 0, i);
        c->x10[2 * (size_t)i + 1] = X(c, 1, i);
      }
      for (int i = 0; i < NN; i++) {
        const double v0 = V(c, 0, i), v1 = V(c, 1, i);
        const float ct = (float)(v0 / sqrt(v0 * v0 + v1 * v1));
        const float st = (float)(v1 / sqrt(v0 * v0 + v1 * v1));
        float r0 = (float)((dx / 2) * (double)ct), r1 = (float)((dx / 2) * (double)st);
        if (r0 > 0 && r0 < dx / 5) r0 = (float)((double)r0 + dx / 3.0);
        if (r1 > 0 && r1 < dx / 5) r1 = (float)((double)r1 + dx / 3.0);
        if (r0 < 0 && r0 > -(dx / 5)) r0 = (float)((double)r0 - dx / 3.0);
        if (r1 < 0 && r1 > -(dx / 5)) r1 = (float)((double)r1 - dx / 3.0);
        if (c->disp10[i] > c->p.disp_tol) {
          const int k = NN + 2 * i;
          X(c, 0, k) = X(c, 0, i) + (double)r0;
          X(c, 1, k) = X(c, 1, i) + (double)r1;
          X(c, 0, k + 1) = X(c, 0, i) - (double)r0;
          X(c, 1, k + 1) = X(c, 1, i) - (double)r1;
        }
      }
    } else {
      for (int i = 0; i < NN; i++) {
        const int k = NN + np * i;
        if (np == 1) {
          X(c, 0, k) = X(c, 0, i) + rx;
          X(c, 1, k) = X(c, 1, i) + ry;
        } else if (np == 2) { /* the second point's y offset is r_x in the reference */
          X(c, 0, k) = X(c, 0, i) + rx;
          X(c, 1, k) = X(c, 1, i) + ry;
          X(c, 0, k + 1) = X(c, 0, i) - rx;
          X(c, 1, k + 1) = X(c, 1, i) - rx;
        } else if (np == 3) {
          X(c, 0, k) = X(c, 0, i);
          X(c, 1, k) = X(c, 1, i) + ry;
          X(c, 0, k + 1) = X(c, 0, i) - rx;
          X(c, 1, k + 1) = X(c, 1, i) - ry;
          X(c, 0, k + 2) = X(c, 0, i) + rx;
          X(c, 1, k + 2) = X(c, 1, i) - ry;
        }
      }
    }
  }
  /* n_int: node-node pairs of each node (isolated_nodes; artificial_viscosity and
     XSPH_update count the same pairs) */
  int32_t* n_int = xcalloc((size_t)NN, sizeof(int32_t));
  for (int64_t k = 0; k < c->npairs; k++)
    if (c->ptype[k] == 3) {
      n_int[c->pi[k]]++;
      n_int[c->pj[k]]++;
    }
  for (int i = 0; i < NN; i++) {
    const double v0 = V(c, 0, i), v1 = V(c, 1, i);
    const float abs_vel = (float)sqrt(v0 * v0 + v1 * v1);
    const int k = NN + np * i;
    const int off = (c->bc_int[i] == 1 && abs_vel > 0.4f) || n_int[i] < 2;
    if (off)
      for (int q = 0; q < np && q < 3; q++) {
        X(c, 0, k + q) = X(c, 0, i);
        X(c, 1, k + q) = X(c, 1, i);
      }
  }
  free(n_int);
}

/* time_integration (2_SPH_main_2018.f90:78-184) */
static int time_integration(orc_ctx* c) {
  const int NN = c->NN, NT = c->NT;
  const int ncrit = (int)c->p.props[1];
  const int outside = c->p.sp_sph && !c->p.inside_approach;
  c->itimestep++;
  check_out_domain(c);
  if (grid_find_new(c)) return SPS_ERR_CAPACITY;
  pint_update(c);
  if (outside && c->p.sph_shift && c->itimestep > 1 &&
      (c->itimestep - 1) % c->p.shift_update == 0) {
    stress_point_update(c);
    if (ncrit == 12) adapt_all(c);
  }
  memcpy(c->vx0, c->vel, 2 * (size_t)NT * sizeof(double));
  memcpy(c->x0, c->x, 2 * (size_t)NT * sizeof(double));
  rk4(c);
  for (int i = NN; i < NT; i++) c->intvars1[i] = c->intvars1[i] + c->p.dt_sph * c->Ddev[i];
  stress_point_update(c);
  if (c->p.sp_sph) {
    if (ncrit == 12) adapt_all(c);
    if (c->p.no_bcs > 0) bcs(c);
  }
  if (c->p.update_x) {
    if (c->p.xsph) {
      xsph_update(c);
    } else {
      for (int i = 0; i < NT; i++)
        for (int d = 0; d < 2; d++) {
          float vh = (float)(0.5 * (c->vx0[d + 2 * (size_t)i] + V(c, d, i)));
          X(c, d, i) = c->x0[d + 2 * (size_t)i] + (double)vh * c->p.dt_sph;
        }
    }
    free_surface(c); /* ndimn == 2 */
    if (outside) shift_stress_points(c);
    if (!c->p.sp_sph)
      for (int i = 0; i < NN; i++)
        for (int d = 0; d < 2; d++) X(c, d, NN + i) = X(c, d, i);
    for (int i = 0; i < NN; i++)
      for (int d = 0; d < 2; d++)
        c->displ[d + 2 * (size_t)i] = X(c, d, i) - c->x00[d + 2 * (size_t)i];
  } else {
    for (int i = 0; i < NN; i++)
      for (int d = 0; d < 2; d++)
        c->displ[d + 2 * (size_t)i] =
            c->displ[d + 2 * (size_t)i] +
            (0.5 * (c->vx0[d + 2 * (size_t)i] + V(c, d, i))) * c->p.dt_sph;
  }
  return SPS_OK;
}

/* ------------------------------------------------------------------------------------ */

int orc_create(const sps_params* p, orc_ctx** out) {
  if (!p || !out) return SPS_ERR_ARG;
  *out = NULL;
  if (p->ndimn != 2 || p->nstre != 4) return SPS_ERR_UNSUPPORTED;
  if (p->nnode <= 0 || p->nstress < 0 || p->ndummy < 0 || p->ndummy2 < 0 ||
      p->ndummy2 > p->ndummy)
    return SPS_ERR_ARG;
  int ntype_eco = (int)p->props[0], ncrit = (int)p->props[1];
  /* Cam Clay (5) is not supported: its yield-surface size Internal_Vars(3) is never
     integrated by the reference and stays 0 */
  if (ntype_eco > 1 && !((ncrit >= 1 && ncrit <= 4) || ncrit == 12)) return SPS_ERR_UNSUPPORTED;
  if (ntype_eco > 1 && ncrit <= 4 && !(p->props[6] > (double)0.001f)) return SPS_ERR_ARG;
  if (ntype_eco > 1 && ncrit <= 4 && (p->ntype_solid < 1 || p->ntype_solid > 3))
    return SPS_ERR_UNSUPPORTED;
  if (p->skf < 1 || p->skf > 3) return SPS_ERR_ARG;
  if (!p->sp_sph && p->nstress != p->nnode) return SPS_ERR_ARG;
  if (p->sp_sph && !p->inside_approach &&
      (p->npoints < 1 || p->npoints > 4 || p->shift_update < 1 ||
       p->nstress != p->npoints * p->nnode || (p->vel_vector && p->npoints != 2)))
    return SPS_ERR_ARG;
  orc_ctx* c = xcalloc(1, sizeof(orc_ctx));
  if (!c) return SPS_ERR_ARG;
  c->p = *p;
  c->NN = p->nnode;
  c->NT = p->nnode + p->nstress;
  c->N2 = c->NT + p->ndummy;
  size_t N2 = c->N2, NT = c->NT, NN = c->NN;
  if (p->ntcurves > 0) {
    size_t nt = (size_t)p->ntcurves * p->mptstcurves;
    c->nptstcurves = xcalloc(p->ntcurves, sizeof(int32_t));
    c->ttcurves = xcalloc(nt, sizeof(double));
    c->ftcurves = xcalloc(nt, sizeof(float));
    memcpy(c->nptstcurves, p->nptstcurves, p->ntcurves * sizeof(int32_t));
    memcpy(c->ttcurves, p->ttcurves, nt * sizeof(double));
    memcpy(c->ftcurves, p->ftcurves, nt * sizeof(float));
  }
  if (p->no_bcs > 0) {
    c->bc_list = xcalloc(8 * (size_t)p->no_bcs, sizeof(double));
    memcpy(c->bc_list, p->bc_list, 8 * (size_t)p->no_bcs * sizeof(double));
  }
  c->wall_position = xcalloc(N2, sizeof(float));
  c->horizontal_or_not = xcalloc(N2, sizeof(float));
  if (p->wall_position) memcpy(c->wall_position, p->wall_position, N2 * sizeof(float));
  if (p->horizontal_or_not)
    memcpy(c->horizontal_or_not, p->horizontal_or_not, N2 * sizeof(float));
  c->p.nptstcurves = c->nptstcurves;
  c->p.ttcurves = c->ttcurves;
  c->p.ftcurves = c->ftcurves;
  c->p.bc_list = c->bc_list;
  c->p.wall_position = c->wall_position;
  c->p.horizontal_or_not = c->horizontal_or_not;
  c->x = xcalloc(2 * N2, sizeof(double));
  c->vel = xcalloc(2 * N2, sizeof(double));
  c->stress = xcalloc(4 * N2, sizeof(double));
  c->mass = xcalloc(N2, sizeof(double));
  c->rho = xcalloc(N2, sizeof(double));
  c->hsml = xcalloc(N2, sizeof(double));
  c->x00 = xcalloc(2 * N2, sizeof(double));
  c->x0 = xcalloc(2 * N2, sizeof(double));
  c->vx0 = xcalloc(2 * N2, sizeof(double));
  c->displ = xcalloc(2 * NN, sizeof(double));
  c->itype = xcalloc(N2, sizeof(int32_t));
  c->out_domain = xcalloc(N2, sizeof(int32_t));
  c->bc_or_not = xcalloc(NT, sizeof(int32_t));
  c->bc_info = xcalloc(8 * NT, sizeof(int32_t));
  c->bc_int = xcalloc(NN, sizeof(int32_t));
  c->normal = xcalloc(2 * (size_t)NT, sizeof(double));
  c->subset = xcalloc((size_t)NT, sizeof(double));
  c->intvars1 = xcalloc(NT, sizeof(double));
  c->f_drucker = xcalloc(NT, sizeof(double));
  c->grad_u = xcalloc(4 * NT, sizeof(double));
  c->Ddev = xcalloc(NT, sizeof(double));
  c->f_bound = xcalloc(2 * NN, sizeof(double));
  c->art_visc = xcalloc(2 * NN, sizeof(double));
  c->art_force = xcalloc(2 * NN, sizeof(double));
  c->x10 = xcalloc(2 * NN, sizeof(double));
  c->disp10 = xcalloc(NN, sizeof(double));
  c->which_cell = xcalloc(N2, sizeof(int32_t));
  c->cell_list = xcalloc(N2, sizeof(int32_t));
  for (size_t i = 0; i < NT; i++) c->bc_info[8 * i] = (int32_t)(i + 1);
  *out = c;
  return SPS_OK;
}

int orc_upload(orc_ctx* c, const double* x, const double* vel, const double* stress,
               const double* mass, const double* rho, const double* hsml, const int32_t* itype,
               const double* intvars1, const double* f_drucker, const double* x00) {
  if (!c || !x || !vel || !stress || !mass || !rho || !hsml || !itype) return SPS_ERR_ARG;
  size_t N2 = c->N2, NT = c->NT;
  memcpy(c->x, x, 2 * N2 * sizeof(double));
  memcpy(c->vel, vel, 2 * N2 * sizeof(double));
  memcpy(c->stress, stress, 4 * N2 * sizeof(double));
  memcpy(c->mass, mass, N2 * sizeof(double));
  memcpy(c->rho, rho, N2 * sizeof(double));
  memcpy(c->hsml, hsml, N2 * sizeof(double));
  memcpy(c->itype, itype, N2 * sizeof(int32_t));
  if (intvars1) memcpy(c->intvars1, intvars1, NT * sizeof(double));
  if (f_drucker) memcpy(c->f_drucker, f_drucker, NT * sizeof(double));
  memcpy(c->x00, x00 ? x00 : x, 2 * N2 * sizeof(double));
  memset(c->out_domain, 0, N2 * sizeof(int32_t));
  memset(c->displ, 0, 2 * (size_t)c->NN * sizeof(double));
  /* Setup_Global_Arrays (3_SPH_material_2018.f90:1032): x_10 starts at the node positions */
  memcpy(c->x10, c->x, 2 * (size_t)c->NN * sizeof(double));
  memset(c->disp10, 0, (size_t)c->NN * sizeof(double));
  c->itimestep = 0;
  c->uploaded = 1;
  return SPS_OK;
}

int orc_upload_bcs(orc_ctx* c, const int32_t* bc_or_not, const int32_t* bc_info) {
  if (!c) return SPS_ERR_ARG;
  if (bc_or_not) memcpy(c->bc_or_not, bc_or_not, (size_t)c->NT * sizeof(int32_t));
  if (bc_info) memcpy(c->bc_info, bc_info, 8 * (size_t)c->NT * sizeof(int32_t));
  return SPS_OK;
}

int orc_step(orc_ctx* c, int32_t nsteps, double* time_sph) {
  if (!c || !time_sph || nsteps < 0) return SPS_ERR_ARG;
  if (!c->uploaded) return SPS_ERR_STATE;
  c->time_sph = *time_sph;
  for (int s = 0; s < nsteps; s++) {
    int rc = time_integration(c);
    if (rc) return rc;
    c->time_sph = c->time_sph + c->p.dt_sph;
    c->step_count++;
  }
  *time_sph = c->time_sph;
  return SPS_OK;
}

int orc_download(orc_ctx* c, double* x, double* vel, double* stress, double* rho,
                 double* intvars1, double* displ, int32_t* bc_or_not, double* f_drucker) {
  if (!c) return SPS_ERR_ARG;
  size_t N2 = c->N2, NT = c->NT;
  if (x) memcpy(x, c->x, 2 * N2 * sizeof(double));
  if (vel) memcpy(vel, c->vel, 2 * N2 * sizeof(double));
  if (stress) memcpy(stress, c->stress, 4 * N2 * sizeof(double));
  if (rho) memcpy(rho, c->rho, N2 * sizeof(double));
  if (intvars1) memcpy(intvars1, c->intvars1, NT * sizeof(double));
  if (displ) memcpy(displ, c->displ, 2 * (size_t)c->NN * sizeof(double));
  if (bc_or_not) memcpy(bc_or_not, c->bc_or_not, NT * sizeof(int32_t));
  if (f_drucker) memcpy(f_drucker, c->f_drucker, NT * sizeof(double));
  return SPS_OK;
}

int orc_dump_pairs(orc_ctx* c, int32_t* pair_i, int32_t* pair_j, int32_t* pint_type, float* w,
                   float* dwdx, float* dwdy, int64_t* npairs) {
  if (!c || !npairs) return SPS_ERR_ARG;
  if (!pair_i) {
    *npairs = c->npairs;
    return SPS_OK;
  }
  if (*npairs < c->npairs) return SPS_ERR_CAPACITY;
  for (int64_t k = 0; k < c->npairs; k++) {
    int64_t q = c->order[k];
    pair_i[k] = c->pi[q] + 1;
    pair_j[k] = c->pj[q] + 1;
    if (pint_type) pint_type[k] = c->ptype[q];
    if (w) w[k] = c->pw[q];
    if (dwdx) dwdx[k] = c->pdx[q];
    if (dwdy) dwdy[k] = c->pdy[q];
  }
  *npairs = c->npairs;
  return SPS_OK;
}

int orc_download_surface(orc_ctx* c, double* normal, int32_t* subset) {
  if (!c) return SPS_ERR_ARG;
  if (normal) memcpy(normal, c->normal, 2 * (size_t)c->NT * sizeof(double));
  if (subset)
    for (int i = 0; i < c->NT; i++) subset[i] = (int32_t)c->subset[i];
  return SPS_OK;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  void* ptrs[] = {c->nptstcurves, c->ttcurves, c->ftcurves, c->bc_list, c->wall_position,
                  c->horizontal_or_not, c->x, c->vel, c->stress, c->mass, c->rho, c->hsml,
                  c->x00, c->x0, c->vx0, c->displ, c->itype, c->out_domain, c->bc_or_not,
                  c->bc_info, c->bc_int, c->intvars1, c->f_drucker, c->grad_u, c->Ddev,
                  c->normal, c->subset,
                  c->f_bound, c->art_visc, c->art_force, c->x10, c->disp10, c->pi, c->pj, c->ptype, c->pw, c->pdx, c->pdy,
                  c->order, c->which_cell, c->cell_cnt, c->cell_start, c->cell_list};
  for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++) free(ptrs[k]);
  free(c);
}
