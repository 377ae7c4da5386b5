/*
 * relx_oracle.c -- CPU restatement of relxill's relativistic convolution path
 * in double precision.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the GPU path is checked
 * against (tests/, __graft_entry__.smoke(), the cpu_baseline leg of bench.py);
 * the product never links or calls it.  Each function restates the reference
 * algorithm it cites (paths inside the relxill repository).  It is pinned
 * against the compiled reference (oracle/build_ref.sh) and the reference's
 * table-free known-answer tests (tests/test_oracle_pins.py).
 *
 * Differences to the reference that do not change results:
 *  - no caches: every call recomputes everything (the reference caches give
 *    the same numbers for the same inputs);
 *  - relb_func's remembered g* index (Relprofile.cpp:497-500) is replaced by
 *    a binary search, which returns the same index for every input;
 *  - tables are loaded eagerly (relline, lamp post) or per spectrum row on
 *    first use (xillver, like check_xilltab_cache).
 *
 * Scope: models relline, relconv, relxill, relxilllp, relline_lp, relconv_lp
 * and xillver (cut-off power law, broken power-law or point lamp-post
 * emissivity, returning radiation with its xillver correction factors,
 * ionisation gradients CONST / PL / ALPHA).
 */
#define _POSIX_C_SOURCE 200809L
#include "relx_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "shim/fftw3.h"
#include "shim/fitsio.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---- constants: common.h:47-180, Xillspec.h:28-38, Relbase.h:38-39 ---- */
#define EMIS_TYPE_BKN 1
#define EMIS_TYPE_LP 2
#define N_FRAD 1000
#define N_ZONES 10
#define N_ZONES_IONGRAD 25
#define N_ZONES_MAX 50
#define RELTABLE_MAX_R 1000.0
#define GFAC_H 5e-3
#define N_ENER_CONV 4096
#define EMIN_RELXILL_CONV 0.00035
#define EMAX_RELXILL_CONV 2000.0
#define N_ENER_COARSE 500
#define EMIN_XILLVER_NORMALIZATION 0.1
#define EMAX_XILLVER_NORMALIZATION 1000.0
#define EMIN_XILLVER 0.01
#define EMAX_XILLVER 1000.0
#define RELCONV_EMIN 0.01
#define RELCONV_EMAX 1000.0
#define ION_GRAD_TYPE_CONST 0
#define ION_GRAD_TYPE_PL 1
#define ION_GRAD_TYPE_ALPHA 2
#define PARAM_GAM 0
#define PARAM_AFE 1
#define PARAM_LXI 2
#define PARAM_ECT 3
#define PARAM_DNS 4
#define PARAM_INC 7

/* ======================================================================= */
/* numerics utilities (relutility.c)                                        */
/* ======================================================================= */

/* relutility.c:24-26 */
static double interp_lin_1d(double ifac_r, double rlo, double rhi) { return ifac_r * rhi + (1.0 - ifac_r) * rlo; }

double relxo_interp_lin_1d(double f, double lo, double hi) { return interp_lin_1d(f, lo, hi); }

/* relutility.c:41-43 */
static double interp_log_1d(double ifac_r, double rlo, double rhi) {
  return exp(ifac_r * log(rhi) + (1.0 - ifac_r) * log(rlo));
}

/* relutility.c:46-58 */
static double interp_lin_2d(double f1, double f2, double r11, double r12, double r21, double r22) {
  return (1.0 - f1) * (1.0 - f2) * r11 + (f1) * (1.0 - f2) * r12 + (1.0 - f1) * (f2) * r21 + (f1) * (f2) * r22;
}

double relxo_interp_lin_2d(double f1, double f2, double r11, double r12, double r21, double r22) {
  return interp_lin_2d(f1, f2, r11, r12, r21, r22);
}
double relxo_interp_lin_2d_float(double f1, double f2, float r11, float r12, float r21, float r22) {
  return interp_lin_2d(f1, f2, r11, r12, r21, r22);
}

/* relutility.c:135-151: arr ascending, returns k with arr[k] <= val < arr[k+1] */
static int binary_search_float(const float *arr, int n, float val) {
  if (n <= 1) return -1;
  int klo = 0, khi = n - 1;
  while (khi - klo > 1) {
    int k = (khi + klo) / 2;
    if (arr[k] > val) khi = k; else klo = k;
  }
  return klo;
}

/* relutility.c:155-171 */
static int binary_search(const double *arr, int n, double val) {
  if (n <= 1) return -1;
  int klo = 0, khi = n - 1;
  while (khi - klo > 1) {
    int k = (khi + klo) / 2;
    if (arr[k] > val) khi = k; else klo = k;
  }
  return klo;
}

/* relutility.c:195-211: arr descending */
static int inv_binary_search(const double *arr, int n, double val) {
  if (n <= 1) return -1;
  int klo = 0, khi = n - 1;
  while (khi - klo > 1) {
    int k = (khi + klo) / 2;
    if (arr[k] < val) khi = k; else klo = k;
  }
  return klo;
}

/* relutility.c:233-244: pi*r*dr/2 ... returns r*dr*pi for a descending grid */
static double trapez_integ_single(const double *re, int ii, int nr) {
  double dr;
  if (ii == 0) dr = 0.5 * (re[ii] - re[ii + 1]);
  else if (ii == nr - 1) dr = 0.5 * (re[ii - 1] - re[ii]);
  else dr = 0.5 * (re[ii - 1] - re[ii + 1]);
  return re[ii] * dr * M_PI;
}

/* relutility.c:260-262 */
static double gstar2ener(double g, double gmin, double gmax, double ener) { return (g * (gmax - gmin) + gmin) * ener; }

/* relutility.c:399-405 */
static void get_log_grid(double *ener, int n, double emin, double emax) {
  for (int ii = 0; ii < n; ii++) {
    ener[ii] = 1.0 * ii / (n - 1) * (log(emax) - log(emin)) + log(emin);
    ener[ii] = exp(ener[ii]);
  }
}

/* relutility.c:407-417 */
static double get_ipol_factor_radius(double rlo, double rhi, double del_inci, double radius) {
  if (del_inci / M_PI * 180.0 <= 75.0) return (radius - rlo) / (rhi - rlo);
  return (log(radius) - log(rlo)) / (log(rhi) - log(rlo));
}

/* relutility.c:419-423 (float arithmetic on the factor, as in the reference) */
static void get_ipol_factor(const float value, const float *arr, int n, int *ind, double *ifac) {
  *ind = binary_search_float(arr, n, value);
  *ifac = (value - arr[*ind]) / (arr[*ind + 1] - arr[*ind]);
}

/* relutility.c:666-677 */
static void get_fine_radial_grid(double rin, double rout, double *re, int nr) {
  double r1 = 1.0 / sqrt(rout);
  double r2 = 1.0 / sqrt(rin);
  for (int ii = 0; ii < nr; ii++) {
    re[ii] = ((double) ii) * (r2 - r1) / (nr - 1) + r1;
    re[ii] = pow(1.0 / re[ii], 2);
  }
}

/* relutility.c:265-308 and IonGradient.cpp:457-492 (identical) */
static void get_rzone_grid(double rmin, double rmax, int nzones, double h, double *rgrid) {
  if (nzones == 1) {
    rgrid[0] = rmin;
    rgrid[1] = rmax;
    return;
  }
  double r_transition = rmin;
  int indr = 0;
  if (h > rmin) {
    r_transition = h;
    get_log_grid(rgrid, nzones + 1, rmin, rmax);
    indr = binary_search(rgrid, nzones + 1, r_transition);
    r_transition = rgrid[indr];
  }
  if (indr < nzones) {
    double rlo = r_transition, rhi = rmax;
    for (int ii = indr; ii < nzones + 1; ii++) {
      rgrid[ii] = 1.0 * (ii - indr) / (nzones - indr) * (1.0 / rhi - 1.0 / rlo) + 1.0 / rlo;
      rgrid[ii] = fabs(1.0 / rgrid[ii]);
    }
  }
}

/* relutility.c:549-601: flux-conserving rebin, ener has nbins+1 edges */
void relxo_rebin_spectrum(const double *ener, double *flu, int nbins, const double *ener0, const double *flu0,
                          int nbins0) {
  int imin = 0, imax = 0;
  for (int ii = 0; ii < nbins; ii++) {
    flu[ii] = 0.0;
    if ((ener0[0] <= ener[ii + 1]) && (ener0[nbins0] >= ener[ii])) {
      while (imin <= nbins0 && ener0[imin] <= ener[ii]) imin++;
      if (imin > 0) imin--;
      while (imax < nbins0 && ener0[imax] <= ener[ii + 1]) imax++;
      if (imax > 0) imax--;
      double elo = ener[ii], ehi = ener[ii + 1];
      if (elo < ener0[imin]) elo = ener0[imin];
      if (ehi > ener0[imax + 1]) ehi = ener0[imax + 1];
      if (imax == imin) {
        flu[ii] = (ehi - elo) / (ener0[imin + 1] - ener0[imin]) * flu0[imin];
      } else {
        double dmin = (ener0[imin + 1] - elo) / (ener0[imin + 1] - ener0[imin]);
        double dmax = (ehi - ener0[imax]) / (ener0[imax + 1] - ener0[imax]);
        flu[ii] += flu0[imin] * dmin + flu0[imax] * dmax;
        for (int jj = imin + 1; jj <= imax - 1; jj++) flu[ii] += flu0[jj];
      }
    }
  }
}

/* relutility.c:636-663: x0 descending, xn ascending */
static int inv_rebin_mean(const double *x0, const double *y0, int n0, const double *xn, double *yn, int nn) {
  if (xn[0] > xn[nn - 1] || x0[nn - 1] > x0[0]) return 1;
  if (xn[0] < x0[n0 - 1] || xn[nn - 1] > x0[0]) return 1;
  int in = nn - 1;
  for (int ii = 0; ii < n0 - 1; ii++) {
    if (x0[ii] > xn[in] && x0[ii + 1] <= xn[in]) {
      double ifac_r = (xn[in] - x0[ii + 1]) / (x0[ii] - x0[ii + 1]);
      yn[in] = interp_lin_1d(ifac_r, y0[ii + 1], y0[ii]);
      in--;
      if (in < 0) break;
    }
  }
  return 0;
}

static int env_is_one(const char *name) {
  const char *v = getenv(name);
  return v != NULL && (int) strtod(v, NULL) == 1;
}

/* ======================================================================= */
/* relativistic physics (Relphysics.cpp)                                    */
/* ======================================================================= */

/* Relphysics.cpp:139-150 */
double relxo_kerr_rms(double a) {
  double sign = (a < 0) ? -1.0 : 1.0;
  double Z1 = 1.0 + pow(1.0 - a * a, 1.0 / 3.0) * (pow(1.0 + a, 1.0 / 3.0) + pow(1.0 - a, 1.0 / 3.0));
  double Z2 = sqrt((3.0 * a * a) + (Z1 * Z1));
  return 3.0 + Z2 - sign * sqrt((3.0 - Z1) * (3.0 + Z1 + (2 * Z2)));
}

/* Relphysics.cpp:153-155 */
static double kerr_rplus(double a) { return 1 + sqrt(1 - a * a); }

/* Relphysics.cpp:127-129 */
static double relat_abberation(double del, double beta) {
  return acos((cos(del) - beta) / (1 - beta * cos(del)));
}

/* Relphysics.cpp:134-136 */
static double calc_g_inf(double height, double a) { return sqrt(1.0 - (2 * height / (height * height + a * a))); }

/* Relphysics.cpp:158-160 */
static double doppler_factor(double del, double bet) { return sqrt(1.0 - bet * bet) / (1.0 + bet * cos(del)); }

/* Relphysics.cpp:163-207 */
double relxo_gi_potential_lp(double r, double a, double h, double bet, double del) {
  double ut_d = ((r * sqrt(r) + a) / (sqrt(r) * sqrt(r * r - 3 * r + 2 * a * sqrt(r))));
  double ut_h = sqrt((h * h + a * a) / (h * h - 2 * h + a * a));
  double gi = ut_d / ut_h;
  if (fabs(bet) < 1e-6) return gi;
  double gam = 1.0 / sqrt(1.0 - bet * bet);
  double sign = (del > M_PI / 2) ? -1.0 : 1.0;
  double delta_eq = h * h - 2 * h + a * a;
  double q2 = (pow(sin(del), 2)) * (pow((h * h + a * a), 2) / delta_eq) - a * a;
  double beta_fac = sqrt(pow((h * h + a * a), 2) - delta_eq * (q2 + a * a));
  beta_fac = gam * (1.0 + sign * beta_fac / (h * h + a * a) * bet);
  return gi / beta_fac;
}

/* Relphysics.cpp:123-125 */
static double density_ss73_zone_a(double radius, double rms) {
  return pow((radius / rms), (3. / 2)) * pow((1 - sqrt(rms / radius)), -2);
}

/* ======================================================================= */
/* parameters (ModelDefinition.cpp, LocalModel.cpp, lmodel_relxill_public.dat) */
/* ======================================================================= */

typedef struct {
  int model;  /* RELXO_RELLINE, ... */
  int is_relxill;
  int emis_type;
  double a, incl, emis1, emis2, rbr, rin, rout, lineE, z, height, htop, gamma, beta;
  int limb, num_zones, return_rad, ion_grad_type;
  /* xillver parameters */
  double gam, afe, lxi, ect, dens, refl_frac, iongrad_index;
  int interpret_reflfrac_as_boost;
  int prim_type;  /* 0: cut-off power law (ect = Ecut), 1: nthcomp (ect = kTe; the Cp models) */
} Params;

/* get_num_zones, relutility.c:506-544 */
static int get_num_zones(int is_relxill, int emis_type, int ion_grad_type) {
  const char *env = getenv("RELXILL_NUM_RZONES");
  int env_n = env ? (int) atof(env) : 0;
  if (ion_grad_type != ION_GRAD_TYPE_CONST) {
    if (env && env_n > 9 && env_n <= N_ZONES_MAX) return env_n;
    return N_ZONES_IONGRAD;
  } else if (is_relxill && emis_type == EMIS_TYPE_LP) {
    if (env && env_n > 0 && env_n <= N_ZONES_MAX) return env_n;
    return N_ZONES;
  }
  return 1;
}

/* check_parameter_bounds, ModelDefinition.cpp:153-273 */
static int check_parameter_bounds(Params *p) {
  if (p->rin < 0) p->rin = -1.0 * p->rin * relxo_kerr_rms(p->a);
  if (p->rout < 0) p->rout = -1.0 * p->rout * relxo_kerr_rms(p->a);
  if (p->rbr < 0) p->rbr = -1.0 * p->rbr * relxo_kerr_rms(p->a);
  int status = 0;
  if (p->rout <= p->rin) status = 1;
  double rms = relxo_kerr_rms(p->a);
  if (p->rin < rms) p->rin = rms;
  if (p->a > 0.9982) return 1;
  if (p->a < -1) return 1;
  if (p->incl < 3 * M_PI / 180 || p->incl > 87 * M_PI / 180) return 1;
  if (p->rout <= p->rin) return 1;
  if (p->rout > 1000.0) p->rout = 1000.0;
  if (p->emis_type == EMIS_TYPE_BKN) {
    if (p->rbr < p->rin) p->rbr = p->rin;
    if (p->rbr > p->rout) p->rbr = p->rout;
  }
  if (p->emis_type == EMIS_TYPE_LP) {
    if (p->beta < 0) p->beta = 0.0;
    if (p->beta > 0.99) p->beta = 0.99;
    if (p->height < 0) p->height = -1.0 * p->height * kerr_rplus(p->a);
    if (p->htop < 0) p->htop = -1.0 * p->htop * kerr_rplus(p->a);
    double r_event = kerr_rplus(p->a);
    if ((1.1 * r_event - p->height) > 1e-4) p->height = r_event * 1.1;
  }
  return status;
}

/* map the lmodel.dat parameter arrays (lmodel_relxill_public.dat:1-75) */
static int map_params(int model, const double *v, int ion_grad_type, double iongrad_index, Params *p) {
  memset(p, 0, sizeof(*p));
  p->model = model;
  p->ect = 300;  /* ModelDefinition.cpp:360 default */
  p->dens = 15;  /* ModelDefinition.cpp:362 default */
  switch (model) {
    case RELXO_RELLINE:
      p->emis_type = EMIS_TYPE_BKN;
      p->lineE = v[0]; p->emis1 = v[1]; p->emis2 = v[2]; p->rbr = v[3]; p->a = v[4];
      p->incl = v[5] * M_PI / 180; p->rin = v[6]; p->rout = v[7]; p->z = v[8]; p->limb = (int) lround(v[9]);
      break;
    case RELXO_RELCONV:
      p->emis_type = EMIS_TYPE_BKN;
      p->emis1 = v[0]; p->emis2 = v[1]; p->rbr = v[2]; p->a = v[3]; p->incl = v[4] * M_PI / 180;
      p->rin = v[5]; p->rout = v[6]; p->limb = (int) lround(v[7]);
      break;
    case RELXO_RELXILL:
      p->is_relxill = 1;
      p->emis_type = EMIS_TYPE_BKN;
      p->emis1 = v[0]; p->emis2 = v[1]; p->rbr = v[2]; p->a = v[3]; p->incl = v[4] * M_PI / 180;
      p->rin = v[5]; p->rout = v[6]; p->z = v[7]; p->gam = v[8]; p->lxi = v[9]; p->afe = v[10];
      p->ect = v[11]; p->refl_frac = v[12];
      break;
    case RELXO_RELXILLLP:
      p->is_relxill = 1;
      p->emis_type = EMIS_TYPE_LP;
      p->height = v[0]; p->beta = v[1]; p->a = v[2]; p->incl = v[3] * M_PI / 180; p->rin = v[4];
      p->rout = v[5]; p->z = v[6]; p->gam = v[7]; p->lxi = v[8]; p->afe = v[9]; p->ect = v[10];
      p->refl_frac = v[11]; p->return_rad = (int) lround(v[12]);
      p->interpret_reflfrac_as_boost = (int) lround(v[13]);
      break;
    case RELXO_RELLINELP:  /* lmodel_relxill_public.dat:23-33 */
      p->emis_type = EMIS_TYPE_LP;
      p->lineE = v[0]; p->height = v[1]; p->a = v[2]; p->incl = v[3] * M_PI / 180; p->rin = v[4]; p->rout = v[5];
      p->z = v[6]; p->limb = (int) lround(v[7]); p->gam = v[8]; p->return_rad = (int) lround(v[9]);
      break;
    case RELXO_RELCONVLP:  /* lmodel_relxill_public.dat:35-44 */
      p->emis_type = EMIS_TYPE_LP;
      p->height = v[0]; p->beta = v[1]; p->a = v[2]; p->incl = v[3] * M_PI / 180; p->rin = v[4]; p->rout = v[5];
      p->limb = (int) lround(v[6]); p->gam = v[7]; p->return_rad = (int) lround(v[8]);
      break;
    case RELXO_XILLVER:  /* lmodel_relxill_public.dat:77-84, get_xill_params (ModelDefinition.cpp:339-388) */
      p->gam = v[0]; p->afe = v[1]; p->ect = v[2]; p->lxi = v[3]; p->z = v[4];
      p->incl = v[5];  /* degrees: xillParam keeps the inclination in degrees */
      p->refl_frac = v[6];
      return 0;      /* no relativistic parameters (get_rel_params returns none for xillver models) */
    case RELXO_XILLVERCP:  /* lmodel_relxill_public.dat:86-94 */
      p->prim_type = 1;
      p->gam = v[0]; p->afe = v[1]; p->ect = v[2]; p->lxi = v[3]; p->dens = v[4]; p->z = v[5];
      p->incl = v[6];
      p->refl_frac = v[7];
      return 0;
    case RELXO_RELXILLCP:  /* lmodel_relxill_public.dat:96-110 */
      p->prim_type = 1;
      p->is_relxill = 1;
      p->emis_type = EMIS_TYPE_BKN;
      p->incl = v[0] * M_PI / 180; p->a = v[1]; p->rin = v[2]; p->rout = v[3]; p->rbr = v[4]; p->emis1 = v[5];
      p->emis2 = v[6]; p->z = v[7]; p->gam = v[8]; p->lxi = v[9]; p->dens = v[10]; p->afe = v[11]; p->ect = v[12];
      p->refl_frac = v[13];
      break;
    case RELXO_RELXILLLPCP:  /* lmodel_relxill_public.dat:112-129: the ionisation gradient is a parameter */
      p->prim_type = 1;
      p->is_relxill = 1;
      p->emis_type = EMIS_TYPE_LP;
      p->incl = v[0] * M_PI / 180; p->a = v[1]; p->rin = v[2]; p->rout = v[3]; p->height = v[4]; p->beta = v[5];
      p->gam = v[6]; p->lxi = v[7]; p->dens = v[8]; p->afe = v[9]; p->ect = v[10]; p->refl_frac = v[11];
      p->z = v[12];
      iongrad_index = v[13];
      ion_grad_type = (int) lround(v[14]);
      p->return_rad = (int) lround(v[15]);
      p->interpret_reflfrac_as_boost = (int) lround(v[16]);
      break;
    default:
      return 1;
  }
  p->gamma = p->gam;  /* relParam gamma = XPar::gamma (ModelDefinition.cpp:305) */
  p->ion_grad_type = ion_grad_type;
  p->iongrad_index = iongrad_index;
  if (check_parameter_bounds(p)) return 1;
  p->num_zones = get_num_zones(p->is_relxill, p->emis_type, p->ion_grad_type);
  return 0;
}

/* do_renorm_model, relutility.c:603-623 */
static int do_renorm_model(const Params *p) {
  if (p->is_relxill) return (p->emis_type == EMIS_TYPE_LP || env_is_one("RELLINE_PHYSICAL_NORM")) ? 0 : 1;
  return env_is_one("RELLINE_PHYSICAL_NORM") ? 0 : 1;
}

/* ======================================================================= */
/* tables (reltable.c, xilltable.c)                                         */
/* ======================================================================= */

typedef struct {
  int n_a, n_mu0, n_r, n_g;
  float *a, *mu0;
  /* [ia][im] blocks: r, gmin, gmax [n_r]; trff1.. [n_r][n_g] */
  float *r, *gmin, *gmax, *trff1, *trff2, *cosne1, *cosne2;
} RelTable;

typedef struct {
  int n_a, n_h, n_rad;
  float *a;
  float *h;       /* [ia][n_h] */
  float *rad;     /* [ia][n_rad] */
  float *intens;  /* [ia][ih][n_rad] */
  float *del;
  float *del_inc;
} LpTable;

typedef struct {
  int n_ener, num_param, n_incl;
  float *elo, *ehi;
  int num_param_vals[6];
  int param_index[6];
  float *param_vals[6];
  float *incl;
  long num_elements;
  float **data;  /* lazily loaded spectra, renormalised (xilltable.c:478-511) */
  fitsfile *fp;
} XillTable;

static char g_table_path[1024] = ".";
static RelTable *g_rel = NULL;
static LpTable *g_lp = NULL;
static XillTable *g_xill = NULL;

static void fullpath(char *out, const char *name) { snprintf(out, 2048, "%s/%s", g_table_path, name); }

/* read_relline_table, reltable.c:235-311 */
static RelTable *load_rel_table(void) {
  char path[2048];
  fullpath(path, "rel_table_v0.5a.fits");
  int st = 0;
  fitsfile *fp = NULL;
  if (fits_open_table(&fp, path, READONLY, &st)) return NULL;
  RelTable *t = calloc(1, sizeof(RelTable));
  int col;
  long n;
  fits_movnam_hdu(fp, BINARY_TBL, "a", 0, &st);
  fits_get_colnum(fp, CASEINSEN, "a", &col, &st);
  fits_get_num_rows(fp, &n, &st);
  t->n_a = (int) n;
  t->a = malloc(sizeof(float) * n);
  fits_read_col(fp, TFLOAT, col, 1, 1, n, NULL, t->a, NULL, &st);
  fits_movnam_hdu(fp, BINARY_TBL, "mu0", 0, &st);
  fits_get_colnum(fp, CASEINSEN, "mu0", &col, &st);
  fits_get_num_rows(fp, &n, &st);
  t->n_mu0 = (int) n;
  t->mu0 = malloc(sizeof(float) * n);
  fits_read_col(fp, TFLOAT, col, 1, 1, n, NULL, t->mu0, NULL, &st);
  /* dimensions of one extension */
  int ext;
  fits_movabs_hdu(fp, 4, &ext, &st);
  fits_get_num_rows(fp, &n, &st);
  t->n_r = (int) n;
  {
    /* n_g from the vector column width: read trff1 of row 1 via column metadata */
    int ct;
    fits_get_colnum(fp, CASEINSEN, "trff1", &ct, &st);
    /* count elements: try reading until the row boundary (n_g <= 4096) */
    float tmp[4096];
    int ng = 0;
    for (ng = 1; ng <= 4096; ng++) {
      int s2 = 0;
      /* element ng of row n_r exists only if n_g >= ng */
      fits_read_col(fp, TFLOAT, ct, t->n_r, ng, 1, NULL, tmp, NULL, &s2);
      if (s2) break;
    }
    t->n_g = ng - 1;
  }
  int na = t->n_a, nm = t->n_mu0, nr = t->n_r, ng = t->n_g;
  size_t blk = (size_t) na * nm;
  t->r = malloc(sizeof(float) * blk * nr);
  t->gmin = malloc(sizeof(float) * blk * nr);
  t->gmax = malloc(sizeof(float) * blk * nr);
  t->trff1 = malloc(sizeof(float) * blk * nr * ng);
  t->trff2 = malloc(sizeof(float) * blk * nr * ng);
  t->cosne1 = malloc(sizeof(float) * blk * nr * ng);
  t->cosne2 = malloc(sizeof(float) * blk * nr * ng);
  for (int ii = 0; ii < na; ii++) {
    for (int jj = 0; jj < nm; jj++) {
      size_t b = (size_t) ii * nm + jj;
      fits_movabs_hdu(fp, ii * nm + jj + 4, &ext, &st);
      int cr, cmin, cmax, c1, c2, c3, c4;
      fits_get_colnum(fp, CASEINSEN, "r", &cr, &st);
      fits_get_colnum(fp, CASEINSEN, "gmin", &cmin, &st);
      fits_get_colnum(fp, CASEINSEN, "gmax", &cmax, &st);
      fits_get_colnum(fp, CASEINSEN, "trff1", &c1, &st);
      fits_get_colnum(fp, CASEINSEN, "trff2", &c2, &st);
      fits_get_colnum(fp, CASEINSEN, "cosne1", &c3, &st);
      fits_get_colnum(fp, CASEINSEN, "cosne2", &c4, &st);
      fits_read_col(fp, TFLOAT, cr, 1, 1, nr, NULL, t->r + b * nr, NULL, &st);
      fits_read_col(fp, TFLOAT, cmin, 1, 1, nr, NULL, t->gmin + b * nr, NULL, &st);
      fits_read_col(fp, TFLOAT, cmax, 1, 1, nr, NULL, t->gmax + b * nr, NULL, &st);
      fits_read_col(fp, TFLOAT, c1, 1, 1, (long long) nr * ng, NULL, t->trff1 + b * nr * ng, NULL, &st);
      fits_read_col(fp, TFLOAT, c2, 1, 1, (long long) nr * ng, NULL, t->trff2 + b * nr * ng, NULL, &st);
      fits_read_col(fp, TFLOAT, c3, 1, 1, (long long) nr * ng, NULL, t->cosne1 + b * nr * ng, NULL, &st);
      fits_read_col(fp, TFLOAT, c4, 1, 1, (long long) nr * ng, NULL, t->cosne2 + b * nr * ng, NULL, &st);
    }
  }
  fits_close_file(fp, &st);
  if (st) { free(t); return NULL; }
  return t;
}

/* read_lp_table, reltable.c:313-448 (del, del_inc are stored as fabsf, :370-377) */
static LpTable *load_lp_table(void) {
  char path[2048];
  fullpath(path, "rel_lp_table_v0.5b.fits");
  int st = 0;
  fitsfile *fp = NULL;
  if (fits_open_table(&fp, path, READONLY, &st)) return NULL;
  fits_movnam_hdu(fp, BINARY_TBL, "I_h", 0, &st);
  LpTable *t = calloc(1, sizeof(LpTable));
  long n;
  int ca, ch, cr;
  fits_get_num_rows(fp, &n, &st);
  t->n_a = (int) n;
  fits_get_colnum(fp, CASEINSEN, "a", &ca, &st);
  fits_get_colnum(fp, CASEINSEN, "hgrid", &ch, &st);
  fits_get_colnum(fp, CASEINSEN, "r", &cr, &st);
  t->a = malloc(sizeof(float) * n);
  fits_read_col(fp, TFLOAT, ca, 1, 1, n, NULL, t->a, NULL, &st);
  /* n_h and n_rad: count the h# columns and the r vector length */
  int nh = 0;
  for (;;) {
    char name[32];
    int c, s2 = 0;
    snprintf(name, sizeof name, "h%d", nh + 1);
    if (fits_get_colnum(fp, CASEINSEN, name, &c, &s2)) break;
    nh++;
  }
  t->n_h = nh;
  {
    float tmp[1];
    int nrd;
    for (nrd = 1; nrd <= 100000; nrd++) {
      int s2 = 0;
      fits_read_col(fp, TFLOAT, cr, t->n_a, nrd, 1, NULL, tmp, NULL, &s2);
      if (s2) break;
    }
    t->n_rad = nrd - 1;
  }
  int na = t->n_a, nrad = t->n_rad;
  t->h = malloc(sizeof(float) * na * nh);
  t->rad = malloc(sizeof(float) * na * nrad);
  t->intens = malloc(sizeof(float) * (size_t) na * nh * nrad);
  t->del = malloc(sizeof(float) * (size_t) na * nh * nrad);
  t->del_inc = malloc(sizeof(float) * (size_t) na * nh * nrad);
  for (int ia = 0; ia < na; ia++) {
    fits_read_col(fp, TFLOAT, ch, ia + 1, 1, nh, NULL, t->h + ia * nh, NULL, &st);
    fits_read_col(fp, TFLOAT, cr, ia + 1, 1, nrad, NULL, t->rad + ia * nrad, NULL, &st);
    for (int k = 0; k < nh; k++) {
      char name[32];
      int c;
      size_t off = ((size_t) ia * nh + k) * nrad;
      snprintf(name, sizeof name, "h%d", k + 1);
      fits_get_colnum(fp, CASEINSEN, name, &c, &st);
      fits_read_col(fp, TFLOAT, c, ia + 1, 1, nrad, NULL, t->intens + off, NULL, &st);
      snprintf(name, sizeof name, "del%d", k + 1);
      fits_get_colnum(fp, CASEINSEN, name, &c, &st);
      fits_read_col(fp, TFLOAT, c, ia + 1, 1, nrad, NULL, t->del + off, NULL, &st);
      snprintf(name, sizeof name, "del_inc%d", k + 1);
      fits_get_colnum(fp, CASEINSEN, name, &c, &st);
      fits_read_col(fp, TFLOAT, c, ia + 1, 1, nrad, NULL, t->del_inc + off, NULL, &st);
      for (int q = 0; q < nrad; q++) {
        t->del[off + q] = fabsf(t->del[off + q]);
        t->del_inc[off + q] = fabsf(t->del_inc[off + q]);
      }
    }
  }
  fits_close_file(fp, &st);
  if (st) { free(t); return NULL; }
  return t;
}

static const char *g_xill_names[] = {"Gamma", "A_Fe", "logXi", "Ecut", "kTe", "Dens", "kTbb", "A_CO", "Frac", "Incl"};
static const int g_xill_index[] = {PARAM_GAM, PARAM_AFE, PARAM_LXI, PARAM_ECT, PARAM_ECT, PARAM_DNS, 5, PARAM_AFE, 6,
                                   PARAM_INC};

/* init_xillver_table, xilltable.c:169-276, 410-447: 5-parameter tables, and the 6-parameter
 * nthcomp table (xillverCp_v3.4.fits, common.h:166) */
static XillTable *load_xill_table_file(const char *fname) {
  char path[2048];
  fullpath(path, fname);
  int st = 0;
  fitsfile *fp = NULL;
  if (fits_open_table(&fp, path, READONLY, &st)) return NULL;
  XillTable *t = calloc(1, sizeof(XillTable));
  long n;
  fits_get_num_rows(fp, &n, &st);  /* first table = PARAMETERS */
  t->num_param = (int) n;
  if (t->num_param != 5 && t->num_param != 6) { fits_close_file(fp, &st); free(t); return NULL; }
  fits_movnam_hdu(fp, BINARY_TBL, "ENERGIES", 0, &st);
  fits_get_num_rows(fp, &n, &st);
  t->n_ener = (int) n;
  t->elo = malloc(sizeof(float) * n);
  t->ehi = malloc(sizeof(float) * n);
  fits_read_col(fp, TFLOAT, 1, 1, 1, n, NULL, t->elo, NULL, &st);
  fits_read_col(fp, TFLOAT, 2, 1, 1, n, NULL, t->ehi, NULL, &st);
  fits_movnam_hdu(fp, BINARY_TBL, "PARAMETERS", 0, &st);
  char names[6][16];
  char *pn[6];
  for (int i = 0; i < 6; i++) pn[i] = names[i];
  fits_read_col(fp, TINT, 9, 1, 1, t->num_param, NULL, t->num_param_vals, NULL, &st);
  fits_read_col(fp, TSTRING, 1, 1, 1, t->num_param, NULL, pn, NULL, &st);
  for (int i = 0; i < t->num_param; i++) {
    t->param_vals[i] = malloc(sizeof(float) * t->num_param_vals[i]);
    fits_read_col(fp, TFLOAT, 10, i + 1, 1, t->num_param_vals[i], NULL, t->param_vals[i], NULL, &st);
    t->param_index[i] = -1;
    for (int j = 0; j < 10; j++)
      if (strcmp(names[i], g_xill_names[j]) == 0) t->param_index[i] = g_xill_index[j];
    if (t->param_index[i] < 0) st = 1;
  }
  t->incl = t->param_vals[t->num_param - 1];
  t->n_incl = t->num_param_vals[t->num_param - 1];
  t->num_elements = 1;
  for (int i = 0; i < t->num_param; i++) t->num_elements *= t->num_param_vals[i];
  t->data = calloc(t->num_elements, sizeof(float *));
  fits_movnam_hdu(fp, BINARY_TBL, "SPECTRA", 0, &st);
  t->fp = fp;
  if (st) return NULL;
  return t;
}

static XillTable *load_xill_table(void) { return load_xill_table_file("xillver-a-Ec5.fits"); }

/* get_xillspec_rownum, xilltable.c:325-337 (1-based row): idx holds one index per table parameter */
static long xill_rownum_idx(const XillTable *t, const int *idx) {
  long row = 0;
  for (int q = 0; q < t->num_param; q++) row = row * t->num_param_vals[q] + idx[q];
  return row + 1;
}

static int xilltab_param_index(const XillTable *t, int ind) {
  for (int i = 0; i < t->num_param; i++)
    if (t->param_index[i] == ind) return i;
  return -1;
}

/* xilltable_fits_load_single_spec + normalizeXillverSpecLogxiDensity + renorm_xill_spec
 * (xilltable.c:478-564).  The stored spectrum is divided by 10^logXi of its
 * grid point (float storage).  For a table without a density parameter the
 * reference also divides by 10^(dens-15) with the density of the zone that
 * loads the row first, and keeps that row in its cache; an evaluation in a
 * process with an empty cache therefore scales every row with the density of
 * the first zone (in zone order) that uses it.  That is the rule restated
 * here: eval_dens[row] remembers the first zone's density within one call. */
static double *g_eval_dens = NULL;
static long g_eval_dens_n = 0;
static float *g_dens_buf = NULL;

static void xill_begin_eval(XillTable *t) {
  if (g_eval_dens_n < t->num_elements) {
    free(g_eval_dens);
    g_eval_dens = malloc(sizeof(double) * t->num_elements);
    g_eval_dens_n = t->num_elements;
  }
  for (long i = 0; i < t->num_elements; i++) g_eval_dens[i] = NAN;
}

/* idx: one index per table parameter.  A table with a density parameter divides its rows by
 * 10^(logN - 15) of the row's grid point as well (renorm_xill_spec, xilltable.c:478-485). */
static const float *xill_spec_idx(XillTable *t, const int *idx, double zone_dens, float *buf) {
  long row = xill_rownum_idx(t, idx);
  const int ind_dns = xilltab_param_index(t, PARAM_DNS);
  if (t->data[row - 1] == NULL) {
    float *spec = malloc(sizeof(float) * t->n_ener);
    int st = 0;
    fits_read_col(t->fp, TFLOAT, 2, row, 1, t->n_ener, NULL, spec, NULL, &st);
    if (st) { free(spec); return NULL; }
    int ind_lxi = xilltab_param_index(t, PARAM_LXI);
    double logxi = 0.0;
    if (ind_lxi >= 0) logxi = t->param_vals[ind_lxi][idx[ind_lxi]];
    const double dens_row = ind_dns >= 0 ? t->param_vals[ind_dns][idx[ind_dns]] : 15.0;
    for (int i = 0; i < t->n_ener; i++) {
      spec[i] /= pow(10, logxi);
      if (fabs(dens_row - 15) > 1e-6) spec[i] /= pow(10, dens_row - 15);
    }
    t->data[row - 1] = spec;
  }
  if (ind_dns >= 0) return t->data[row - 1];
  if (g_eval_dens[row - 1] != g_eval_dens[row - 1]) g_eval_dens[row - 1] = zone_dens;
  double dens = g_eval_dens[row - 1];
  if (!(fabs(dens - 15) > 1e-6)) return t->data[row - 1];
  const float *src = t->data[row - 1];
  for (int i = 0; i < t->n_ener; i++) {
    buf[i] = src[i];
    buf[i] /= pow(10, dens - 15);
  }
  return buf;
}

static const float *xill_spec(XillTable *t, int ii, int jj, int kk, int ll, int mm, double zone_dens, float *buf) {
  const int idx[5] = {ii, jj, kk, ll, mm};
  return xill_spec_idx(t, idx, zone_dens, buf);
}

static XillTable *g_xill_cp = NULL;

static int ensure_tables(int need_xill, int need_cp) {
  if (!g_rel) g_rel = load_rel_table();
  if (!g_lp) g_lp = load_lp_table();
  if (need_xill && !g_xill) g_xill = load_xill_table();
  if (need_cp && !g_xill_cp) g_xill_cp = load_xill_table_file("xillverCp_v3.4.fits");
  return (g_rel && g_lp && (!need_xill || g_xill) && (!need_cp || g_xill_cp)) ? 0 : 1;
}

/* ======================================================================= */
/* system parameters: interpol_relTable (Relprofile.cpp:141-303)           */
/* ======================================================================= */

typedef struct {
  int nr, ng;
  double re[N_FRAD], gmin[N_FRAD], gmax[N_FRAD];
  double *trff;   /* [nr][ng][2] */
  double *cosne;  /* [nr][ng][2] */
  double *gstar, *d_gstar;
  /* emissivity profile (emisProfile, common.h:288-300) */
  double emis[N_FRAD], del_emit[N_FRAD], del_inc[N_FRAD];
  double refl_frac, f_bh, f_ad, f_inf, f_inf_rest;
  int limb_law;
} SysPar;

static void free_syspar(SysPar *s) {
  if (!s) return;
  free(s->trff);
  free(s->cosne);
  free(s->gstar);
  free(s->d_gstar);
  free(s);
}

static int interpol_rel_table(const RelTable *tab, double a, double incl, double rin, double rout, SysPar *sp) {
  int na = tab->n_a, nm = tab->n_mu0, nr = tab->n_r, ng = tab->n_g;
  double mu0 = cos(incl);
  int ind_a = binary_search_float(tab->a, na, (float) a);
  int ind_mu0 = binary_search_float(tab->mu0, nm, (float) mu0);
  float ifac_a = ((float) a - tab->a[ind_a]) / (tab->a[ind_a + 1] - tab->a[ind_a]);
  float ifac_mu0 = ((float) mu0 - tab->mu0[ind_mu0]) / (tab->mu0[ind_mu0 + 1] - tab->mu0[ind_mu0]);
  size_t b00 = ((size_t) ind_a * nm + ind_mu0), b10 = ((size_t) (ind_a + 1) * nm + ind_mu0);
  size_t b01 = ((size_t) ind_a * nm + ind_mu0 + 1), b11 = ((size_t) (ind_a + 1) * nm + ind_mu0 + 1);
  double *re_tab = malloc(sizeof(double) * nr);
  double *gmin_t = malloc(sizeof(double) * nr), *gmax_t = malloc(sizeof(double) * nr);
  double *trff_t = malloc(sizeof(double) * nr * ng * 2), *cosne_t = malloc(sizeof(double) * nr * ng * 2);
  for (int ii = 0; ii < nr; ii++) re_tab[ii] = interp_lin_1d(ifac_a, tab->r[b00 * nr + ii], tab->r[b10 * nr + ii]);
  if ((re_tab[nr - 1] > relxo_kerr_rms(a)) && ((re_tab[nr - 1] - relxo_kerr_rms(a)) / re_tab[nr - 1] < 1e-3))
    re_tab[nr - 1] = relxo_kerr_rms(a);
  int ind_rmin = inv_binary_search(re_tab, nr, rin);
  int ind_rmax = inv_binary_search(re_tab, nr, rout);
  /* interpol_a_mu0 for every table radius (the condition at :211 covers all radii) */
  for (int ii = 0; ii < nr; ii++) {
#define C4(arr, i) (arr)[b00 * nr + (i)], (arr)[b10 * nr + (i)], (arr)[b01 * nr + (i)], (arr)[b11 * nr + (i)]
    gmin_t[ii] = interp_lin_2d(ifac_a, ifac_mu0, C4(tab->gmin, ii));
    gmax_t[ii] = interp_lin_2d(ifac_a, ifac_mu0, C4(tab->gmax, ii));
#undef C4
#define G4(arr) (arr)[(b00 * nr + ii) * ng + jj], (arr)[(b10 * nr + ii) * ng + jj], \
                (arr)[(b01 * nr + ii) * ng + jj], (arr)[(b11 * nr + ii) * ng + jj]
    for (int jj = 0; jj < ng; jj++) {
      trff_t[(ii * ng + jj) * 2 + 0] = interp_lin_2d(ifac_a, ifac_mu0, G4(tab->trff1));
      trff_t[(ii * ng + jj) * 2 + 1] = interp_lin_2d(ifac_a, ifac_mu0, G4(tab->trff2));
      cosne_t[(ii * ng + jj) * 2 + 0] = interp_lin_2d(ifac_a, ifac_mu0, G4(tab->cosne1));
      cosne_t[(ii * ng + jj) * 2 + 1] = interp_lin_2d(ifac_a, ifac_mu0, G4(tab->cosne2));
    }
#undef G4
  }
  sp->nr = N_FRAD;
  sp->ng = ng;
  sp->trff = malloc(sizeof(double) * N_FRAD * ng * 2);
  sp->cosne = malloc(sizeof(double) * N_FRAD * ng * 2);
  sp->gstar = malloc(sizeof(double) * ng);
  sp->d_gstar = malloc(sizeof(double) * ng);
  /* new_relSysPar, Relprofile.cpp:104-116 */
  for (int ii = 0; ii < ng; ii++) sp->gstar[ii] = GFAC_H + (1.0 - 2 * GFAC_H) / (ng - 1) * ((float) (ii));
  for (int ii = 0; ii < ng; ii++) {
    if (ii == 0 || ii == ng - 1) sp->d_gstar[ii] = 0.5 * (sp->gstar[1] - sp->gstar[0]) + GFAC_H;
    else sp->d_gstar[ii] = sp->gstar[1] - sp->gstar[0];
  }
  get_fine_radial_grid(rin, rout, sp->re, N_FRAD);
  if (re_tab[ind_rmax] < 1000.0 && re_tab[ind_rmax] * 1.01 > 1000.0) re_tab[ind_rmax] = 1000.0;
  int status = 0;
  int ind_tabr = ind_rmin;
  for (int ii = N_FRAD - 1; ii >= 0; ii--) {
    while (sp->re[ii] >= re_tab[ind_tabr]) {
      ind_tabr--;
      if (ind_tabr < 0) {
        if (sp->re[ii] - RELTABLE_MAX_R <= 1e-6) { ind_tabr = 0; break; }
        status = 1;
        break;
      }
    }
    if (status) break;
    double ifac_r = (sp->re[ii] - re_tab[ind_tabr + 1]) / (re_tab[ind_tabr] - re_tab[ind_tabr + 1]);
    if (ifac_r > 1.0 && ind_tabr > 0) { status = 1; break; }
    for (int jj = 0; jj < ng; jj++) {
      for (int kk = 0; kk < 2; kk++) {
        sp->trff[(ii * ng + jj) * 2 + kk] = interp_lin_1d(ifac_r, trff_t[((ind_tabr + 1) * ng + jj) * 2 + kk],
                                                          trff_t[(ind_tabr * ng + jj) * 2 + kk]);
        sp->cosne[(ii * ng + jj) * 2 + kk] = interp_lin_1d(ifac_r, cosne_t[((ind_tabr + 1) * ng + jj) * 2 + kk],
                                                           cosne_t[(ind_tabr * ng + jj) * 2 + kk]);
      }
    }
    sp->gmin[ii] = interp_lin_1d(ifac_r, gmin_t[ind_tabr + 1], gmin_t[ind_tabr]);
    sp->gmax[ii] = interp_lin_1d(ifac_r, gmax_t[ind_tabr + 1], gmax_t[ind_tabr]);
  }
  free(re_tab);
  free(gmin_t);
  free(gmax_t);
  free(trff_t);
  free(cosne_t);
  return status;
}

/* ======================================================================= */
/* emissivity (Rellp.cpp)                                                   */
/* ======================================================================= */

/* norm_emis_profile, Rellp.cpp:91-109 (descending grid) */
static void norm_emis_profile(const double *re, int nr, double *emis) {
  double integ_area = 0.0;
  for (int ii = 0; ii < nr; ii++) integ_area += emis[ii] * (trapez_integ_single(re, ii, nr) * 2);
  for (int ii = 0; ii < nr; ii++) emis[ii] /= integ_area;
}

/* get_emis_bkn, Rellp.cpp:421-437 */
static void get_emis_bkn(double *emis, const double *re, int nr, double index1, double index2, double rbr) {
  for (int ii = 0; ii < nr; ii++) {
    double alpha = index1;
    if (re[ii] > rbr) alpha = index2;
    emis[ii] = pow(re[ii] / rbr, -alpha);
  }
  norm_emis_profile(re, nr, emis);
}

/* calc_emis_jet_point_source, Rellp.cpp:120-285 */
static int emis_lamp_post(const LpTable *tab, const Params *p, SysPar *sp) {
  int nrad = tab->n_rad, nh = tab->n_h, nr = sp->nr;
  int ind_a;
  double ifac_a;
  get_ipol_factor((float) p->a, tab->a, tab->n_a, &ind_a, &ifac_a);
  const float *rad0 = tab->rad + (size_t) ind_a * nrad, *rad1 = tab->rad + (size_t) (ind_a + 1) * nrad;
  double *jet_rad = malloc(sizeof(double) * nrad);
  double *e_tab = malloc(sizeof(double) * nrad), *d_tab = malloc(sizeof(double) * nrad),
         *di_tab = malloc(sizeof(double) * nrad);
  for (int ii = 0; ii < nrad; ii++) jet_rad[ii] = interp_lin_1d(ifac_a, rad0[ii], rad1[ii]);
  int ind_h[2];
  double ifac_h[2];
  for (int q = 0; q < 2; q++)
    get_ipol_factor((float) p->height, tab->h + (size_t) (ind_a + q) * nh, nh, &ind_h[q], &ifac_h[q]);
  /* interpol_emisprofile_spin_height, Rellp.cpp:190-210 */
  for (int ii = 0; ii < nrad; ii++) {
#define TV(arr, q, k) (arr)[(((size_t) (ind_a + (q)) * nh) + (k)) * nrad + ii]
    e_tab[ii] = (1.0 - ifac_a) * interp_lin_1d(ifac_h[0], TV(tab->intens, 0, ind_h[0]), TV(tab->intens, 0, ind_h[0] + 1))
        + (ifac_a) * interp_lin_1d(ifac_h[1], TV(tab->intens, 1, ind_h[1]), TV(tab->intens, 1, ind_h[1] + 1));
    d_tab[ii] = (1.0 - ifac_a) * interp_lin_1d(ifac_h[0], TV(tab->del, 0, ind_h[0]), TV(tab->del, 0, ind_h[0] + 1))
        + (ifac_a) * interp_lin_1d(ifac_h[1], TV(tab->del, 1, ind_h[1]), TV(tab->del, 1, ind_h[1] + 1));
    di_tab[ii] = (1.0 - ifac_a)
        * interp_lin_1d(ifac_h[0], TV(tab->del_inc, 0, ind_h[0]), TV(tab->del_inc, 0, ind_h[0] + 1))
        + (ifac_a) * interp_lin_1d(ifac_h[1], TV(tab->del_inc, 1, ind_h[1]), TV(tab->del_inc, 1, ind_h[1] + 1));
#undef TV
  }
  /* rebin_emisprofile_on_radial_grid, Rellp.cpp:120-175 */
  int status = 0;
  int kk = binary_search(jet_rad, nrad, sp->re[nr - 1]);
  for (int ii = nr - 1; ii >= 0; ii--) {
    while (sp->re[ii] >= jet_rad[kk + 1]) {
      kk++;
      if (kk >= nrad - 1) {
        if (sp->re[ii] - RELTABLE_MAX_R <= 1e-6) { kk = nrad - 2; break; }
        status = 1;
        break;
      }
    }
    if (status) break;
    double inter_r = get_ipol_factor_radius(jet_rad[kk], jet_rad[kk + 1], d_tab[kk], sp->re[ii]);
    sp->emis[ii] = interp_log_1d(inter_r, e_tab[kk], e_tab[kk + 1]);
    sp->del_emit[ii] = interp_lin_1d(inter_r, d_tab[kk], d_tab[kk + 1]);
    sp->del_inc[ii] = interp_lin_1d(inter_r, di_tab[kk], di_tab[kk + 1]);
  }
  /* calc_refl_frac, Rellp.cpp:36-89 */
  double del_emit_ad_max = d_tab[nrad - 1];
  double del_bh = sp->del_emit[inv_binary_search(sp->re, nr, p->rin)];
  double del_ad = sp->del_emit[inv_binary_search(sp->re, nr, p->rout)];
  if (del_emit_ad_max < M_PI / 2.0) del_emit_ad_max = M_PI / 2.0;
  if (p->beta > 1e-6) {
    del_bh = relat_abberation(del_bh, -1. * p->beta);
    del_ad = relat_abberation(del_ad, -1. * p->beta);
  }
  sp->f_bh = 0.5 * (1.0 - cos(del_bh));
  sp->f_ad = 0.5 * (cos(del_bh) - cos(del_ad));
  sp->f_inf_rest = 0.5 * (1.0 + cos(del_emit_ad_max));
  if (p->beta > 1e-6) sp->f_inf = 0.5 * (1.0 + cos(relat_abberation(del_emit_ad_max, -1. * p->beta)));
  else sp->f_inf = sp->f_inf_rest;
  sp->refl_frac = sp->f_ad / sp->f_inf;
  /* apply_emis_fluxboost_source_disk, Rellp.cpp:249-253; Relphysics.cpp:301-311 */
  for (int ii = 0; ii < nr; ii++) {
    double boost = pow(relxo_gi_potential_lp(sp->re[ii], p->a, p->height, p->beta, sp->del_emit[ii]), p->gamma);
    if (p->beta > 1e-6) boost *= pow(doppler_factor(sp->del_emit[ii], p->beta), 2);
    sp->emis[ii] *= boost;
  }
  free(jet_rad);
  free(e_tab);
  free(d_tab);
  free(di_tab);
  return status;
}

/* ======================================================================= */
/* returning radiation (Relreturn_Table.cpp, Relreturn_Corona.cpp)          */
/* ======================================================================= */

#define RRAD_NR 50  /* RETURNRAD_TABLE_NR / _NG, common.h:127-128 */
#define RRAD_NG 20

/* one spin of the table (tabulatedReturnFractions, Relreturn_Datastruct.h): row = incident bin,
 * column = emitting bin */
typedef struct {
  double rlo[RRAD_NR], rhi[RRAD_NR];
  double tf_r[RRAD_NR][RRAD_NR], gmin[RRAD_NR][RRAD_NR], gmax[RRAD_NR][RRAD_NR];
  double frac_g[RRAD_NR][RRAD_NR][RRAD_NG];
} RradFrac;

typedef struct {
  int nspin;
  double *spin;
  RradFrac *frac;
} RradTable;

static RradTable *g_rrad = NULL;

/* fits_read_returnRadTable / fits_rr_load_single_fractions, Relreturn_Table.cpp:180-330 */
static RradTable *load_rrad_table(void) {
  char path[2048];
  fullpath(path, "table_returnRad_v20220301.fits");
  int st = 0;
  fitsfile *fp = NULL;
  if (fits_open_table(&fp, path, READONLY, &st)) return NULL;
  RradTable *t = calloc(1, sizeof(RradTable));
  long n = 0;
  int c = 0;
  fits_movnam_hdu(fp, BINARY_TBL, "SPIN", 0, &st);
  fits_get_num_rows(fp, &n, &st);
  fits_get_colnum(fp, CASEINSEN, "a", &c, &st);
  if (!st && n > 0 && n <= 99) {
    t->nspin = (int) n;
    t->spin = malloc(sizeof(double) * n);
    t->frac = calloc(n, sizeof(RradFrac));
    fits_read_col(fp, TDOUBLE, c, 1, 1, n, NULL, t->spin, NULL, &st);
  } else {
    st = 1;
  }
  for (int k = 0; k < t->nspin && !st; k++) {
    char ext[16];
    snprintf(ext, sizeof ext, "FRAC%02d", k + 1);
    fits_movnam_hdu(fp, BINARY_TBL, ext, 0, &st);
    long nr = 0;
    fits_get_num_rows(fp, &nr, &st);
    if (st || nr != RRAD_NR) { st = 1; break; }
    RradFrac *f = &t->frac[k];
    const char *names[6] = {"rlo", "rhi", "tf_r", "gmin", "gmax", "frac_g"};
    double *dst[6] = {f->rlo, f->rhi, &f->tf_r[0][0], &f->gmin[0][0], &f->gmax[0][0], &f->frac_g[0][0][0]};
    const long cnt[6] = {RRAD_NR, RRAD_NR, RRAD_NR * RRAD_NR, RRAD_NR * RRAD_NR, RRAD_NR * RRAD_NR,
                         (long) RRAD_NR * RRAD_NR * RRAD_NG};
    for (int q = 0; q < 6 && !st; q++) {
      fits_get_colnum(fp, CASEINSEN, names[q], &c, &st);
      fits_read_col(fp, TDOUBLE, c, 1, 1, cnt[q], NULL, dst[q], NULL, &st);
    }
  }
  fits_close_file(fp, &st);
  if (st) {
    free(t->spin);
    free(t->frac);
    free(t);
    return NULL;
  }
  return t;
}

/* returningFractions (Relreturn_Datastruct.h) on the radial range of a model */
typedef struct {
  const RradFrac *tab;
  int nrad;
  int irad[RRAD_NR];
  double rlo[RRAD_NR], rhi[RRAD_NR], rad[RRAD_NR];
  double tf_r[RRAD_NR][RRAD_NR];
} RradFractions;

/* rradCorrFactors (common.h:182-189): per ionisation zone */
typedef struct {
  int n_zones;
  double rgrid[N_ZONES_MAX + 1];
  double corrfac_flux[N_ZONES_MAX], corrfac_gshift[N_ZONES_MAX];
} RradCorr;

/* get_ring_area_correction_factor, Relreturn_Table.cpp:518-538 */
static double rrad_area_correction(const RradFractions *rf, int idx, double a) {
  double rlo_table = rf->tab->rlo[rf->irad[idx]];
  if (rf->irad[idx] == 0 && rlo_table > relxo_kerr_rms(a)) rlo_table = relxo_kerr_rms(a);
  double rhi_table = rf->tab->rhi[rf->irad[idx]];
  double area_table = 0.5 * (rlo_table + rhi_table) * (rhi_table - rlo_table);
  double area_model = 0.5 * (rf->rlo[idx] + rf->rhi[idx]) * (rf->rhi[idx] - rf->rlo[idx]);
  return area_model / area_table;
}

/* get_rrad_fractions: select_spinIndexForTable, allocate_radial_grid, get_interpolated_tfr
 * (Relreturn_Table.cpp:393-611) */
static int get_rrad_fractions(double a, double rin, double rout, RradFractions *rf) {
  const RradTable *t = g_rrad;
  int k = binary_search(t->spin, t->nspin, a);
  if (t->spin[k] < a) k++;
  if (k >= t->nspin || k < 0) return 1;
  const RradFrac *tab = &t->frac[k];
  rf->tab = tab;
  int klo = binary_search(tab->rlo, RRAD_NR, rin);
  int khi = binary_search(tab->rhi, RRAD_NR, rout);
  if (fabs(rout - tab->rhi[RRAD_NR - 1]) < 1e-6) khi = RRAD_NR - 1;
  else khi++;
  if (fabs(rin - tab->rlo[0]) < 1e-6) klo = 0;
  int n = (khi + 1) - klo;
  if (n <= 0 || n > RRAD_NR) return 1;
  rf->nrad = n;
  for (int ii = 0; ii < n; ii++) {
    rf->irad[ii] = klo + ii;
    rf->rlo[ii] = tab->rlo[rf->irad[ii]];
    rf->rhi[ii] = tab->rhi[rf->irad[ii]];
  }
  if (!(rin >= rf->rlo[0] - 1e-4)) return 1;
  rf->rlo[0] = rin;
  rf->rhi[n - 1] = rout;
  for (int ii = 0; ii < n; ii++) rf->rad[ii] = 0.5 * (rf->rlo[ii] + rf->rhi[ii]);
  for (int ii = 0; ii < n; ii++)
    for (int jj = 0; jj < n; jj++) rf->tf_r[ii][jj] = tab->tf_r[rf->irad[ii]][rf->irad[jj]];
  const double corr_rin = rrad_area_correction(rf, 0, a);
  const double corr_rout = rrad_area_correction(rf, n - 1, a);
  if (!(corr_rin - 1 < 1e-6) || !(corr_rout - 1 < 1e-6)) return 1;
  for (int ii = 0; ii < n - 1; ii++) rf->tf_r[ii][0] *= corr_rin;
  for (int ii = 0; ii < n - 2; ii++) rf->tf_r[ii][n - 1] *= corr_rout;
  return 0;
}

/* corrected_gshift_fluxboost_factor, Relreturn_Corona.cpp:37-86 */
static double corrected_gshift_fluxboost_factor(double xill_gshift_fac, double g, double gamma) {
  const double g0 = 2. / 3;
  double gshift_corr_factor;
  if (xill_gshift_fac < 1) {
    double a = (xill_gshift_fac / g0 - 1) / (g0 - 1);
    double b = 1 - a;
    gshift_corr_factor = (g >= 1) ? 1. / g * (1. / g * a + b) : g * (g * a + b);
  } else {
    double alin = (xill_gshift_fac - 1) / (g0 - 1);
    double blin = 1 - alin;
    gshift_corr_factor = (g >= 1) ? (1. / g * alin + blin) : (g * alin + blin);
  }
  double fluxboost_factor = pow(g, gamma) * gshift_corr_factor;
  if (g < 1 && fluxboost_factor > 1) fluxboost_factor = 1;
  if (fluxboost_factor < 0) fluxboost_factor = 0;
  return fluxboost_factor;
}

/* calc_rrad_emis_zone + get_gfac_grid, Relreturn_Corona.cpp:103-123, Relreturn_Datastruct.cpp:51-59 */
static double rrad_emis_zone(const RradFrac *tab, int ro, int re, double gamma, double corrfac_gshift) {
  double emis_zone = 0.0;
  for (int jj = 0; jj < RRAD_NG; jj++) {
    const double g = (jj + 0.5) / RRAD_NG * (tab->gmax[ro][re] - tab->gmin[ro][re]) + tab->gmin[ro][re];
    double e = tab->frac_g[ro][re][jj];
    if (fabs(corrfac_gshift - 1) > 1e-3) e *= corrected_gshift_fluxboost_factor(corrfac_gshift, g, gamma) / g;
    else if (fabs(g - 1) > 1e-3) e *= pow(g, gamma - 1);
    emis_zone += e;
  }
  return emis_zone;
}

/* rebin_to_grid, Relreturn_Corona.cpp:208-222 */
static void rrad_rebin_to_grid(double *value, const double *rmean, int nzones, const double *rgrid0,
                               const double *value0, int n0) {
  for (int ii = 0; ii < nzones; ii++) {
    int ind = binary_search(rgrid0, n0 + 1, rmean[ii]);
    if (rmean[ii] < rgrid0[0]) ind = 0;
    else if (rmean[ii] > rgrid0[n0]) ind = n0 - 1;  /* the reference reads value0[n0] here; never reached */
    value[ii] = value0[ind];
  }
}

/* get_rrad_emis_corona + calc_rrad_emis_corona + rebin_emisprofile_on_radial_grid
 * (Relreturn_Corona.cpp:125-160, 271-321; Rellp.cpp:120-175): the returning-radiation
 * emissivity on the fine grid of sp from the direct emissivity sp->emis */
static int get_rrad_emis_corona(const SysPar *sp, const Params *p, const RradCorr *corr, double *emis_ret) {
  const int nr = sp->nr;
  RradFractions rf;
  if (get_rrad_fractions(p->a, sp->re[nr - 1], sp->re[0], &rf)) return 1;
  const int n = rf.nrad;
  double emis_in[RRAD_NR], cf_flux[RRAD_NR], cf_g[RRAD_NR], er[RRAD_NR], single[RRAD_NR];
  if (inv_rebin_mean(sp->re, sp->emis, nr, rf.rad, emis_in, n)) return 1;
  if (corr) {
    rrad_rebin_to_grid(cf_flux, rf.rad, n, corr->rgrid, corr->corrfac_flux, corr->n_zones);
    rrad_rebin_to_grid(cf_g, rf.rad, n, corr->rgrid, corr->corrfac_gshift, corr->n_zones);
  }
  for (int ii = 0; ii < n; ii++) {
    const int ro = rf.irad[ii];
    for (int jj = 0; jj < n; jj++) {
      const double cg = corr ? cf_g[jj] : 1.0;
      single[jj] = rrad_emis_zone(rf.tab, ro, rf.irad[jj], p->gamma, cg) * rf.tf_r[ii][jj] * emis_in[jj];
    }
    double sum = 0.0;
    for (int jj = 0; jj < n; jj++) sum += single[jj];
    er[ii] = sum;
    if (corr) er[ii] *= cf_flux[ii];
  }
  /* onto the fine grid (descending); the table profile has del_emit = 0, so the radial
   * interpolation factor is linear (get_ipol_factor_radius) */
  if (n < 2) return 1;
  int kk = binary_search(rf.rad, n, sp->re[nr - 1]);
  for (int ii = nr - 1; ii >= 0; ii--) {
    while (sp->re[ii] >= rf.rad[kk + 1]) {
      kk++;
      if (kk >= n - 1) {
        if (sp->re[ii] - RELTABLE_MAX_R <= 1e-6) { kk = n - 2; break; }
        return 1;
      }
    }
    const double inter = get_ipol_factor_radius(rf.rad[kk], rf.rad[kk + 1], 0.0, sp->re[ii]);
    emis_ret[ii] = interp_log_1d(inter, er[kk], er[kk + 1]);
  }
  return 0;
}

/* add_returnrad_emis, Rellp.cpp:483-509 */
static int add_returnrad_emis(const Params *p, const RradCorr *corr, SysPar *sp) {
  if (!g_rrad) g_rrad = load_rrad_table();
  if (!g_rrad) return 1;
  double *er = malloc(sizeof(double) * sp->nr);
  int status = get_rrad_emis_corona(sp, p, corr, er);
  for (int ii = 0; ii < sp->nr && !status; ii++) {
    if (p->return_rad == 1) sp->emis[ii] += er[ii];
    else if (p->return_rad == -1 || p->return_rad == 2) sp->emis[ii] = er[ii];
    else status = 1;
  }
  free(er);
  return status;
}

/* get_system_parameters, Relprofile.cpp:310-358 (without the cache); corr: the returning-radiation
 * correction factors (Relxill.cpp:337-344) or NULL */
static SysPar *get_system_parameters(const Params *p, const RradCorr *corr, int *status) {
  SysPar *sp = calloc(1, sizeof(SysPar));
  if (interpol_rel_table(g_rel, p->a, p->incl, p->rin, p->rout, sp)) { *status = 1; return sp; }
  sp->limb_law = p->limb;
  if (p->emis_type == EMIS_TYPE_BKN) {
    get_emis_bkn(sp->emis, sp->re, sp->nr, p->emis1, p->emis2, p->rbr);
    for (int ii = 0; ii < sp->nr; ii++) sp->del_emit[ii] = sp->del_inc[ii] = -1.0;
  } else {
    if (emis_lamp_post(g_lp, p, sp)) *status = 1;
  }
  /* calc_emis_profile, Rellp.cpp:556-558 */
  if (!*status && abs(p->return_rad) > 1e-6 && add_returnrad_emis(p, corr, sp)) *status = 1;
  return sp;
}

/* ======================================================================= */
/* line profile (Relprofile.cpp:476-958)                                    */
/* ======================================================================= */

typedef struct {
  double re, gmin, gmax, del_g, emis;
  int limb_law, ng;
  const double *trff, *cosne, *gstar;  /* [ng][2] at this radius */
} RelbFunc;

/* evaluations of relb_func since the last reset (the algorithmic work of the line profile) */
static long long g_relb_calls = 0;
long long relxo_relb_calls(int reset) {
  const long long n = g_relb_calls;
  if (reset) g_relb_calls = 0;
  return n;
}

/* relb_func, Relprofile.cpp:489-521 */
static double relb_func(double eg, int k, const RelbFunc *s) {
  g_relb_calls++;
  double egstar = (eg - s->gmin) * s->del_g;
  int ind = binary_search(s->gstar, s->ng, egstar);
  double inte = (egstar - s->gstar[ind]) / (s->gstar[ind + 1] - s->gstar[ind]);
  double inte1 = 1.0 - inte;
  double ftrf = inte * s->trff[ind * 2 + k] + inte1 * s->trff[(ind + 1) * 2 + k];
  double val = pow(eg, 3) / ((s->gmax - s->gmin) * sqrt(egstar - egstar * egstar)) * ftrf * s->emis;
  if (s->limb_law == 0) return val;
  double fmu0 = inte * s->cosne[ind * 2 + k] + inte1 * s->cosne[(ind + 1) * 2 + k];
  double limb = 1.0;
  if (s->limb_law == 1) limb = (1.0 + 2.06 * fmu0);
  else if (s->limb_law == 2) limb = log(1.0 + 1.0 / fmu0);
  return val * limb;
}

/* romberg_integration, Relprofile.cpp:524-579 (the end-point cache of the
 * reference never hits: cache_bin_ener stays -1, so f(a) is always evaluated) */
static double romberg_integration(double a, double b, int k, const RelbFunc *s) {
  const double prec = 0.02;
  double obtprec = 1.0;
  const int itermin = 0;
  int itermax = 5;
  enum { maxiter = 6 };
  double t[maxiter + 1][maxiter + 1];
  int niter = 0;
  double r = relb_func(a, k, s);
  double rb = relb_func(b, k, s);
  double ta = (r + rb) / 2.0;
  double pas = b - a;
  double pasm = 1.0;
  t[0][0] = ta * pas;
  while ((niter < itermin) || ((obtprec > prec) && (niter <= itermax))) {
    niter++;
    pas = pas / 2.0;
    pasm = pasm / 2.0;
    double sum = ta;
    for (int ii = 1; ii <= pow(2, niter) - 1; ii++) sum += relb_func(a + pas * ii, k, s);
    t[0][niter] = sum * pas;
    r = 1.0;
    for (int ii = 1; ii <= niter; ii++) {
      r *= 4.0;
      int jj = niter - ii;
      t[ii][jj] = (r * t[ii - 1][jj + 1] - t[ii - 1][jj]) / (r - 1.0);
    }
    obtprec = fabs(t[niter][0] - t[niter - 1][0]) / t[niter][0];
  }
  return t[niter][0];
}

/* int_edge, Relprofile.cpp:585-621 */
static double int_edge(double blo, double bhi, double h, const RelbFunc *s, double line_energy) {
  double hex, lo, hi;
  if (blo <= 0.5) { hex = h; lo = blo; hi = bhi; }
  else { hex = 1.0 - h; lo = 1.0 - bhi; hi = 1.0 - blo; }
  double norm = 0.0;
  for (int k = 0; k < 2; k++) norm = norm + relb_func(gstar2ener(hex, s->gmin, s->gmax, line_energy), k, s);
  norm = norm * sqrt(h);
  return 2 * norm * (sqrt(hi) - sqrt(lo)) * line_energy * (s->gmax - s->gmin);
}

/* int_romb, Relprofile.cpp:628-647 */
static double int_romb(double lo, double hi, const RelbFunc *s, double line_energy) {
  double flu = 0.0;
  if (lo >= line_energy * 0.95) {
    for (int k = 0; k < 2; k++) flu += romberg_integration(lo, hi, k, s);
  } else {
    for (int k = 0; k < 2; k++) flu += relb_func((hi + lo) / 2.0, k, s) * (hi - lo);
  }
  return flu;
}

/* integ_relline_bin, Relprofile.cpp:650-726 */
static double integ_relline_bin(const RelbFunc *s, double rlo0, double rhi0) {
  double line_ener = 1.0, flu = 0.0;
  double gblo = (rlo0 / line_ener - s->gmin) * s->del_g;
  if (gblo < 0.0) gblo = 0.0; else if (gblo > 1.0) gblo = 1.0;
  double gbhi = (rhi0 / line_ener - s->gmin) * s->del_g;
  if (gbhi < 0.0) gbhi = 0.0; else if (gbhi > 1.0) gbhi = 1.0;
  if (gbhi == 0) return 0.0;
  double rlo = rlo0, rhi = rhi0, hlo, hhi;
  if (gblo <= GFAC_H) {
    hlo = gblo;
    hhi = GFAC_H;
    rlo = gstar2ener(GFAC_H, s->gmin, s->gmax, line_ener);
    if (gbhi <= GFAC_H) { hhi = gbhi; rlo = -1.0; }
    flu = flu + int_edge(hlo, hhi, GFAC_H, s, line_ener);
  }
  if (gbhi >= (1.0 - GFAC_H)) {
    hhi = gbhi;
    hlo = 1.0 - GFAC_H;
    rhi = gstar2ener(1 - GFAC_H, s->gmin, s->gmax, line_ener);
    if (gblo >= (1.0 - GFAC_H)) { hlo = gblo; rhi = -1.0; }
    flu = flu + int_edge(hlo, hhi, GFAC_H, s, line_ener);
  }
  if ((rhi >= 0) && (rlo >= 0)) flu = flu + int_romb(rlo, rhi, s, line_ener);
  return flu;
}

/* get_cosne_bin, Relprofile.cpp:799-801 */
static int get_cosne_bin(double mu, int n_cosne) { return ((int) (n_cosne * (1 - mu) + 1)) - 1; }

/* calc_relline_profile (Relprofile.cpp:835-958) + renorm_relline_profile
 * (:749-796).  flux[nzones][n_ener]; dist[nzones][n_incl] when n_incl > 0. */
static int relline_profile(const SysPar *sp, const Params *p, const double *ener, int n_ener, int nzones,
                           const double *rgrid, double *flux, int n_incl, double *dist) {
  memset(flux, 0, sizeof(double) * nzones * n_ener);
  if (n_incl > 0) memset(dist, 0, sizeof(double) * nzones * n_incl);
  int status = 0;
  for (int ii = 0; ii < sp->nr; ii++) {
    double egmin = sp->gmin[ii], egmax = sp->gmax[ii];
    if ((egmax > ener[0]) && (egmin < ener[n_ener])) {
      if (egmin < ener[0]) egmin = ener[0];
      if (egmax > ener[n_ener]) egmax = ener[n_ener];
      int ielo = binary_search(ener, n_ener + 1, egmin);
      int iehi = binary_search(ener, n_ener + 1, egmax);
      int izone = binary_search(rgrid, nzones + 1, sp->re[ii]);
      RelbFunc s;
      s.re = sp->re[ii];
      s.gmin = sp->gmin[ii];
      s.gmax = sp->gmax[ii];
      s.del_g = 1. / (s.gmax - s.gmin);
      s.emis = sp->emis[ii];
      s.trff = sp->trff + (size_t) ii * sp->ng * 2;
      s.cosne = sp->cosne + (size_t) ii * sp->ng * 2;
      s.gstar = sp->gstar;
      s.ng = sp->ng;
      s.limb_law = sp->limb_law;
      double weight = trapez_integ_single(sp->re, ii, sp->nr) / 2;
      for (int jj = ielo; jj <= iehi; jj++)
        flux[izone * n_ener + jj] += integ_relline_bin(&s, ener[jj], ener[jj + 1]) * weight;
      if (n_incl > 0) {
        for (int jj = 0; jj < sp->ng; jj++) {
          double g = s.gstar[jj] * (s.gmax - s.gmin) + s.gmin;
          for (int kk = 0; kk < 2; kk++) {
            int imu = get_cosne_bin(s.cosne[jj * 2 + kk], n_incl);
            double tmp = s.re * pow(2 * M_PI * g * s.re, 2) / sqrt(s.gstar[jj] - s.gstar[jj] * s.gstar[jj])
                * s.trff[jj * 2 + kk] * s.emis * weight * sp->d_gstar[jj];
            if (tmp != tmp) status = 1;
            dist[izone * n_incl + imu] += tmp;
          }
        }
      }
    }
  }
  /* renorm_relline_profile */
  double sum = 0.0;
  for (int ii = 0; ii < nzones; ii++) {
    for (int jj = 0; jj < n_ener; jj++) {
      flux[ii * n_ener + jj] /= 0.5 * (ener[jj] + ener[jj + 1]);
      sum += flux[ii * n_ener + jj];
    }
  }
  if (do_renorm_model(p)) {
    double relline_norm = 1;
    if (p->is_relxill && p->emis_type == EMIS_TYPE_BKN) relline_norm = 0.5 * cos(p->incl * 180.0 / M_PI * M_PI / 180);
    for (int ii = 0; ii < nzones; ii++)
      for (int jj = 0; jj < n_ener; jj++) flux[ii * n_ener + jj] *= relline_norm / sum;
  }
  if (n_incl > 0) {
    for (int ii = 0; ii < nzones; ii++) {
      double s2 = 0.0;
      for (int jj = 0; jj < n_incl; jj++) s2 += dist[ii * n_incl + jj];
      if (!(s2 > 1e-8)) status = 1;
      for (int jj = 0; jj < n_incl; jj++) dist[ii * n_incl + jj] /= s2;
    }
  }
  return status;
}

/* ======================================================================= */
/* convolution (Relbase.cpp:93-230)                                         */
/* ======================================================================= */

/* fftw_conv_spectrum + normalizeFFTOutput (Relbase.cpp:119-222) */
static void conv_spectrum_normalized(const double *ener, const double *fxill, const double *frel, double *fout,
                                     int n) {
  double *cf = malloc(sizeof(double) * n);
  for (int ii = 0; ii < n; ii++) cf[ii] = 0.5 * (ener[ii] + ener[ii + 1]) / (ener[ii + 1] - ener[ii]);
  int pos1 = binary_search(ener, n + 1, 1.0);
  double *x = malloc(sizeof(double) * n), *r = malloc(sizeof(double) * n), *o = malloc(sizeof(double) * n);
  fftw_complex *X = malloc(sizeof(fftw_complex) * n), *R = malloc(sizeof(fftw_complex) * n),
               *P = malloc(sizeof(fftw_complex) * n);
  for (int ii = 0; ii < n; ii++) x[ii] = fxill[ii] * cf[ii];
  for (int ii = 0; ii < n; ii++) r[(ii - pos1 + n) % n] = frel[ii] * cf[ii];
  fftw_plan px = fftw_plan_dft_r2c_1d(n, x, X, FFTW_ESTIMATE);
  fftw_execute(px);
  fftw_destroy_plan(px);
  fftw_plan pr = fftw_plan_dft_r2c_1d(n, r, R, FFTW_ESTIMATE);
  fftw_execute(pr);
  fftw_destroy_plan(pr);
  for (int ii = 0; ii <= n / 2; ii++) {
    P[ii][0] = X[ii][0] * R[ii][0] - X[ii][1] * R[ii][1];
    P[ii][1] = X[ii][0] * R[ii][1] + X[ii][1] * R[ii][0];
  }
  fftw_plan pc = fftw_plan_dft_c2r_1d(n, P, o, FFTW_ESTIMATE);
  fftw_execute(pc);
  fftw_destroy_plan(pc);
  for (int ii = 0; ii < n; ii++) fout[ii] = o[ii] / cf[ii];
  /* calcFFTNormFactor, Relbase.cpp:199-213 */
  double sr = 0.0, sx = 0.0, sc = 0.0;
  for (int jj = 0; jj < n; jj++) {
    if (ener[jj] >= EMIN_XILLVER && ener[jj + 1] < EMAX_XILLVER) {
      sx += fxill[jj];
      sr += frel[jj];
      sc += fout[jj];
    }
  }
  double norm_fac = sr * sx / sc;
  for (int ii = 0; ii < n; ii++) fout[ii] *= norm_fac;
  free(cf); free(x); free(r); free(o); free(X); free(R); free(P);
}

void relxo_conv_spectrum_normalized(const double *ener, const double *fxill, const double *frel, double *fout,
                                    int n) {
  conv_spectrum_normalized(ener, fxill, frel, fout, n);
}

/* ======================================================================= */
/* xillver spectra and the primary continuum (Xillspec.cpp, xilltable.c)   */
/* ======================================================================= */

/* spec_cutoffpl, Xillspec.cpp:215-233 */
static void spec_cutoffpl(double *pl, const double *ener, int n, double ect, double gamma, double ener_shift) {
  double ecut = ect * ener_shift;
  for (int ii = 0; ii < n; ii++) {
    double en = 0.5 * (ener[ii] + ener[ii + 1]);
    pl[ii] = exp(1.0 / ecut) * pow(en, -gamma) * exp(-en / ecut) * (ener[ii + 1] - ener[ii]);
  }
}

/* calcNormWrtXillverTableSpec, Xillspec.cpp:179-205 */
double relxo_norm_wrt_xillver(const double *flux, const double *ener, int n) {
  double keV2erg = 1.602177e-09;
  double sum_pl = 0.0;
  for (int ii = 0; ii < n; ii++) {
    if (ener[ii] >= EMIN_XILLVER_NORMALIZATION && ener[ii] <= EMAX_XILLVER_NORMALIZATION)
      sum_pl += flux[ii] * 0.5 * (ener[ii] + ener[ii + 1]) * 1e20 * keV2erg;
  }
  double norm_xillver_table = 1e15 / 4.0 / M_PI;
  return sum_pl / norm_xillver_table;
}

static double g_coarse[N_ENER_COARSE + 1];
static int g_coarse_init = 0;
static const double *coarse_grid(void) {
  if (!g_coarse_init) {
    get_log_grid(g_coarse, N_ENER_COARSE + 1, EMIN_XILLVER_NORMALIZATION, EMAX_XILLVER_NORMALIZATION);
    g_coarse_init = 1;
  }
  return g_coarse;
}

/* 1/calcNormWrtXillverTableSpec of the cut-off power law on the coarse grid */
/* ----------------------------------------------------------------------- */
/* nthcomp (donthcomp.c): thermal Comptonization of disk-blackbody seed     */
/* photons, the Kompaneets equation with relativistic corrections solved on */
/* a logarithmic grid (Lightman & Zdziarski 1987; Zdziarski, Johnson &     */
/* Magdziarz 1996; Zycki, Done & Smith 1999).  Restated for the parameters  */
/* the Cp models pass (get_nthcomp_param, relutility.c:625-631): seed      */
/* temperature 0.05 keV, disk-blackbody seed (inp_type 1).                  */
/* ----------------------------------------------------------------------- */

#define NTH_LOG10E 0.43429448190325182765
static double nth_lg10(double x) { return NTH_LOG10E * log(x); }

/* multi-colour disk spectrum integrand (Mitsuda et al. 1984, Makishima et al. 1986; interpolation
 * formula with residual table, donthcomp.c:52-103) */
static double nth_mcdint(double et) {
  static const double gc[3] = {.078196667, -1.066202, 1.192418};
  static const double gw[3] = {.5207874, .513457, .4077983};
  static const double gn[3] = {.3728691, .039775528, .037766505};
  static const double res[98] = {
      9.6198382e-4, .0010901181, .0012310012, .0013841352, .0015481583, .0017210036, .0018988943, .002076939,
      .0022484281, .0024049483, .0025366202, .0026316255, .0026774985, .0026613059, .0025708784, .0023962965,
      .002130655, .0017725174, .0013268656, 8.0657672e-4, 2.3337584e-4, -3.6291778e-4, -9.4443569e-4, -.0014678875,
      -.0018873741, -.0021588493, -.0022448371, -.0021198179, -.0017754602, -.0012246034, -5.0414167e-4,
      3.2507078e-4, .0011811065, .0019673402, .0025827094, .0029342526, .0029517083, .0026012166, .0018959062,
      9.0128649e-4, -2.6757144e-4, -.0014567885, -.002492855, -.0032079776, -.0034678637, -.0031988217,
      -.0024080969, -.001193624, 2.6134145e-4, .0017117758, .0028906898, .0035614435, .0035711778, .0028921374,
      .0016385898, 4.9857464e-5, -.0015572671, -.0028578151, -.0035924212, -.0036253044, -.002975086,
      -.0018044436, -3.7796664e-4, .0010076215, .0020937327, .0027090854, .0028031667, .0024276576, .0017175597,
      8.1030795e-4, -1.2592304e-4, -9.4888491e-4, -.0015544816, -.0018831972, -.0019203142, -.0016905849,
      -.0012487737, -6.6789911e-4, -2.7079461e-5, 5.9931935e-4, .0011499748, .0015816521, .0018709224,
      .0020129966, .0020184702, .0019089181, .0017122289, .001458377, .0011760717, 8.9046768e-4, 6.2190822e-4,
      3.8553762e-4, 1.9155022e-4, 4.5837109e-5, -4.9177834e-5, -9.3670762e-5, -8.9622968e-5, -4.01538532e-5};
  const double loget = nth_lg10(et);
  const double lo = 0.001;
  double pos = (loget - nth_lg10(lo)) / .06 + 1;
  const int j = (int) pos;
  double resfact;
  if (j < 1) {
    resfact = res[0];
  } else if (j >= 98) {
    resfact = res[97];
  } else {
    pos -= j;
    resfact = res[j - 1] * (1. - pos) + res[j] * pos;
  }
  double gaufact = 1.;
  for (int k = 0; k < 3; k++) {
    const double zz = (loget - gc[k]) / gw[k];
    gaufact += gn[k] * exp(-zz * zz / 2.);
  }
  const double et0 = et / .001;
  return pow(et0, -.66666666666666663) * 193.21556 * (pow(et, 1.663753) * .52876731 + 1.) * exp(-et) * gaufact *
         (resfact + 1.);
}

/* disk-blackbody photon spectrum per bin, five-point Gauss-Legendre per bin (donthcomp.c:137-191):
 * ear[0..ne], photar[0..ne-1] */
static void nth_diskbb(const double *ear, int ne, double tin, double *photar) {
  static const double gw5[5] = {.236926885, .47862867, .568888888, .47862867, .236926885};
  static const double gx5[5] = {-.906179846, -.53846931, 0., .53846931, .906179846};
  for (int i = 1; i <= ne; i++) {
    const double xn = (ear[i] - ear[i - 1]) / 2.f;
    double acc = 0.f;
    const double xh = xn + ear[i - 1];
    for (int k = 0; k < 5; k++) {
      const double e = xn * gx5[k] + xh;
      double photon = 0.;
      if (tin != 0.) photon = nth_mcdint(e / tin) * tin * tin * 1. / 361.;
      acc += (double) (gw5[k] * photon);
    }
    photar[i - 1] = acc * xn;
  }
}

/* Kompaneets equation as a tridiagonal system a u(j+1) + b u(j) + c u(j-1) = d, zero flux at both
 * ends (donthcomp.c:194-280).  x and dphesc are indexed j = 1..jmax (x up to jmax + 1); c2, bet and
 * dphdot hold the value of point j at j - 1. */
static void nth_solve(double tautom, double theta, double deltal, const double *x, int jmax, double *dphesc,
                      const double *dphdot, const double *bet, const double *c2) {
  double a[900], b[900], c[900], d[900], g[900], u[900], gam[900], alp[900];
  const double c20 = tautom / deltal;
  for (int j = 2; j <= jmax - 1; j++) {
    const double w1 = sqrt(x[j] * x[j + 1]), w2 = sqrt(x[j - 1] * x[j]);
    a[j - 1] = -c20 * c2[j - 1] * (theta / deltal / w1 + .5);
    const double t1 = -c20 * c2[j - 1] * (.5 - theta / deltal / w1);
    const double t2 = c20 * c2[j - 2] * (theta / deltal / w2 + .5);
    const double t3 = pow(x[j], 3.) * (tautom * bet[j - 1]);
    b[j - 1] = t1 + t2 + t3;
    c[j - 1] = c20 * c2[j - 2] * (.5 - theta / deltal / w2);
    d[j - 1] = x[j] * dphdot[j - 1];
  }
  const double x32 = sqrt(x[1] * x[2]);
  const double aa = (theta / deltal / x32 + .5) / (theta / deltal / x32 - .5);
  u[jmax - 1] = 0.;
  alp[1] = b[1] + c[1] * aa;
  gam[1] = a[1] / alp[1];
  for (int j = 3; j <= jmax - 1; j++) {
    alp[j - 1] = b[j - 1] - c[j - 1] * gam[j - 2];
    gam[j - 1] = a[j - 1] / alp[j - 1];
  }
  g[1] = d[1] / alp[1];
  for (int j = 3; j <= jmax - 2; j++) g[j - 1] = (d[j - 1] - c[j - 1] * g[j - 2]) / alp[j - 1];
  g[jmax - 2] = (d[jmax - 2] - a[jmax - 2] * u[jmax - 1] - c[jmax - 2] * g[jmax - 3]) / alp[jmax - 2];
  u[jmax - 2] = g[jmax - 2];
  for (int j = 3; j <= jmax - 1; j++) {
    const int jj = jmax + 1 - j;
    u[jj - 1] = g[jj - 1] - gam[jj - 1] * u[jj];
  }
  u[0] = aa * u[1];
  for (int j = 1; j <= jmax; j++) dphesc[j] = x[j] * x[j] * u[j - 1] * bet[j - 1] * tautom;
}

/* Comptonized disk-blackbody spectrum in E F_E on the grid x (units of m_e c^2): x[1..jmax + 1],
 * sptot[1..jmax - 1] (donthcomp.c:458-616) */
static int nth_thdscompton(double tempbb, double theta, double gamma, double *x, double *sptot) {
  double c2[901], rel[900], bet[901], dphdot[901], dphesc[901], ear[5001], photar[5000];
  double d1 = gamma + .5;
  const double tautom = sqrt(3. / (theta * (d1 * d1 - 2.25)) + 2.25) - 1.5;
  for (int j = 0; j < 900; j++) {
    dphesc[j] = dphdot[j] = rel[j] = bet[j] = c2[j] = 0.;
    sptot[j + 1] = 0.;
  }
  const double delta = .02;
  const double deltal = delta * log(10.);
  const double xmin = tempbb * 1e-4, xmax = theta * 40.;
  int jmax = (int) (nth_lg10(xmax / xmin) / delta) + 1;
  if (jmax > 899) jmax = 899;
  for (int j = 1; j <= jmax + 1; j++) x[j] = xmin * pow(10., (j - 1) * delta);
  for (int j = 1; j <= jmax; j++) {
    const double w = x[j], w1 = sqrt(x[j] * x[j + 1]);
    c2[j - 1] = (double) (pow(w1, 4.) / (w1 * 4.6 + 1. + w1 * 1.1 * w1));
    if (w <= .05) {
      rel[j - 1] = (double) (1 - w * 2 + w * 26 * w / 5);
    } else {
      const double z1 = (w + 1) / (w * (w * w)), z2 = w * 2 + 1, z3 = log(z2), z4 = w * 2 * (w + 1) / z2,
                   z5 = z3 / 2 / w, z6 = (w * 3 + 1) / z2 / z2;
      rel[j - 1] = (double) ((z1 * (z4 - z3) + z5 - z6) * .75);
    }
  }
  int jmaxth = (int) (nth_lg10(tempbb * 50. / xmin) / delta);
  if (jmaxth > 900) jmaxth = 900;
  if (jmaxth > jmax) jmaxth = jmax;
  for (int j = 1; j <= jmaxth - 1; j++) ear[j - 1] = sqrt(x[j] * x[j + 1]) * 511.;
  const int ne = jmaxth - 2;
  nth_diskbb(ear, ne, tempbb * 511., photar);
  for (int j = 1; j <= ne; j++) dphdot[j] = photar[j - 1] * 511. / (ear[j] - ear[j - 1]);
  dphdot[0] = dphdot[1];
  int jnr = (int) (nth_lg10(.1 / xmin) / delta + 1);
  if (jnr > jmax - 1) jnr = jmax - 1;
  int jrel = (int) (nth_lg10(1. / xmin) / delta + 1);
  if (jrel > jmax) jrel = jmax;
  const double xnr = x[jnr], xr = x[jrel];
  for (int j = 1; j <= jnr - 1; j++) {
    const double taukn = tautom * rel[j - 1];
    bet[j - 1] = 1 / tautom / (taukn / 3 + 1);
  }
  for (int j = jnr; j <= jrel; j++) {
    const double taukn = tautom * rel[j - 1];
    const double arg = (x[j] - xnr) / (xr - xnr);
    const double flz = 1 - arg;
    bet[j - 1] = 1 / tautom / (taukn / 3 * flz + 1);
  }
  for (int j = jrel + 1; j <= jmax; j++) bet[j - 1] = 1 / tautom;
  nth_solve(tautom, theta, deltal, x, jmax, dphesc, dphdot, bet, c2);
  for (int j = 1; j <= jmax - 1; j++) {
    const double xj = x[j];
    sptot[j] = dphesc[j] * (xj * xj);
  }
  return jmax;
}

/* c_donthcomp (donthcomp.c:640-793) with kTbb = 0.05 keV and the disk-blackbody seed: photon flux
 * per bin on ear[0..ne], normalised to 1 at 1 keV in E F_E (observer frame, redshift z) */
static void nthcomp_spectrum(const double *ear, int ne, double gamma, double kte, double z, double *photar) {
  double xth[901], spt[901];
  const int nth = nth_thdscompton(.05 / 511., kte / 511., gamma, xth, spt);
  /* xth[1..], spt[1..]: the reference's xth[j-1], spt[j-1] */
  const double xn = (z + 1) / 511.;
  const double xx = 1 / (1 / xn);
  int ih = 2;  /* f_spp__ (donthcomp.c:617-638): linear interpolation in E F_E */
  while (ih < nth && xx > xth[ih]) ++ih;
  const int il = ih - 1;
  const double spp = spt[il] + (spt[ih] - spt[il]) * (xx - xth[il]) / (xth[ih] - xth[il]);
  const double normfac = 1 / spp;
  double *prim = calloc(ne + 1, sizeof(double));
  int j = 1;
  for (int i = 0; i <= ne; i++) {
    while (j <= nth && xth[j] * 511. < ear[i] * (z + 1)) ++j;
    if (j <= nth) {
      if (j > 1) {
        const int jl = j - 1;
        prim[i] = spt[jl] + (ear[i] / 511. * (z + 1) - xth[jl]) * (spt[jl + 1] - spt[jl]) / (xth[jl + 1] - xth[jl]);
      } else {
        prim[i] = spt[1];
      }
    }
  }
  for (int i = 1; i <= ne; i++)
    photar[i - 1] = (prim[i] / pow(ear[i], 2.) + prim[i - 1] / pow(ear[i - 1], 2.)) * .5 * (ear[i] - ear[i - 1]) * normfac;
  free(prim);
}

void relxo_nthcomp(const double *ear, int ne, double gamma, double kte, double z, double *photar) {
  nthcomp_spectrum(ear, ne, gamma, kte, z, photar);
}

/* calc_primary_spectrum (Xillspec.cpp:274-300): cut-off power law or nthcomp, shifted by ener_shift */
#define PRIM_ECUT 0
#define PRIM_NTHCOMP 1
static void primary_spectrum(int prim_type, double *out, const double *ener, int n, double ect, double gam,
                             double ener_shift) {
  if (prim_type == PRIM_NTHCOMP) nthcomp_spectrum(ener, n, gam, ect, 1 / ener_shift - 1, out);
  else spec_cutoffpl(out, ener, n, ect, gam, ener_shift);
}

/* 1 / calcNormWrtXillverTableSpec of the source-frame primary on the coarse grid */
static double primary_norm_factor(int prim_type, double ect, double gam) {
  double pl[N_ENER_COARSE];
  primary_spectrum(prim_type, pl, coarse_grid(), N_ENER_COARSE, ect, gam, 1.0);
  return 1. / relxo_norm_wrt_xillver(pl, coarse_grid(), N_ENER_COARSE);
}

double relxo_primary_norm_factor(double ect, double gam) {
  double pl[N_ENER_COARSE];
  spec_cutoffpl(pl, coarse_grid(), N_ENER_COARSE, ect, gam, 1.0);
  return 1. / relxo_norm_wrt_xillver(pl, coarse_grid(), N_ENER_COARSE);
}

/* calc_xillver_normalization_change, Xillspec.cpp:373-397 */
double relxo_norm_change(double energy_shift, double ect, double gam) {
  double src = relxo_primary_norm_factor(ect, gam);
  double disk = relxo_primary_norm_factor(ect * energy_shift, gam);
  return disk / src;
}

/* get_xilltab_indices_for_paramvals + interp_xill_table + interp_5d_tab_incl
 * (xilltable.c:278-323, 812-876, 1054-1181) for relxill models (all incl) */
static int xillver_spectra_all_incl(XillTable *t, double gam, double afe, double lxi, double ect, double incl_deg,
                                    double dens, double *flu /* [n_incl][n_ener] */) {
  float inp[10] = {0};
  inp[PARAM_GAM] = (float) gam;
  inp[PARAM_AFE] = (float) afe;
  inp[PARAM_LXI] = (float) lxi;
  inp[PARAM_ECT] = (float) ect;
  inp[PARAM_DNS] = (float) dens;
  inp[PARAM_INC] = (float) incl_deg;
  const int np = t->num_param;
  int ind[6];
  for (int ii = 0; ii < np; ii++) {
    ind[ii] = binary_search_float(t->param_vals[ii], t->num_param_vals[ii], inp[t->param_index[ii]]);
    if (ind[ii] < 0) ind[ii] = 0;
    else if (ind[ii] > t->num_param_vals[ii] - 2) ind[ii] = t->num_param_vals[ii] - 2;
  }
  double ipol[6];
  for (int ii = 0; ii < np; ii++) {
    int pind = t->param_index[ii];
    if (pind != PARAM_INC) {  /* resetInpvalsToBoundaries, xilltable.c:1069-1088 */
      float lo = t->param_vals[ii][0], hi = t->param_vals[ii][t->num_param_vals[ii] - 1];
      if (inp[pind] < lo) inp[pind] = lo;
      else if (inp[pind] > hi) inp[pind] = hi;
    }
    ipol[ii] = (inp[pind] - t->param_vals[ii][ind[ii]]) / (t->param_vals[ii][ind[ii] + 1] - t->param_vals[ii][ind[ii]]);
  }
  /* ensure_ecut_within_boundarys, xilltable.c:1054-1067 */
  int iect = xilltab_param_index(t, PARAM_ECT);
  if (iect >= 0) {
    const float *ev = t->param_vals[t->param_index[iect]];
    if (ect <= ev[0]) ipol[iect] = 0.0;
    if (ect >= ev[t->num_param_vals[t->param_index[iect]] - 1]) ipol[iect] = 1.0;
  }
  /* 5 parameters: interp_5d_tab_incl over parameters 0..3; 6 parameters: interp_6d_tab_incl, the
   * same over parameters 1..4 at both brackets of parameter 0, then linear in parameter 0
   * (xilltable.c:812-876, 999-1020) */
  const int q0 = np - 5;  /* first parameter of the 16-corner block */
  const double f1 = ipol[q0], f2 = ipol[q0 + 1], f3 = ipol[q0 + 2], f4 = ipol[q0 + 3];
  const double fw[16] = {
      (1.0 - f1) * (1.0 - f2) * (1.0 - f3) * (1 - f4), (f1) * (1.0 - f2) * (1.0 - f3) * (1 - f4),
      (1.0 - f1) * (f2) * (1.0 - f3) * (1 - f4),       (1.0 - f1) * (1.0 - f2) * (f3) * (1 - f4),
      (f1) * (f2) * (1.0 - f3) * (1 - f4),             (f1) * (1.0 - f2) * (f3) * (1 - f4),
      (1.0 - f1) * (f2) * (f3) * (1 - f4),             (f1) * (f2) * (f3) * (1 - f4),
      (1.0 - f1) * (1.0 - f2) * (1.0 - f3) * (f4),     (f1) * (1.0 - f2) * (1.0 - f3) * (f4),
      (1.0 - f1) * (f2) * (1.0 - f3) * (f4),           (1.0 - f1) * (1.0 - f2) * (f3) * (f4),
      (f1) * (f2) * (1.0 - f3) * (f4),                 (f1) * (1.0 - f2) * (f3) * (f4),
      (1.0 - f1) * (f2) * (f3) * (f4),                 (f1) * (f2) * (f3) * (f4)};
  /* order of interp_5d_tab_incl, xilltable.c:816-834 */
  const int off[16][4] = {{0, 0, 0, 0}, {1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {1, 1, 0, 0}, {1, 0, 1, 0},
                          {0, 1, 1, 0}, {1, 1, 1, 0}, {0, 0, 0, 1}, {1, 0, 0, 1}, {0, 1, 0, 1}, {0, 0, 1, 1},
                          {1, 1, 0, 1}, {1, 0, 1, 1}, {0, 1, 1, 1}, {1, 1, 1, 1}};
  if (!g_dens_buf) g_dens_buf = malloc(sizeof(float) * 16 * t->n_ener);
  double *s1 = malloc(sizeof(double) * t->n_ener), *s2 = malloc(sizeof(double) * t->n_ener);
  int status = 0;
  for (int mm = 0; mm < t->n_incl && !status; mm++) {
    for (int half = 0; half < (np == 6 ? 2 : 1) && !status; half++) {
      const float *d[16];
      for (int c = 0; c < 16 && !status; c++) {
        int idx[6];
        if (np == 6) idx[0] = ind[0] + half;
        for (int q = 0; q < 4; q++) idx[q0 + q] = ind[q0 + q] + off[c][q];
        idx[np - 1] = mm;
        d[c] = xill_spec_idx(t, idx, dens, g_dens_buf + (size_t) c * t->n_ener);
        if (!d[c]) status = 1;
      }
      if (status) break;
      double *out = (np == 6) ? (half ? s2 : s1) : flu + (size_t) mm * t->n_ener;
      for (int ii = 0; ii < t->n_ener; ii++) {
        out[ii] = fw[0] * (double) (d[0][ii]) + fw[1] * (double) (d[1][ii]) + fw[2] * (double) (d[2][ii])
            + fw[3] * (double) (d[3][ii]) + fw[4] * (double) (d[4][ii]) + fw[5] * (double) (d[5][ii])
            + fw[6] * (double) (d[6][ii]) + fw[7] * (double) (d[7][ii]) + fw[8] * (double) (d[8][ii])
            + fw[9] * (double) (d[9][ii]) + fw[10] * (double) (d[10][ii]) + fw[11] * (double) (d[11][ii])
            + fw[12] * (double) (d[12][ii]) + fw[13] * (double) (d[13][ii]) + fw[14] * (double) (d[14][ii])
            + fw[15] * (double) (d[15][ii]);
      }
    }
    if (np == 6 && !status) {
      double *out = flu + (size_t) mm * t->n_ener;
      for (int ii = 0; ii < t->n_ener; ii++) out[ii] = interp_lin_1d(ipol[0], s1[ii], s2[ii]);
    }
  }
  free(s1);
  free(s2);
  return status;
}

/* get_xilltab_indices_for_paramvals + interp_xill_table + interp_5d_tab (xilltable.c:278-323,
 * 878-995, 1090-1181) for the xillver model: all five parameters, the inclination included,
 * are interpolated (32 corner spectra) */
static int xillver_spectrum_at_incl(XillTable *t, double gam, double afe, double lxi, double ect, double incl_deg,
                                    double dens, double *flu /* [n_ener] */) {
  float inp[10] = {0};
  inp[PARAM_GAM] = (float) gam;
  inp[PARAM_AFE] = (float) afe;
  inp[PARAM_LXI] = (float) lxi;
  inp[PARAM_ECT] = (float) ect;
  inp[PARAM_DNS] = (float) dens;
  inp[PARAM_INC] = (float) incl_deg;
  int ind[6];
  for (int ii = 0; ii < t->num_param; ii++) {
    ind[ii] = binary_search_float(t->param_vals[ii], t->num_param_vals[ii], inp[t->param_index[ii]]);
    if (ind[ii] < 0) ind[ii] = 0;
    else if (ind[ii] > t->num_param_vals[ii] - 2) ind[ii] = t->num_param_vals[ii] - 2;
  }
  double ipol[6];
  for (int ii = 0; ii < t->num_param; ii++) {
    int pind = t->param_index[ii];
    /* resetInpvalsToBoundaries (xilltable.c:1069-1088), the inclination included for xillver models */
    float lo = t->param_vals[ii][0], hi = t->param_vals[ii][t->num_param_vals[ii] - 1];
    if (inp[pind] < lo) inp[pind] = lo;
    else if (inp[pind] > hi) inp[pind] = hi;
    ipol[ii] = (inp[pind] - t->param_vals[ii][ind[ii]]) / (t->param_vals[ii][ind[ii] + 1] - t->param_vals[ii][ind[ii]]);
  }
  int iect = xilltab_param_index(t, PARAM_ECT);
  if (iect >= 0) {  /* ensure_ecut_within_boundarys, xilltable.c:1054-1067 */
    const float *ev = t->param_vals[t->param_index[iect]];
    if (ect <= ev[0]) ipol[iect] = 0.0;
    if (ect >= ev[t->num_param_vals[t->param_index[iect]] - 1]) ipol[iect] = 1.0;
  }
  /* 5 parameters: interp_5d_tab; 6 parameters: interp_6d_tab, the same over parameters 1..5 at both
   * brackets of parameter 0, then linear in parameter 0 (xilltable.c:878-995, 1022-1043) */
  const int np = t->num_param, q0 = np - 5;
  const double f1 = ipol[q0], f2 = ipol[q0 + 1], f3 = ipol[q0 + 2], f4 = ipol[q0 + 3], f5 = ipol[q0 + 4];
  /* the 32 corners in the order of interp_5d_tab's weights and sum (xilltable.c:884-992):
   * bits (c1 c2 c3 c4 c5) of the corner offsets */
  static const int corner[32][5] = {
      {0, 0, 0, 0, 0}, {1, 0, 0, 0, 0}, {0, 1, 0, 0, 0}, {0, 0, 1, 0, 0}, {1, 1, 0, 0, 0}, {1, 0, 1, 0, 0},
      {0, 1, 1, 0, 0}, {1, 1, 1, 0, 0}, {0, 0, 0, 1, 0}, {1, 0, 0, 1, 0}, {0, 1, 0, 1, 0}, {0, 0, 1, 1, 0},
      {1, 1, 0, 1, 0}, {1, 0, 1, 1, 0}, {0, 1, 1, 1, 0}, {1, 1, 1, 1, 0}, {0, 0, 0, 0, 1}, {1, 0, 0, 0, 1},
      {0, 1, 0, 0, 1}, {0, 0, 1, 0, 1}, {1, 1, 0, 0, 1}, {1, 0, 1, 0, 1}, {0, 1, 1, 0, 1}, {1, 1, 1, 0, 1},
      {0, 0, 0, 1, 1}, {1, 0, 0, 1, 1}, {0, 1, 0, 1, 1}, {0, 0, 1, 1, 1}, {1, 1, 0, 1, 1}, {1, 0, 1, 1, 1},
      {0, 1, 1, 1, 1}, {1, 1, 1, 1, 1}};
  double w[32];
  const float *d[32];
  float *buf = malloc(sizeof(float) * 32 * (size_t) t->n_ener);
  double *s1 = malloc(sizeof(double) * t->n_ener);
  for (int half = 0; half < (np == 6 ? 2 : 1); half++) {
    for (int c = 0; c < 32; c++) {
      const int *o = corner[c];
      w[c] = (o[0] ? f1 : (1.0 - f1)) * (o[1] ? f2 : (1.0 - f2)) * (o[2] ? f3 : (1.0 - f3)) *
             (o[3] ? f4 : (1 - f4)) * (o[4] ? f5 : (1 - f5));
      int idx[6];
      if (np == 6) idx[0] = ind[0] + half;
      for (int q = 0; q < 5; q++) idx[q0 + q] = ind[q0 + q] + o[q];
      d[c] = xill_spec_idx(t, idx, dens, buf + (size_t) c * t->n_ener);
      if (!d[c]) { free(buf); free(s1); return 1; }
    }
    double *out = (np == 6 && half == 0) ? s1 : flu;
    for (int ii = 0; ii < t->n_ener; ii++) {
      double acc = w[0] * (double) d[0][ii];
      for (int c = 1; c < 32; c++) acc = acc + w[c] * (double) d[c][ii];
      out[ii] = acc;
    }
  }
  if (np == 6)
    for (int ii = 0; ii < t->n_ener; ii++) flu[ii] = interp_lin_1d(ipol[0], s1[ii], flu[ii]);
  free(buf);
  free(s1);
  return 0;
}

/* ======================================================================= */
/* models                                                                   */
/* ======================================================================= */

static double g_conv[N_ENER_CONV + 1];
static int g_conv_init = 0;
static const double *conv_grid(void) {
  if (!g_conv_init) {
    get_log_grid(g_conv, N_ENER_CONV + 1, EMIN_RELXILL_CONV, EMAX_RELXILL_CONV);
    g_conv_init = 1;
  }
  return g_conv;
}

/* relbase (Relbase.cpp:524-538) for one zone on the grid ener */
static int relbase_single(const Params *p, const double *ener, int n, double *flux) {
  int status = 0;
  SysPar *sp = get_system_parameters(p, NULL, &status);
  if (!status) {
    double rgrid[2];
    get_rzone_grid(p->rin, p->rout, 1, p->height, rgrid);
    status = relline_profile(sp, p, ener, n, 1, rgrid, flux, 0, NULL);
  }
  free_syspar(sp);
  return status;
}

/* get_xillver_fluxcorrection_factors with calc_angle_averaged_xill_spec, get_xillver_fluxcorr and
 * get_xillver_gshift_fluxcorr (Xillspec.cpp:109-160, 344-361, 457-526) for one zone: flu holds the
 * zone's spectra per inclination on the xillver grid xener.  The reference weights inclination i
 * by norm_factor_semi_infinite_slab(incl_i * 180 / pi) / n_incl with incl_i the table value in
 * degrees, i.e. 0.5 cos(incl_i) with incl_i read as radians; restated as it is. */
static void xillver_fluxcorrection_factors(const XillTable *t, const double *flu, const double *xener, int prim_type,
                                           double ect_zone, double gam, double *fac_flux, double *fac_gshift) {
  const int n_x = t->n_ener, ni = t->n_incl;
  double *avg = calloc(n_x, sizeof(double)), *ener_z = malloc(sizeof(double) * (n_x + 1)),
         *flu_z = malloc(sizeof(double) * n_x);
  for (int ii = 0; ii < ni; ii++) {
    const double incl_deg = (double) t->incl[ii] * 180 / M_PI;
    const double incl_factor = 0.5 * cos(incl_deg * M_PI / 180) / ni;
    for (int jj = 0; jj < n_x; jj++) avg[jj] += incl_factor * flu[(size_t) ii * n_x + jj];
  }
  /* energy flux in 0.1-1000 keV of the reflection and of the normalised direct spectrum */
  double ef_refl = 0.0;
  for (int ii = 0; ii < n_x; ii++)
    if (xener[ii] >= 0.1 && xener[ii + 1] <= 1000) ef_refl += avg[ii] * 0.5 * (xener[ii] + xener[ii + 1]);
  const double *cg = coarse_grid();
  double direct[N_ENER_COARSE];
  primary_spectrum(prim_type, direct, cg, N_ENER_COARSE, ect_zone, gam, 1.0);
  const double nf = 1. / relxo_norm_wrt_xillver(direct, cg, N_ENER_COARSE);
  double ef_direct = 0.0;
  for (int ii = 0; ii < N_ENER_COARSE; ii++) {
    direct[ii] *= nf;
    if (cg[ii] >= 0.1 && cg[ii + 1] <= 1000) ef_direct += direct[ii] * 0.5 * (cg[ii] + cg[ii + 1]);
  }
  *fac_flux = ef_refl / ef_direct;
  /* photon flux in 0.15-500 keV unshifted and shifted by g = 2/3 */
  const double g0 = 2. / 3.;
  for (int ii = 0; ii <= n_x; ii++) ener_z[ii] = xener[ii] / g0;
  relxo_rebin_spectrum(ener_z, flu_z, n_x, xener, avg, n_x);
  for (int ii = 0; ii < n_x; ii++) flu_z[ii] *= g0;
  double pf = 0.0, pf_z = 0.0;
  for (int ii = 0; ii < n_x; ii++)
    if (xener[ii] >= 0.15 && xener[ii + 1] <= 500.0) pf += avg[ii];
  for (int ii = 0; ii < n_x; ii++)
    if (xener[ii] >= 0.15 && xener[ii + 1] <= 500.0) pf_z += flu_z[ii];
  *fac_gshift = (pf / pf_z) / pow(1.5, gam);
  free(avg);
  free(ener_z);
  free(flu_z);
}

/* relxill_kernel, Relxill.cpp:289-413, for relxill / relxilllp */
static int relxill_kernel(const Params *p, double *out_conv /* [N_ENER_CONV] */) {
  const double *ener = conv_grid();
  int status = 0;
  int nz = p->num_zones;
  SysPar *sp = get_system_parameters(p, NULL, &status);
  if (status) { free_syspar(sp); return status; }
  /* PrimarySourceParameters (PrimarySource.h:43-218) */
  double g_inf = 1.0;
  if (p->emis_type == EMIS_TYPE_LP) {
    g_inf = calc_g_inf(p->height, p->a);
    if (!(p->beta < 1e-4)) g_inf *= doppler_factor(M_PI - p->incl, p->beta);
  }
  double ect_source = p->ect;  /* the cut-off energy of the lamp post is given in the observer frame,
                                 kTe in the source frame (Relxill.cpp:220-230) */
  if (p->emis_type == EMIS_TYPE_LP && p->prim_type == PRIM_ECUT) ect_source /= g_inf;
  /* IonGradient (IonGradient.cpp:340-390, 457-492) */
  double rgrid[N_ZONES_MAX + 1], rmean[N_ZONES_MAX], del_emit[N_ZONES_MAX], shift[N_ZONES_MAX];
  double lxi[N_ZONES_MAX], dens[N_ZONES_MAX];
  get_rzone_grid(p->rin, p->rout, nz, p->height, rgrid);
  for (int ii = 0; ii < nz; ii++) {
    rmean[ii] = 0.5 * (rgrid[ii] + rgrid[ii + 1]);
    dens[ii] = 15.0;
    lxi[ii] = 0.0;
    shift[ii] = 1.0;
  }
  if (inv_rebin_mean(sp->re, sp->del_emit, sp->nr, rmean, del_emit, nz)) status = 1;
  for (int ii = 0; ii < nz; ii++)
    shift[ii] = (p->emis_type == EMIS_TYPE_LP) ? relxo_gi_potential_lp(rmean[ii], p->a, p->height, p->beta, del_emit[ii])
                                               : 1.0;
  if (p->ion_grad_type == ION_GRAD_TYPE_PL) {
    for (int ii = 0; ii < nz; ii++) {
      lxi[ii] = (exp(p->lxi)) * pow((rmean[ii] / rmean[0]), -1.0 * p->iongrad_index);
      lxi[ii] = log(lxi[ii]);
      dens[ii] = p->dens;
    }
  } else if (p->ion_grad_type == ION_GRAD_TYPE_ALPHA) {
    /* calc_ion_grad_alpha, IonGradient.cpp:128-171 */
    double rin = rgrid[0];
    double irr[N_ZONES_MAX], dinc[N_ZONES_MAX];
    if (inv_rebin_mean(sp->re, sp->emis, sp->nr, rmean, irr, nz)) status = 1;
    if (inv_rebin_mean(sp->re, sp->del_inc, sp->nr, rmean, dinc, nz)) status = 1;
    double rad_lxi = pow((11. / 9.), 2) * rin;
    int kk = inv_binary_search(sp->re, sp->nr, rad_lxi);
    double ip = (rad_lxi - sp->re[kk + 1]) / (sp->re[kk] - sp->re[kk + 1]);
    double emis_r = interp_lin_1d(ip, sp->emis[kk + 1], sp->emis[kk]);
    double dinc_r = interp_lin_1d(ip, sp->del_inc[kk + 1], sp->del_inc[kk]);
    double lxi_max = log10(4.0 * M_PI * emis_r / density_ss73_zone_a(rad_lxi, rin) * (cos(M_PI / 4) / cos(dinc_r)));
    double fac_lxi_norm = p->lxi - lxi_max;
    double density_min = density_ss73_zone_a((25. / 9.) * rin, rin);
    int const_dens = env_is_one("RELXILL_CONSTANT_DENSITY");
    for (int ii = 0; ii < nz; ii++) {
      double dn = 1.0;
      if (!const_dens) dn = density_ss73_zone_a(rmean[ii], rin) / density_min;
      dens[ii] = log10(dn) + p->dens;
      lxi[ii] = log10(4.0 * M_PI * irr[ii] / dn * (cos(M_PI / 4) / cos(dinc[ii])));
      lxi[ii] += fac_lxi_norm;
    }
  } else {
    for (int ii = 0; ii < nz; ii++) {
      lxi[ii] = p->lxi;
      dens[ii] = p->dens;
    }
  }
  for (int ii = 0; ii < nz; ii++) {
    if (lxi[ii] < 0.0) lxi[ii] = 0.0;
    else if (lxi[ii] > 4.7) lxi[ii] = 4.7;
  }
  XillTable *xt = (p->prim_type == PRIM_NTHCOMP) ? g_xill_cp : g_xill;
  int n_incl = xt->n_incl, n_x = xt->n_ener;
  double *xener = malloc(sizeof(double) * (n_x + 1));
  for (int ii = 0; ii < n_x; ii++) xener[ii] = xt->elo[ii];
  xener[n_x] = xt->ehi[n_x - 1];
  double *flu = malloc(sizeof(double) * n_incl * n_x);
  xill_begin_eval(xt);
  /* returning-radiation correction factors from the zones' xillver spectra, then the emissivity
   * again with them (Relxill.cpp:336-344; SPIN_MIN_RRAD_CALC_CORRFAC = 0, Relxill.h:32) */
  SysPar *sp_rel = sp;
  if (!status && p->return_rad != 0 && p->a > 0.0) {
    RradCorr corr;
    corr.n_zones = nz;
    for (int ii = 0; ii <= nz; ii++) corr.rgrid[ii] = rgrid[ii];
    for (int zz = 0; zz < nz && !status; zz++) {
      double ect_zone = ect_source * shift[zz];
      if (xillver_spectra_all_incl(xt, p->gam, p->afe, lxi[zz], ect_zone, p->incl * 180 / M_PI, dens[zz], flu)) {
        status = 1;
        break;
      }
      xillver_fluxcorrection_factors(xt, flu, xener, p->prim_type, ect_zone, p->gam, &corr.corrfac_flux[zz],
                                     &corr.corrfac_gshift[zz]);
    }
    if (!status) sp_rel = get_system_parameters(p, &corr, &status);
  }
  /* relline profile on the conv grid (Relbase.cpp:461-512 with xill_tab != NULL) */
  double *rel = malloc(sizeof(double) * nz * N_ENER_CONV);
  double *dist = malloc(sizeof(double) * nz * n_incl);
  if (!status) status = relline_profile(sp_rel, p, ener, N_ENER_CONV, nz, rgrid, rel, n_incl, dist);
  if (sp_rel != sp) free_syspar(sp_rel);
  /* xillver spectra per zone, angle weighted (Relxill.cpp:357-386) */
  double *xz = malloc(sizeof(double) * nz * n_x);
  double src_norm = primary_norm_factor(p->prim_type, ect_source, p->gam);
  for (int zz = 0; zz < nz && !status; zz++) {
    double ect_zone = ect_source * shift[zz];
    if (xillver_spectra_all_incl(xt, p->gam, p->afe, lxi[zz], ect_zone, p->incl * 180 / M_PI, dens[zz], flu)) {
      status = 1;
      break;
    }
    double *xf = xz + (size_t) zz * n_x;
    for (int jj = 0; jj < n_x; jj++) xf[jj] = 0.0;
    for (int ii = 0; ii < n_incl; ii++)
      for (int jj = 0; jj < n_x; jj++) xf[jj] += dist[zz * n_incl + ii] * flu[(size_t) ii * n_x + jj];
    double nf = primary_norm_factor(p->prim_type, ect_zone, p->gam) / src_norm;
    for (int jj = 0; jj < n_x; jj++) xf[jj] /= nf;
  }
  /* relxill_convolution_multizone, Relxill.cpp:432-482 */
  double *xr = malloc(sizeof(double) * N_ENER_CONV), *co = malloc(sizeof(double) * N_ENER_CONV);
  for (int ie = 0; ie < N_ENER_CONV; ie++) out_conv[ie] = 0.0;
  for (int zz = 0; zz < nz && !status; zz++) {
    double s = 0.0;
    for (int jj = 0; jj < N_ENER_CONV; jj++) s += rel[zz * N_ENER_CONV + jj];
    if (s < 1e-12) continue;
    relxo_rebin_spectrum(ener, xr, N_ENER_CONV, xener, xz + (size_t) zz * n_x, n_x);
    conv_spectrum_normalized(ener, xr, rel + (size_t) zz * N_ENER_CONV, co, N_ENER_CONV);
    for (int ie = 0; ie < N_ENER_CONV; ie++) out_conv[ie] += co[ie];
  }
  /* PrimarySource::add_primary_spectrum, PrimarySource.cpp:66-125 */
  if (!status) {
    double *prim = malloc(sizeof(double) * N_ENER_CONV);
    double eshift = (p->emis_type == EMIS_TYPE_LP) ? g_inf : 1.0;
    primary_spectrum(p->prim_type, prim, ener, N_ENER_CONV, ect_source, p->gam, eshift);
    for (int ie = 0; ie < N_ENER_CONV; ie++) prim[ie] *= src_norm;
    if (p->emis_type != EMIS_TYPE_LP) {
      for (int ie = 0; ie < N_ENER_CONV; ie++) out_conv[ie] *= fabs(p->refl_frac);
    } else {
      double refl_frac_input = p->refl_frac;
      if (p->interpret_reflfrac_as_boost) refl_frac_input *= sp->refl_frac;
      double prim_fac = sp->f_inf_rest / 0.5 * pow(g_inf, p->gam);
      if (p->beta > 1e-4) prim_fac *= pow(doppler_factor(M_PI - p->incl, p->beta), 2);
      double norm_fac_refl = (fabs(refl_frac_input)) / sp->refl_frac;
      for (int ie = 0; ie < N_ENER_CONV; ie++) out_conv[ie] *= norm_fac_refl;
      for (int ie = 0; ie < N_ENER_CONV; ie++) prim[ie] *= prim_fac;
    }
    if (p->refl_frac >= 0)
      for (int ie = 0; ie < N_ENER_CONV; ie++) out_conv[ie] += prim[ie];
    free(prim);
  }
  free(rel); free(dist); free(xener); free(flu); free(xz); free(xr); free(co);
  free_syspar(sp);
  return status;
}

/* xillver_model (LocalModel.cpp:103-128): the table spectrum at the inclination, the
 * semi-infinite slab factor 0.5 cos(incl) (Xillspec.cpp:528-545), rebinned to the caller's grid,
 * and add_primary_component without relativistic parameters (Relbase.cpp:294-349) */
static int xillver_model(const Params *p, const double *ener, int n, double *flux) {
  XillTable *t = (p->prim_type == PRIM_NTHCOMP) ? g_xill_cp : g_xill;
  xill_begin_eval(t);
  const int nx = t->n_ener;
  double *spec = malloc(sizeof(double) * nx), *xe = malloc(sizeof(double) * (nx + 1));
  int status = xillver_spectrum_at_incl(t, p->gam, p->afe, p->lxi, p->ect, p->incl, p->dens, spec);
  if (!status) {
    const double nf = 0.5 * cos(p->incl * M_PI / 180);
    for (int ii = 0; ii < nx; ii++) spec[ii] *= nf;
    for (int ii = 0; ii < nx; ii++) xe[ii] = t->elo[ii];
    xe[nx] = t->ehi[nx - 1];
    relxo_rebin_spectrum(ener, flux, n, xe, spec, nx);
    /* calc_normalized_primary_spectrum (Xillspec.cpp:302-332) on the caller's grid */
    double *pl = malloc(sizeof(double) * n);
    primary_spectrum(p->prim_type, pl, ener, n, p->ect, p->gam, 1.0);
    const double norm = primary_norm_factor(p->prim_type, p->ect, p->gam);
    for (int ii = 0; ii < n; ii++) pl[ii] *= norm;
    for (int ii = 0; ii < n; ii++) flux[ii] *= fabs(p->refl_frac);
    if (p->refl_frac >= 0)
      for (int ii = 0; ii < n; ii++) flux[ii] += pl[ii];
    free(pl);
  }
  free(spec); free(xe);
  return status;
}

/* ======================================================================= */
/* public entry points                                                      */
/* ======================================================================= */

int relxo_set_table_path(const char *path) {
  snprintf(g_table_path, sizeof g_table_path, "%s", path);
  return 0;
}

/* LocalModel::eval_model (LocalModel.h:108-128) + the model kernels */
int relxo_eval_ext(int model, const double *params, int ion_grad_type, double iongrad_index, const double *energy,
                   int n_flux, double *flux) {
  Params p;
  const int is_conv = (model == RELXO_RELCONV || model == RELXO_RELCONVLP);
  for (int ii = 0; ii < n_flux; ii++) if (!is_conv) flux[ii] = 0.0;
  if (map_params(model, params, ion_grad_type, iongrad_index, &p)) return 1;
  const int is_cp = (model == RELXO_XILLVERCP || model == RELXO_RELXILLCP || model == RELXO_RELXILLLPCP);
  int is_rx = (model == RELXO_RELXILL || model == RELXO_RELXILLLP || model == RELXO_XILLVER);
  if (ensure_tables(is_rx, is_cp)) return 2;
  /* XspecSpectrum copy + shift_energy_grid_redshift (XspecSpectrum.h:35-76) */
  double *ener = malloc(sizeof(double) * (n_flux + 1));
  for (int ii = 0; ii <= n_flux; ii++) ener[ii] = energy[ii];
  if (p.z > 0)
    for (int ii = 0; ii <= n_flux; ii++) ener[ii] *= (1 + p.z);
  int status = 0;
  if (model == RELXO_XILLVER || model == RELXO_XILLVERCP) {
    status = xillver_model(&p, ener, n_flux, flux);
  } else if (model == RELXO_RELLINE || model == RELXO_RELLINELP) {
    /* line_model, LocalModel.cpp:32-51 */
    for (int ii = 0; ii <= n_flux; ii++) ener[ii] /= p.lineE;
    status = relbase_single(&p, ener, n_flux, flux);
  } else if (model == RELXO_RELCONV || model == RELXO_RELCONVLP) {
    /* conv_model + relconv_kernel, LocalModel.cpp:82-98, Relbase.cpp:257-289 */
    double s = 0.0;
    for (int ii = 0; ii < n_flux; ii++) s += flux[ii];
    if (s <= 0.0) { free(ener); return 3; }
    const double *cg = conv_grid();
    double *prof = malloc(sizeof(double) * N_ENER_CONV), *rb = malloc(sizeof(double) * N_ENER_CONV),
           *co = malloc(sizeof(double) * N_ENER_CONV);
    status = relbase_single(&p, cg, N_ENER_CONV, prof);
    if (!status) {
      relxo_rebin_spectrum(cg, rb, N_ENER_CONV, ener, flux, n_flux);
      conv_spectrum_normalized(cg, rb, prof, co, N_ENER_CONV);
      relxo_rebin_spectrum(ener, flux, n_flux, cg, co, N_ENER_CONV);
      for (int ii = 0; ii < n_flux; ii++)
        if (ener[ii + 1] < RELCONV_EMIN || ener[ii] > RELCONV_EMAX) flux[ii] = 0;
    }
    free(prof); free(rb); free(co);
  } else {
    double *conv = malloc(sizeof(double) * N_ENER_CONV);
    status = relxill_kernel(&p, conv);
    if (!status) {
      /* rebin_and_normalize_relxill_for_xspec, Relxill.cpp:249-278 */
      const double *cg = conv_grid();
      if (env_is_one("RELXILL_RENORMALIZE")) {
        int ind = binary_search(cg, N_ENER_CONV, 3.0);
        double dE = cg[ind + 1] - cg[ind];
        double nf = 1.0 / (conv[ind] / dE);
        for (int ii = 0; ii < N_ENER_CONV; ii++) conv[ii] *= nf;
      }
      relxo_rebin_spectrum(ener, flux, n_flux, cg, conv, N_ENER_CONV);
    }
    free(conv);
  }
  free(ener);
  return status;
}

int relxo_eval(int model, const double *params, const double *energy, int n_flux, double *flux) {
  return relxo_eval_ext(model, params, ION_GRAD_TYPE_CONST, 0.0, energy, n_flux, flux);
}

/* the 4096-bin convolution grid of get_relxill_conv_energy_grid (Xillspec.cpp:44-54) */
void relxo_conv_grid(double *out) {
  const double *g = conv_grid();
  memcpy(out, g, sizeof(double) * (N_ENER_CONV + 1));
}

/* relline profile on an arbitrary grid (for component tests): model params as relline */
int relxo_relline_profile_zones(int model, const double *params, const double *ener, int n_ener, int *nzones_out,
                                double *flux, int n_incl, double *dist) {
  Params p;
  if (map_params(model, params, ION_GRAD_TYPE_CONST, 0.0, &p)) return 1;
  if (ensure_tables(0, 0)) return 2;
  int status = 0;
  SysPar *sp = get_system_parameters(&p, NULL, &status);
  double rgrid[N_ZONES_MAX + 1];
  get_rzone_grid(p.rin, p.rout, p.num_zones, p.height, rgrid);
  *nzones_out = p.num_zones;
  if (!status) status = relline_profile(sp, &p, ener, n_ener, p.num_zones, rgrid, flux, n_incl, dist);
  free_syspar(sp);
  return status;
}
