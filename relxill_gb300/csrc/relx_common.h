// relx_common.h -- definitions shared by the host runtime and the sm_103a kernels
// of the relativistic convolution path (relline / relconv / relxill / relxilllp).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define RELX_HD __host__ __device__
#else
#define RELX_HD
#endif

// model ids (lmodel_relxill_public.dat:1,13,23,35,46,61,77,86,96,112)
enum RelxModel {
  RELX_RELLINE = 0, RELX_RELCONV = 1, RELX_RELXILL = 2, RELX_RELXILLLP = 3,
  RELX_RELLINELP = 4, RELX_RELCONVLP = 5, RELX_XILLVER = 6,
  RELX_XILLVERCP = 7, RELX_RELXILLCP = 8, RELX_RELXILLLPCP = 9, RELX_NMODELS = 10
};

// The kernels work on four kinds of evaluation: a line profile (relline, relline_lp), a
// convolution of the caller's spectrum (relconv, relconv_lp), a relativistic reflection
// spectrum (relxill, relxilllp) and the non-relativistic reflection spectrum (xillver).  The
// lamp-post line and convolution models differ from their broken-power-law twins only in the
// emissivity (LocalModel.cpp:32-98 runs the same code for both).
// The Cp models (relxillCp, relxilllpCp, xillverCp) are the reflection kinds with the nthcomp
// continuum and the 6-parameter xillverCp table.
RELX_HD inline int relx_kind(int model) {
  switch (model) {
    case RELX_RELLINELP: return RELX_RELLINE;
    case RELX_RELCONVLP: return RELX_RELCONV;
    case RELX_XILLVERCP: return RELX_XILLVER;
    case RELX_RELXILLCP: return RELX_RELXILL;
    case RELX_RELXILLLPCP: return RELX_RELXILLLP;
    default: return model;
  }
}
RELX_HD inline bool relx_is_cp(int model) {
  return model == RELX_XILLVERCP || model == RELX_RELXILLCP || model == RELX_RELXILLLPCP;
}
RELX_HD inline bool relx_is_relxill(int kind) { return kind == RELX_RELXILL || kind == RELX_RELXILLLP; }

// error codes written per set and returned by the C ABI
enum RelxStatus {
  RELX_OK = 0,
  RELX_ERR_PARAM = 1,        // parameter out of the allowed range (check_parameter_bounds)
  RELX_ERR_TABLE = 2,        // table missing or inconsistent
  RELX_ERR_UNSUPPORTED = 3,  // unsupported model option
  RELX_ERR_GRID = 4,         // radial interpolation outside the table (Relprofile.cpp:255-278)
  RELX_ERR_INPUT = 5,        // relconv input spectrum with sum <= 0 (LocalModel.cpp:84-86)
  RELX_ERR_CUDA = 6,         // CUDA runtime error
  RELX_ERR_NOMEM = 7,        // device memory budget exceeded
  RELX_ERR_TIMEOUT = 8,      // a bounded device wait gave up
  RELX_ERR_ARG = 9,          // bad arguments at the C ABI
  RELX_ERR_NOTABLE = 10,     // tables not loaded
};

// constants of the reference (common.h:133-136, Xillspec.h:28-38, Relbase.h:38-39)
#define RELX_NFRAD 1000
#define RELX_NZONES 10
#define RELX_NZONES_IONGRAD 25
#define RELX_NZMAX 50
#define RELX_NCONV 4096
#define RELX_EMIN_CONV 0.00035
#define RELX_EMAX_CONV 2000.0
#define RELX_NCOARSE 500
#define RELX_EMIN_NORM 0.1
#define RELX_EMAX_NORM 1000.0
#define RELX_EMIN_XILL 0.01
#define RELX_EMAX_XILL 1000.0
#define RELX_GFAC_H 5e-3
#define RELX_RELTABLE_MAX_R 1000.0

// capacity limits of the device kernels (checked when tables load)
#define RELX_MAX_NG 64
#define RELX_MAX_NRTAB 128
#define RELX_MAX_NRADLP 128
#define RELX_MAX_INCL 16
#define RELX_MAX_XPAR 8
#define RELX_ZDENSE 16            // zones handled with the de-duplicated xillver corner list
#define RELX_MAX_UCORNER 256      // 16 corners x RELX_ZDENSE zones
#define RELX_NPARAM_MAX 18

// returning-radiation table (common.h:127-129)
#define RELX_RR_NR 50
#define RELX_RR_NG 20
#define RELX_RR_MAXSPIN 99

#define RELX_EMIS_BKN 1
#define RELX_EMIS_LP 2

// Device-resident tables (uploaded once).  All arrays are device pointers.
struct NthGrid;
struct RelxTables {
  // relline table (reltable.h:24-48): [a][mu0][r] and [a][mu0][r][g] (float4 = trff1,trff2,cosne1,cosne2)
  int rel_na, rel_nmu0, rel_nr, rel_ng;
  const float *rel_a, *rel_mu0;
  const float *rel_r, *rel_gmin, *rel_gmax;
  const float4 *rel_tc;
  // lamp-post table (reltable.h:51-69): [a][h], [a][rad], [a][h][rad]; del, del_inc stored as |x|
  int lp_na, lp_nh, lp_nrad;
  const float *lp_a, *lp_h, *lp_rad, *lp_intens, *lp_del, *lp_delinc;
  // xillver table (common.h:254-277), 5 parameters, Incl last
  int x_npar, x_nener, x_nener_pad, x_nincl;
  int x_nvals[RELX_MAX_XPAR];
  int x_pindex[RELX_MAX_XPAR];
  int x_has_dens;
  const float *x_vals;       // [x_npar][x_maxvals]
  int x_maxvals;
  const float *x_spec;       // [rows][x_nener_pad], each row divided by 10^logXi of its grid point
  int64_t x_rows;
  // the same rows rebinned onto the conv grid and weighted by E/dE of the conv bin (the form the
  // convolution reads): conv bins [x_clo, x_clo + x_cn), rows of x_cpad floats (a multiple of 4)
  const float *x_cspec;
  int x_clo, x_cn, x_cpad;
  // conv grid and precomputed maps
  const double *conv_e;      // [RELX_NCONV+1]
  const float2 *conv_eff;    // float-float edges
  const float *conv_inv_emid;  // 1/(0.5(e_j+e_j+1))
  const float *conv_cf;      // 0.5(e_j+e_j+1)/(e_j+1-e_j)  (Relbase.cpp:93-103)
  const float2 *conv_cw;     // (float) 0.5(e_j+e_j+1), (float) (e_j+1-e_j)
  int conv_pos1;             // binary_search(conv_e, 1.0)  (Relbase.cpp:133-137)
  float conv_lg0, conv_ilg;  // log(conv_e[0]) and N / log(conv_e[N] / conv_e[0]): first guess of a bin index
  int conv_band_lo, conv_band_hi;  // bins with e_j >= 0.01 && e_j+1 < 1000 (Relbase.cpp:205)
  const double *coarse_e;    // [RELX_NCOARSE+1]
  const float4 *coarse_t;    // per coarse bin: (float) centre, (float) width, centre as float-float; zero
                             // centre weight outside [RELX_EMIN_NORM, RELX_EMAX_NORM] (Xillspec.cpp:185-190)
  // rebin map xillver grid -> conv grid (relutility.c:549-601): per conv bin
  const int *rb_imin, *rb_imax;
  const float *rb_fmin, *rb_fmax;  // fractions (single-bin case: rb_fmin, rb_imax == rb_imin)
  const int4 *rb_pack;       // per conv bin: imin, imax, fmin and fmax as float bits
  const double *x_e;         // xillver edges [x_nener+1] (double of the float table values)
  const float2 *x_ew;        // per xillver edge: the edge, (float) (x_e[k+1] - x_e[k]) (0 at the last edge)
  // per xillver corner (table row of incl 0 / x_nincl): the inclination-averaged energy flux in
  // 0.1-1000 keV, photon flux in 0.15-500 keV, and photon flux of the spectrum shifted by g = 2/3
  // (get_xillver_fluxcorrection_factors, Xillspec.cpp:109-160, 344-361, 457-526)
  const double *x_fcorr;     // [corners][3]
  int coarse_b2_skip[2];     // coarse bins in the normalisation band but outside the 0.1-1000 keV flux band (-1: none)
  // returning-radiation table (Relreturn_Table.cpp:180-330); rr_nspin = 0 when it is not loaded
  int rr_nspin;
  const double *rr_spin;     // [nspin]
  const double *rr_rlo, *rr_rhi;  // [nspin][RELX_RR_NR]
  const double *rr_tfr;      // [nspin][RELX_RR_NR][RELX_RR_NR], row = incident bin, column = emitting bin
  const float4 *rr_g;        // [nspin][NR incident][NG][NR emitting]: frac_g, g, log2 g, 1 if |g - 1| > 1e-3 else 0
  // nthcomp photon grid of the Cp models (nthcomp.cu)
  const NthGrid *nth_grid;
};

// per-set inputs
struct RelxSetIn {
  double p[RELX_NPARAM_MAX];
  int64_t e_off;     // offset of the set's user energy grid (n+1 edges) in the concatenated grid array
  int n_ener;        // number of user bins
  int ion_grad_type; // hidden switch (0 const, 1 PL, 2 ALPHA)
  double iongrad_index;
  int nzones_env;    // RELXILL_NUM_RZONES value or 0
  int flags;         // bit0 RELLINE_PHYSICAL_NORM, bit1 RELXILL_RENORMALIZE, bit2 RELXILL_CONSTANT_DENSITY
  int nza;           // zones the batch's per-set arrays hold (a set needing more fails)
};

// per-set state written by the setup kernel
struct RelxSetState {
  int status, model, emis_type, limb, nz, ion_grad_type, boost_switch;
  int pmodel;       // the caller's model id (model holds its kind, relx_kind)
  int prim;         // primary continuum: 0 cut-off power law, 1 nthcomp (Cp models)
  int rr_corr;      // returning radiation with xillver correction factors (line profile not cacheable)
  int cached;       // line profile, tile sums and angle histograms come from the profile cache
  int g_n;          // bins of the line-profile grid (user grid for relline, conv grid otherwise)
  int win_lo, win_hi;  // line-profile bins touched by any radius
  int ind_a, ind_mu0;
  float ifac_a, ifac_mu0;
  int ucount;       // unique xillver corners (dense mode)
  int xdense;       // 1: the zone spectra come from the de-duplicated corner list (RelxCorners),
                    // 0: from the per-zone lists (RelxZoneCorners)
  int out_lo, out_hi;  // conv-grid bins the caller's grid needs (inclusive)
  double a, incl, rin, rout, height, beta, gamma, z, lineE;
  double gam, ect_src, refl_frac;
  double relline_norm;   // renormalisation target; <= 0 means no renormalisation
  double g_inf, f_inf_rest, refl_frac_lp, prim_fac, norm_fac_refl, src_norm;
  double rgrid[RELX_NZMAX + 1];
  int zi0[RELX_NZMAX], zi1[RELX_NZMAX];   // fine-radius index range of each zone (inclusive)
  int zw_lo[RELX_NZMAX], zw_hi[RELX_NZMAX]; // line-profile bins touched by the zone's radii [lo, hi)
  float inv_nc[RELX_NZMAX];               // 1 / normalisation change source->disk (Xillspec.cpp:408-440)
  double zshift[RELX_NZMAX];              // energy shift source -> disk of each zone (Ecut / kTe factor)
};

// nthcomp (nthcomp.cu): the photon grid of the Kompaneets solve.  The seed temperature is fixed
// (0.05 keV), so the grid and every quantity on it that does not depend on kTe or Gamma are computed
// once: per point j (float-float) Cooper's coefficient / deltal, 1 / (deltal sqrt(x_j x_j+1)), the
// Klein-Nishina factor / 3, x^3, x times the seed photon rate, x^4, the normalisation weight of the
// point on the 500-bin coarse grid, and x itself.
#define RELX_NTH_N 901
struct __align__(16) NthPoint {
  float2 cd, iw, rel3, x3, xd, x4, g, x;
};
struct NthGrid {
  NthPoint p[RELX_NTH_N + 1];  // j = 1..901
  double x[RELX_NTH_N + 2];    // x_j (FP64), j = 1..902
  int jnr0, jrel0, ih0, pad_;  // region bounds of the escape probability, index of the 1 keV point
  float l2x511, inv_l2step;    // log2(x_1 511 keV), 1 / (log2 of the grid ratio): grid position of an energy
};
// E F_E table of a set's source continuum, sp[1..n] on the grid's x, and its float copy
struct NthTable {
  double sp[RELX_NTH_N];
  float spf[RELX_NTH_N];
  int n;
  int pad_[3];
};

// per-radius record of the line-profile kernels (64 bytes, staged into shared memory as int4 rows)
struct __align__(16) RelxRadRec {
  float2 gmin, gmax, dg;  // float-float gmin, gmax, gmax - gmin
  float2 eH, e1H;         // gstar2ener(H), gstar2ener(1-H) (relutility.c:260-262)
  float inv_dg;           // 1/(gmax-gmin)
  float ew;               // emissivity * trapez weight / 2
  float ifac;             // radial interpolation factor of the table
  int ielo, iehi;         // line-profile bins touched (-1: none)
  short itab;             // table radius index: re_tab[itab+1] <= re < re_tab[itab]
  unsigned char red_H;    // gstar2ener(H) >= 0.95 (int_romb, Relprofile.cpp:636)
  unsigned char zone;
};
static_assert(sizeof(RelxRadRec) == 64, "radius record is four int4 rows");

// per-set radial data [RELX_NFRAD] (written by setup, read by the line-profile kernels)
struct RelxRadial {
  RelxRadRec rec[RELX_NFRAD];
  double re[RELX_NFRAD];
  double ifac[RELX_NFRAD];    // FP64 radial factor (emission-angle bin decisions near bin edges)
  float  wt[RELX_NFRAD];      // trapez weight / 2
};
static_assert(sizeof(RelxRadial) % 16 == 0, "per-set radial records stay 16-byte aligned");

// xillver corners of one set (dense mode: de-duplicated across zones)
struct RelxCorners {
  int row[RELX_MAX_UCORNER];              // spectrum row of incl 0 (rows of incl i are row + i)
  float w[RELX_MAX_UCORNER][RELX_ZDENSE]; // weight of the corner in each zone (0 if unused)
};

// per-zone corners (used when nz > RELX_ZDENSE)
struct RelxZoneCorners {
  int row[RELX_NZMAX][32];   // 16 corners for a 5-parameter table, 32 for the 6-parameter one
  float w[RELX_NZMAX][32];
};
