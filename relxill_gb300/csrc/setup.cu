// setup.cu -- per-parameter-set preparation kernel (one CTA per set).
//
// Everything the reference computes once per evaluation before the line
// integration: parameter mapping and bounds (ModelDefinition.cpp:153-385),
// the (a, mu0) interpolation of the relline table on its own radii and the
// 1000-point fine radial grid (Relprofile.cpp:141-303, relutility.c:666-677),
// the emissivity (broken power law, Rellp.cpp:91-109,421-437; lamp post,
// Rellp.cpp:36-285), the radial zones and ionisation gradient
// (IonGradient.cpp:128-211,340-390,457-492), the xillver brackets and
// interpolation factors per zone (xilltable.c:297-323,1054-1181) and the
// primary-continuum normalisations (Xillspec.cpp:179-233,302-332,408-440).
// FP64 is used for the radii, the zone grid, the ISCO/horizon and the
// normalisation sums; per-radius transcendental work that has no
// cancellation runs in FP32.
#include "relx_device.cuh"

namespace relx {

constexpr int kSetupThreads = 256;
constexpr int kQGroup = 8;
constexpr double kDeg75 = 75.0 / 180.0 * 3.14159265358979323846;  // 75 degrees in radians  // continua summed together (normalisation of the primary continuum)
// the table normalisation's unit factor (Xillspec.cpp:179-205), one product
constexpr double kQsumScale = 1e20 * 1.602177e-09 / (1e15 / 4.0 / kPi);

// returning radiation of one set on the radial bins of the return table (Relreturn_Corona.cpp)
struct RradSmem {
  int n, klo, spin;                  // trimmed bins, first table bin, table spin index
  double rad[RELX_RR_NR];            // bin centres (ascending)
  float cg_f[RELX_RR_NR];            // g-shift correction of the emitting bin, as float
  unsigned char use_corr[RELX_RR_NR];  // that correction differs from 1 by more than 1e-3
  double inv_drad[RELX_RR_NR];       // 1 / (rad[k + 1] - rad[k])
  double area_in, area_out;          // ring-area corrections of the first and last bin
  float emis_in[RELX_RR_NR];         // direct emissivity at the bin centres
  float er[RELX_RR_NR], dl[RELX_RR_NR];  // returning emissivity per bin, log2(er[k + 1] / er[k])
  float cf_flux[RELX_RR_NR];         // xillver correction factors on the table bins
  double zcf_flux[RELX_NZMAX], zcf_g[RELX_NZMAX];  // per ionisation zone
};

struct SetupSmem {
  RelxSetState s;
  double re_tab[RELX_MAX_NRTAB], gmin_t[RELX_MAX_NRTAB], gmax_t[RELX_MAX_NRTAB];
  double re[RELX_NFRAD];
  union {
    double sqre[RELX_NFRAD];   // 1/u of the fine grid, i.e. sqrt(re) (lamp-post flux boost only)
    struct {                   // returning radiation, after the lamp-post emissivity
      RradSmem rr;
      float emis_lp[RELX_NFRAD];  // direct lamp-post emissivity
    } rt;
  };
  double inv_dtab[RELX_MAX_NRTAB];
  double dgmin_t[RELX_MAX_NRTAB], dgmax_t[RELX_MAX_NRTAB];  // gmin, gmax of table radius i less those of i + 1
  float jet_rad_f[RELX_MAX_NRADLP];
  float lp_dle[RELX_MAX_NRADLP], lp_dlr[RELX_MAX_NRADLP], lp_d[RELX_MAX_NRADLP], lp_di[RELX_MAX_NRADLP];
  float lp_e[RELX_MAX_NRADLP], inv_jr_f[RELX_MAX_NRADLP], inv_drad_f[RELX_MAX_NRADLP];
  unsigned char lp_log[RELX_MAX_NRADLP];  // logarithmic radial factor (emission angle above 75 deg)
  double qsum[RELX_NZMAX + 1];       // normalisation sums of the primary continuum
  float qecut[RELX_NZMAX + 1];       // their cut-off energies
  float2 qpart[kSetupThreads / 32][8];  // per-warp partial sums of a group of continua
  float cpow[RELX_NCOARSE];          // E^-Gamma at the coarse-grid bin centres
  double jet_rad[RELX_MAX_NRADLP], d_tab[RELX_MAX_NRADLP];
  double red[40];
  int ired[40];
  int zlo[RELX_NZMAX], zhi[RELX_NZMAX];  // per-zone profile windows (inclusive bins)
  int ind_rmin, ind_rmax, status;
  double rms;        // ISCO radius of the set's spin
  // parameters beyond the state
  double emis1, emis2, rbr, htop, lxi, afe, dens, iongrad_index;
  int return_rad, flags, is_relxill;
  // lamp post interpolation
  int lp_ind_a, ind_h[2];
  double ginf_pow;   // g_inf^Gamma of the primary's flux factor (computed early, beside other work)
  double fg_r1, fg_du;  // fine radial grid: u = 1/sqrt(r) of Rout and the step in u
  float ut_h, inv_rbr;  // lamp-post u^t of the source; 1 / Rbr
  double lp_ifac_a, ifac_h[2];
  // zones
  double rmean[RELX_NZMAX], shift[RELX_NZMAX], zlxi[RELX_NZMAX], zdens[RELX_NZMAX], xscale[RELX_NZMAX];
  double zdel_emit[RELX_NZMAX];
  int zind[RELX_NZMAX][RELX_MAX_XPAR];
  double zfac[RELX_NZMAX][RELX_MAX_XPAR];
  // the emissivity of the fine radii (FP32 values) is read up to the zones' ionisation, the corner
  // lists only after it: they share their storage
  union {
    struct {
      float emis[RELX_NFRAD], del_emit[RELX_NFRAD], del_inc[RELX_NFRAD];
    } pr;
    struct {
      int crow[RELX_NZMAX * 16];
      short cfirst[RELX_NZMAX * 16];
      short cuniq[RELX_NZMAX * 16];
      float cw[RELX_NZMAX * 16];            // weight of every (zone, corner) entry
      unsigned char clive[RELX_NZMAX * 16]; // row has a non-zero weight in some zone
    } cr;
  };
};
static_assert(sizeof(RradSmem) + sizeof(float) * RELX_NFRAD <= sizeof(double) * RELX_NFRAD,
              "returning-radiation scratch fits in the lamp-post scratch it reuses");

// ---------------------------------------------------------------------------
// parameter mapping (lmodel_relxill_public.dat:1-75, ModelDefinition.cpp:153-385)
// ---------------------------------------------------------------------------
__device__ void map_params(int model, const RelxSetIn &in, SetupSmem &m) {
  RelxSetState &s = m.s;
  const double *v = in.p;
  s.model = relx_kind(model);
  s.pmodel = model;
  s.status = RELX_OK;
  s.cached = 0;
  s.rr_corr = 0;
  s.prim = relx_is_cp(model) ? 1 : 0;
  s.limb = 0;
  s.height = 0;
  s.beta = 0;
  s.z = 0;
  s.lineE = 0;
  s.gam = 0;
  s.refl_frac = 0;
  s.boost_switch = 0;
  m.emis1 = m.emis2 = m.rbr = 0;
  m.htop = 0;
  m.lxi = 0;
  m.afe = 0;
  m.dens = 15;     // ModelDefinition.cpp:362
  s.ect_src = 300; // ModelDefinition.cpp:360
  m.return_rad = 0;
  m.is_relxill = 0;
  m.flags = in.flags;
  m.iongrad_index = in.iongrad_index;
  s.ion_grad_type = in.ion_grad_type;
  switch (model) {
    case RELX_RELLINE:
      s.emis_type = RELX_EMIS_BKN;
      s.lineE = v[0]; m.emis1 = v[1]; m.emis2 = v[2]; m.rbr = v[3]; s.a = v[4]; s.incl = v[5] * kPi / 180;
      s.rin = v[6]; s.rout = v[7]; s.z = v[8]; s.limb = (int) llround(v[9]);
      break;
    case RELX_RELCONV:
      s.emis_type = RELX_EMIS_BKN;
      m.emis1 = v[0]; m.emis2 = v[1]; m.rbr = v[2]; s.a = v[3]; s.incl = v[4] * kPi / 180;
      s.rin = v[5]; s.rout = v[6]; s.limb = (int) llround(v[7]);
      break;
    case RELX_RELLINELP:  // lmodel_relxill_public.dat:23-33; no source velocity
      s.emis_type = RELX_EMIS_LP;
      s.lineE = v[0]; s.height = v[1]; s.a = v[2]; s.incl = v[3] * kPi / 180; s.rin = v[4]; s.rout = v[5];
      s.z = v[6]; s.limb = (int) llround(v[7]); s.gam = v[8]; m.return_rad = (int) llround(v[9]);
      break;
    case RELX_RELCONVLP:  // lmodel_relxill_public.dat:35-44
      s.emis_type = RELX_EMIS_LP;
      s.height = v[0]; s.beta = v[1]; s.a = v[2]; s.incl = v[3] * kPi / 180; s.rin = v[4]; s.rout = v[5];
      s.limb = (int) llround(v[6]); s.gam = v[7]; m.return_rad = (int) llround(v[8]);
      break;
    case RELX_RELXILL:
      m.is_relxill = 1;
      s.emis_type = RELX_EMIS_BKN;
      m.emis1 = v[0]; m.emis2 = v[1]; m.rbr = v[2]; s.a = v[3]; s.incl = v[4] * kPi / 180;
      s.rin = v[5]; s.rout = v[6]; s.z = v[7]; s.gam = v[8]; m.lxi = v[9]; m.afe = v[10];
      s.ect_src = v[11]; s.refl_frac = v[12];
      break;
    case RELX_RELXILLCP:  // lmodel_relxill_public.dat:96-110
      m.is_relxill = 1;
      s.emis_type = RELX_EMIS_BKN;
      s.incl = v[0] * kPi / 180; s.a = v[1]; s.rin = v[2]; s.rout = v[3]; m.rbr = v[4]; m.emis1 = v[5];
      m.emis2 = v[6]; s.z = v[7]; s.gam = v[8]; m.lxi = v[9]; m.dens = v[10]; m.afe = v[11]; s.ect_src = v[12];
      s.refl_frac = v[13];
      break;
    case RELX_RELXILLLPCP:  // lmodel_relxill_public.dat:112-129: the ionisation gradient is a parameter
      m.is_relxill = 1;
      s.emis_type = RELX_EMIS_LP;
      s.incl = v[0] * kPi / 180; s.a = v[1]; s.rin = v[2]; s.rout = v[3]; s.height = v[4]; s.beta = v[5];
      s.gam = v[6]; m.lxi = v[7]; m.dens = v[8]; m.afe = v[9]; s.ect_src = v[10]; s.refl_frac = v[11]; s.z = v[12];
      m.iongrad_index = v[13];
      s.ion_grad_type = (int) llround(v[14]);
      m.return_rad = (int) llround(v[15]);
      s.boost_switch = (int) llround(v[16]);
      break;
    case RELX_RELXILLLP:
      m.is_relxill = 1;
      s.emis_type = RELX_EMIS_LP;
      s.height = v[0]; s.beta = v[1]; s.a = v[2]; s.incl = v[3] * kPi / 180; s.rin = v[4]; s.rout = v[5];
      s.z = v[6]; s.gam = v[7]; m.lxi = v[8]; m.afe = v[9]; s.ect_src = v[10]; s.refl_frac = v[11];
      m.return_rad = (int) llround(v[12]);
      s.boost_switch = (int) llround(v[13]);
      break;
    default:
      s.status = RELX_ERR_ARG;
      return;
  }
  s.gamma = s.gam;
  // check_parameter_bounds, ModelDefinition.cpp:168-273
  double rms = kerr_rms(s.a);
  m.rms = rms;
  if (s.rin < 0) s.rin = -1.0 * s.rin * rms;
  if (s.rout < 0) s.rout = -1.0 * s.rout * rms;
  if (m.rbr < 0) m.rbr = -1.0 * m.rbr * rms;
  int bad = 0;
  if (s.rout <= s.rin) bad = 1;
  if (s.rin < rms) s.rin = rms;
  if (s.a > 0.9982 || s.a < -1) bad = 1;
  if (s.incl < 3 * kPi / 180 || s.incl > 87 * kPi / 180) bad = 1;
  if (s.rout <= s.rin) bad = 1;
  if (bad) { s.status = RELX_ERR_PARAM; return; }
  if (s.rout > 1000.0) s.rout = 1000.0;
  if (s.emis_type == RELX_EMIS_BKN) {
    if (m.rbr < s.rin) m.rbr = s.rin;
    if (m.rbr > s.rout) m.rbr = s.rout;
  }
  if (s.emis_type == RELX_EMIS_LP) {
    if (s.beta < 0) s.beta = 0.0;
    if (s.beta > 0.99) s.beta = 0.99;
    double rp = kerr_rplus(s.a);
    if (s.height < 0) s.height = -1.0 * s.height * rp;
    if ((1.1 * rp - s.height) > 1e-4) s.height = rp * 1.1;
  }
  // $switch_returnrad: 1 adds the returning radiation, -1 and 2 keep only it (add_returnrad_emis,
  // Rellp.cpp:483-509); the models without the switch pass 0
  if (m.return_rad != 0 && m.return_rad != 1 && m.return_rad != -1 && m.return_rad != 2) {
    s.status = RELX_ERR_PARAM;
    return;
  }
  // get_num_zones, relutility.c:506-544 (RELXILL_NUM_RZONES arrives in nzones_env)
  int envn = in.nzones_env;
  if (s.ion_grad_type != 0) {
    s.nz = (envn > 9 && envn <= RELX_NZMAX) ? envn : RELX_NZONES_IONGRAD;
  } else if (m.is_relxill && s.emis_type == RELX_EMIS_LP) {
    s.nz = (envn > 0 && envn <= RELX_NZMAX) ? envn : RELX_NZONES;
  } else {
    s.nz = 1;
  }
  if (s.nz > in.nza) {  // the batch's per-set arrays were sized for fewer zones
    s.status = RELX_ERR_ARG;
    return;
  }
  // renormalisation target (renorm_relline_profile, Relprofile.cpp:749-781; do_renorm_model, relutility.c:603-623)
  int phys = in.flags & 1;
  s.relline_norm = 1.0;
  if (m.is_relxill) {
    if (s.emis_type == RELX_EMIS_LP || phys) s.relline_norm = 0.0;
    else s.relline_norm = 0.5 * cos(s.incl * 180.0 / kPi * kPi / 180);
  } else if (phys) {
    s.relline_norm = 0.0;
  }
  // energy shift source -> observer (Relphysics.cpp:239-255) and the source-frame Ecut (Relxill.cpp:196-200);
  // kTe of the nthcomp continuum is already given in the source frame
  s.g_inf = 1.0;
  if (s.emis_type == RELX_EMIS_LP) {
    s.g_inf = calc_g_inf(s.height, s.a);
    if (!(s.beta < 1e-4)) s.g_inf *= doppler_factor(kPi - s.incl, s.beta);
    if (s.prim == 0) s.ect_src /= s.g_inf;
  }
}

// get_rzone_grid / RadialGrid::calculate_radial_grid (relutility.c:265-308, IonGradient.cpp:457-492),
// one warp: every lane computes its own edges (the same formula per edge as the serial loop)
__device__ void zone_grid_warp(double rmin, double rmax, int nz, double h, double *rg) {
  const int lane = threadIdx.x & 31;
  if (nz == 1) {
    if (lane == 0) { rg[0] = rmin; rg[1] = rmax; }
    __syncwarp();
    return;
  }
  double r_tr = rmin;
  int indr = 0;
  if (h > rmin) {
    r_tr = h;
    for (int ii = lane; ii < nz + 1; ii += 32) rg[ii] = exp(1.0 * ii / nz * (log(rmax) - log(rmin)) + log(rmin));
    __syncwarp();
    if (lane == 0) indr = bsearch_asc<double>(rg, nz + 1, r_tr);
    indr = __shfl_sync(0xffffffffu, indr, 0);
    r_tr = rg[indr];
    __syncwarp();
  }
  if (indr < nz) {
    double rlo = r_tr, rhi = rmax;
    for (int ii = indr + lane; ii < nz + 1; ii += 32) {
      double v = 1.0 * (ii - indr) / (nz - indr) * (1.0 / rhi - 1.0 / rlo) + 1.0 / rlo;
      rg[ii] = fabs(1.0 / v);
    }
  }
  __syncwarp();
}

// x0 descending; index ii with x0[ii] > xn >= x0[ii+1] (inv_rebin_mean, relutility.c:636-663)
__device__ double rebin_mean_at(const double *x0, const float *y0, int n0, double xn) {
  int klo = 0, khi = n0 - 1;  // count of x0 > xn via bisection
  while (khi - klo > 1) {
    int k = (khi + klo) >> 1;
    if (dgt(x0[k], xn)) klo = k; else khi = k;
  }
  int ii = klo;
  double f = (xn - x0[ii + 1]) / (x0[ii] - x0[ii + 1]);
  return lerp1(f, f2d(y0[ii + 1]), f2d(y0[ii]));
}


// ---------------------------------------------------------------------------
// returning radiation (Relreturn_Table.cpp:393-611, Relreturn_Corona.cpp:37-321)
// ---------------------------------------------------------------------------

// get_rrad_fractions for the set, serial part (thread 0): spin index (the first table spin >= a),
// the table bins covering [rin, rout] and the ring-area corrections of the end bins, whose first
// and last bin are reset to rin and rout.  rin, rout: the ends of the fine radial grid
// (determine_rlo_rhi).
__device__ int rrad_bins(const RelxTables &tab, RradSmem &q, double a, double rms, double rin, double rout) {
  const int NR = RELX_RR_NR;
  int k = bsearch_asc<double>(tab.rr_spin, tab.rr_nspin, a);
  if (tab.rr_spin[k] < a) k++;
  if (k >= tab.rr_nspin || k < 0) return RELX_ERR_TABLE;
  const double *rlo = tab.rr_rlo + (size_t) k * NR, *rhi = tab.rr_rhi + (size_t) k * NR;
  int klo = bsearch_asc<double>(rlo, NR, rin);
  int khi = bsearch_asc<double>(rhi, NR, rout);
  if (fabs(rout - rhi[NR - 1]) < 1e-6) khi = NR - 1;
  else khi++;
  if (fabs(rin - rlo[0]) < 1e-6) klo = 0;
  const int n = (khi + 1) - klo;
  // the reference asserts these (Relreturn_Table.cpp:455-456, 480; Rellp.cpp:150-151)
  if (n < 2 || n > NR || !(rin >= rlo[klo] - 1e-4)) return RELX_ERR_GRID;
  q.n = n;
  q.klo = klo;
  q.spin = k;
  // get_ring_area_correction_factor (Relreturn_Table.cpp:518-538)
  for (int e = 0; e < 2; e++) {
    const int i = e ? n - 1 : 0;
    double rlo_t = rlo[klo + i];
    if (klo + i == 0 && rlo_t > rms) rlo_t = rms;
    const double rhi_t = rhi[klo + i];
    const double lo = (i == 0) ? rin : rlo[klo + i], hi = (i == n - 1) ? rout : rhi[klo + i];
    const double c = (0.5 * (lo + hi) * (hi - lo)) / (0.5 * (rlo_t + rhi_t) * (rhi_t - rlo_t));
    if (!(c - 1 < 1e-6)) return RELX_ERR_GRID;
    if (e) q.area_out = c; else q.area_in = c;
  }
  return RELX_OK;
}

// get_rrad_fractions, the bin centres and their spacing (all threads, after rrad_bins)
__device__ void rrad_centres(const RelxTables &tab, RradSmem &q, double rin, double rout, int nt) {
  const int NR = RELX_RR_NR, n = q.n, klo = q.klo;
  const double *rlo = tab.rr_rlo + (size_t) q.spin * NR, *rhi = tab.rr_rhi + (size_t) q.spin * NR;
  for (int i = threadIdx.x; i < n; i += nt) {
    const double lo = (i == 0) ? rin : rlo[klo + i], hi = (i == n - 1) ? rout : rhi[klo + i];
    q.rad[i] = 0.5 * (lo + hi);
  }
  __syncthreads();
  for (int i = threadIdx.x; i + 1 < n; i += nt) q.inv_drad[i] = 1.0 / (q.rad[i + 1] - q.rad[i]);
  __syncthreads();
}

// the g-shift correction's linear coefficients of an emitting bin with correction cg
// (corrected_gshift_fluxboost_factor, Relreturn_Corona.cpp:37-86): a, 1 - a below cg = 1, al, 1 - al above
__device__ __forceinline__ float2 rrad_corr_coef(float cg) {
  const float g0 = 2.0f / 3.0f;
  if (cg < 1.0f) {
    const float a = (cg / g0 - 1.0f) / (g0 - 1.0f);
    return make_float2(a, 1.0f - a);
  }
  const float al = (cg - 1.0f) / (g0 - 1.0f);
  return make_float2(al, 1.0f - al);
}

// corrected_gshift_fluxboost_factor / g (Relreturn_Corona.cpp:37-86), FP32; ab from rrad_corr_coef(cg)
__device__ __forceinline__ float rrad_corrected_boost_over_g(float cg, float2 ab, float g, float lg, float gamma) {
  float gc;
  if (cg < 1.0f) {
    if (g >= 1.0f) {
      const float ig = 1.0f / g;
      gc = ig * (ig * ab.x + ab.y);
    } else {
      gc = g * (g * ab.x + ab.y);
    }
  } else {
    gc = (g >= 1.0f) ? (1.0f / g * ab.x + ab.y) : (g * ab.x + ab.y);
  }
  float fb = exp2f(gamma * lg) * gc;
  if (g < 1.0f && fb > 1.0f) fb = 1.0f;
  if (fb < 0.0f) fb = 0.0f;
  return fb / g;
}

// calc_rrad_emis_corona (Relreturn_Corona.cpp:125-160) on the table bins: er[i] = sum_j
// h(i, j) tf_r[i][j] emis_in[j] (times the flux correction of bin i), h(i, j) = sum over the g
// samples of frac_g times g^(gamma-1), or the corrected boost / g where the emitting bin's
// g-shift correction differs from 1 by more than 1e-3.  One warp per incident bin, lanes over
// the emitting bins, FP32, a fixed reduction order.
__device__ void rrad_pass(const RelxTables &tab, RradSmem &q, float gamma, bool corr) {
  const int NR = RELX_RR_NR, NG = RELX_RR_NG;
  const int n = q.n, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double *tfr = tab.rr_tfr + (size_t) q.spin * NR * NR;
  const float4 *gt = tab.rr_g + (size_t) q.spin * NR * NR * NG;
  for (int i = warp; i < n; i += kSetupThreads / 32) {
    const int ro = q.klo + i;
    float acc = 0.0f;
    for (int j = lane; j < n; j += 32) {
      const int re = q.klo + j;
      double t = tfr[(size_t) ro * NR + re];
      if (j == 0 && i < n - 1) t *= q.area_in;   // get_interpolated_tfr (Relreturn_Table.cpp:540-572)
      if (j == n - 1 && i < n - 2) t *= q.area_out;
      const float4 *g = gt + (size_t) ro * NG * NR + re;  // sample k at g[k * NR]
      const bool use_corr = corr && q.use_corr[j];
      const float cg = corr ? q.cg_f[j] : 1.0f;
      const float2 ab = rrad_corr_coef(cg);
      float h = 0.0f;
#pragma unroll 5
      for (int k = 0; k < NG; k++) {
        const float4 v = __ldg(g + (size_t) k * NR);  // frac_g, g, log2 g, |g - 1| > 1e-3
        float e = v.x;
        if (use_corr) e *= rrad_corrected_boost_over_g(cg, ab, v.y, v.z, gamma);
        else if (v.w != 0.0f) e *= exp2f((gamma - 1.0f) * v.z);
        h += e;
      }
      acc += h * d2f(t) * q.emis_in[j];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) q.er[i] = corr ? acc * q.cf_flux[i] : acc;
  }
}

// rebin_emisprofile_on_radial_grid of the table-bin profile onto fine radius r (Rellp.cpp:120-175):
// bins clamped to [0, n-2], linear radial factor (the profile's emission angles are 0), logarithmic
// interpolation of the emissivity
__device__ __forceinline__ double rrad_at(const RradSmem &q, double r) {
  const int kk = bsearch_asc_pos(q.rad, q.n, r);
  const float inter = d2f(r - q.rad[kk]) * d2f(q.inv_drad[kk]);
  return f2d(q.er[kk] * exp2f(inter * q.dl[kk]));
}

// the ionisation and density of zone z without an emissivity-based gradient: a power law in the
// zone's mean radius (ion_grad_type 1, IonGradient.cpp:128-138) or the set's values, clamped to
// the table's logxi range
__device__ void zone_ionisation(SetupSmem &m, const RelxSetState &s, int z) {
  if (s.ion_grad_type == 1) {
    double l = exp(m.lxi) * pow(m.rmean[z] / (0.5 * (s.rgrid[0] + s.rgrid[1])), -1.0 * m.iongrad_index);
    m.zlxi[z] = log(l);
  } else {
    m.zlxi[z] = m.lxi;
  }
  m.zdens[z] = m.dens;
  if (m.zlxi[z] < 0.0) m.zlxi[z] = 0.0;
  else if (m.zlxi[z] > 4.7) m.zlxi[z] = 4.7;
}

__global__ void __launch_bounds__(kSetupThreads, 4) setup_kernel(RelxTables tab, int model, const RelxSetIn *__restrict__ sin,
                                                               const double *__restrict__ user_e, double *__restrict__ line_e,
                                                               RelxSetState *__restrict__ sout, RelxRadial *__restrict__ rout,
                                                               RelxCorners *__restrict__ cout, RelxZoneCorners *__restrict__ zcout) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SetupSmem &m = *reinterpret_cast<SetupSmem *>(smem_raw);
  RelxSetState &s = m.s;
  const int set = blockIdx.x;
  const int tid = threadIdx.x;
  const RelxSetIn &in = sin[set];
  const int NR = RELX_NFRAD;
  const int kind = relx_kind(model);

  if (tid == 0) {
    map_params(model, in, m);
    m.status = s.status;
  }
  for (int z = tid; z < RELX_NZMAX; z += kSetupThreads) { m.zlo[z] = 1 << 30; m.zhi[z] = -1; }
  __syncthreads();
  if (m.status != RELX_OK) {
    if (tid == 0) { s.win_lo = 0; s.win_hi = 0; s.nz = 0; sout[set] = s; }
    return;
  }

  // ---- line-profile grid: user grid (redshift, 1 keV line) for relline, conv grid otherwise
  const double *ge;
  int gn;
  if (kind == RELX_RELLINE) {
    const double *ue = user_e + in.e_off;
    double *le = line_e + in.e_off;
    gn = in.n_ener;
    for (int j = tid; j <= gn; j += kSetupThreads) {
      double e = ue[j];
      if (s.z > 0) e *= (1 + s.z);       // shift_energy_grid_redshift, XspecSpectrum.h:70-76
      le[j] = e / s.lineE;               // shift_energy_grid_1keV, XspecSpectrum.h:61-65
    }
    ge = le;
  } else {
    ge = tab.conv_e;
    gn = RELX_NCONV;
  }

  // ---- relline table in the (a, mu0) plane on the table radii (Relprofile.cpp:159-223)
  const int nr = tab.rel_nr, nm = tab.rel_nmu0;
  if (tid == 32) {  // warp 1, beside warp 0's zone grid
    double mu0 = cos(s.incl);
    const float af = d2f(s.a), muf = d2f(mu0);
    int ia = bsearch_asc<float>(tab.rel_a, tab.rel_na, af);
    int im = bsearch_asc<float>(tab.rel_mu0, nm, muf);
    s.ind_a = ia;
    s.ind_mu0 = im;
    s.ifac_a = (af - tab.rel_a[ia]) / (tab.rel_a[ia + 1] - tab.rel_a[ia]);
    s.ifac_mu0 = (muf - tab.rel_mu0[im]) / (tab.rel_mu0[im + 1] - tab.rel_mu0[im]);
    s.g_n = gn;
  }
  if (tid == 96) {  // warp 3: the set's FP64 constants of the per-radius loops, computed once
    m.fg_r1 = 1.0 / sqrt(s.rout);
    m.fg_du = (1.0 / sqrt(s.rin) - m.fg_r1) / (NR - 1);
    if (s.emis_type == RELX_EMIS_LP) {
      const double hh = s.height, aa = s.a;
      m.ut_h = (float) sqrt((hh * hh + aa * aa) / (hh * hh - 2 * hh + aa * aa));
    } else {
      m.inv_rbr = (float) (1.0 / m.rbr);
    }
  }
  __syncthreads();
  // warp 0: the zone grid, then the zone means and, where they need no emission angle, the zones'
  // energy shifts and ionisation (IonGradient.cpp:128-171, 340-390); warp 2: g_inf^Gamma.  Both are
  // FP64 chains on a few lanes; the other warps start the table interpolation and the fine grid,
  // which need neither, and warps 0 and 2 join them after.
  const bool early_shift = s.emis_type != RELX_EMIS_LP || fabs(s.beta) < 1e-6;
  if (tid < 32) {
    zone_grid_warp(s.rin, s.rout, s.nz, s.height, s.rgrid);
    if (m.is_relxill) {
      for (int z = tid; z < s.nz; z += 32) {
        m.rmean[z] = 0.5 * (s.rgrid[z] + s.rgrid[z + 1]);
        if (early_shift)  // a source at rest: gi_potential_lp does not read the emission angle
          m.shift[z] = (s.emis_type == RELX_EMIS_LP) ? gi_potential_lp(m.rmean[z], s.a, s.height, s.beta, 0.0) : 1.0;
        if (s.ion_grad_type != 2) zone_ionisation(m, s, z);
      }
    }
  }
  if (tid == 64) m.ginf_pow = pow(s.g_inf, s.gam);
  {
    const size_t b00 = (size_t) s.ind_a * nm + s.ind_mu0, b10 = (size_t) (s.ind_a + 1) * nm + s.ind_mu0;
    const size_t b01 = b00 + 1, b11 = b10 + 1;
    const double fa = f2d(s.ifac_a), fm = f2d(s.ifac_mu0);
    for (int i = tid; i < nr; i += kSetupThreads) {
      // the float table values widened on the integer pipes (f2d is exact)
      m.re_tab[i] = lerp1(fa, f2d(tab.rel_r[b00 * nr + i]), f2d(tab.rel_r[b10 * nr + i]));
      m.gmin_t[i] = lerp2(fa, fm, f2d(tab.rel_gmin[b00 * nr + i]), f2d(tab.rel_gmin[b10 * nr + i]),
                          f2d(tab.rel_gmin[b01 * nr + i]), f2d(tab.rel_gmin[b11 * nr + i]));
      m.gmax_t[i] = lerp2(fa, fm, f2d(tab.rel_gmax[b00 * nr + i]), f2d(tab.rel_gmax[b10 * nr + i]),
                          f2d(tab.rel_gmax[b01 * nr + i]), f2d(tab.rel_gmax[b11 * nr + i]));
    }
  }
  // fine radial grid (relutility.c:666-677)
  {
    const double r1 = m.fg_r1, du = m.fg_du;  // 1/sqrt(rout) and the step in u
    for (int ii = tid; ii < NR; ii += kSetupThreads) {
      double u = f2d((float) ii) * du + r1;  // ii < 2^24: exact
      // 1/u: the float reciprocal refined by two Newton steps in FP64 (within an ulp of the
      // correctly rounded quotient)
      double iu = f2d(__frcp_rn(d2f(u)));
      iu = fma(iu, fma(-u, iu, 1.0), iu);
      iu = fma(iu, fma(-u, iu, 1.0), iu);
      m.re[ii] = iu * iu;
      m.sqre[ii] = iu;
    }
  }
  __syncthreads();
  if (tid == 0) {
    // (re - rms) / re < 1e-3 as a product: a division is a long FP64 chain on one thread
    const double rms = m.rms, rl = m.re_tab[nr - 1];
    if (rl > rms && (rl - rms) < 1e-3 * rl) m.re_tab[nr - 1] = rms;
    m.ind_rmin = bsearch_desc_pos(m.re_tab, nr, s.rin);
    m.ind_rmax = bsearch_desc_pos(m.re_tab, nr, s.rout);
    if (m.re_tab[m.ind_rmax] < 1000.0 && m.re_tab[m.ind_rmax] * 1.01 > 1000.0) m.re_tab[m.ind_rmax] = 1000.0;
  }
  __syncthreads();
  for (int i = tid; i < nr - 1; i += kSetupThreads) {
    m.inv_dtab[i] = 1.0 / (m.re_tab[i] - m.re_tab[i + 1]);
    m.dgmin_t[i] = m.gmin_t[i] - m.gmin_t[i + 1];  // the interpolation below as lo + f (hi - lo)
    m.dgmax_t[i] = m.gmax_t[i] - m.gmax_t[i + 1];
  }
  __syncthreads();

  RelxRadial &R = rout[set];
  // ---- per fine radius: table radius, interpolation factor, gmin/gmax, weight, zone, bin range.
  // FP64 arithmetic for the interpolation factor and gmin/gmax as the reference computes them (the
  // radial factor and the line's energy range); conversions and comparisons of these positive
  // values on the integer pipes (d2f, dgt); the trapezoid weight from a float-float difference of
  // neighbouring radii.
  int my_lo = 1 << 30, my_hi = -1;
  const double ge0 = ge[0], gen = ge[gn];
  const float wt_c = (float) (kPi / 2);
  for (int ii = tid; ii < NR; ii += kSetupThreads) {
    const double r = m.re[ii];
    // index ind with re_tab[ind+1] <= r < re_tab[ind], as the walk of Relprofile.cpp:252-266
    const int lo = count_gt_desc_pos(m.re_tab, nr, r);  // count of table radii > r
    int ind = lo - 1;
    if (ind > m.ind_rmin) ind = m.ind_rmin;
    if (ind < 0) {
      if (r - RELX_RELTABLE_MAX_R <= 1e-6) ind = 0; else atomicExch(&m.status, RELX_ERR_GRID);
    }
    if (ind < 0) ind = 0;
    const double ifac = (r - m.re_tab[ind + 1]) * m.inv_dtab[ind];
    if (ind > 0 && dgt(ifac, 1.0)) atomicExch(&m.status, RELX_ERR_GRID);
    // interp_lin_1d (relutility.c:24-26) as lo + f (hi - lo), one FMA each
    const double gmn = fma(ifac, m.dgmin_t[ind], m.gmin_t[ind + 1]);
    const double gmx = fma(ifac, m.dgmax_t[ind], m.gmax_t[ind + 1]);
    const double dg = gmx - gmn;
    R.re[ii] = r;
    R.ifac[ii] = ifac;
    RelxRadRec rr;
    rr.gmin = ff_split(gmn);
    rr.gmax = ff_split(gmx);
    rr.dg = ff_split(dg);
    rr.inv_dg = 1.0f / d2f(dg);
    {  // gstar2ener(H) and gstar2ener(1 - H) in float-float from the splits (FP32 pipe)
      rr.eH = ff_add(rr.gmin, ff_mul(rr.dg, ff_split(RELX_GFAC_H)));
      rr.e1H = ff_add(rr.gmin, ff_mul(rr.dg, ff_split(1 - RELX_GFAC_H)));
      rr.red_H = ff_ge(rr.eH, ff_split(0.95)) ? 1 : 0;
    }
    rr.itab = (short) ind;
    rr.ifac = d2f(ifac);
    rr.ew = 0.0f;  // set with the emissivity below
    // trapez_integ_single / 2 (relutility.c:233-244): r * dr * pi / 2 with dr half the difference of
    // the neighbouring radii (one-sided at the ends), from their float-float splits (the high words
    // of neighbouring radii differ by less than a factor 2, so their difference is exact)
    {
      const int ia = (ii == 0) ? 0 : ii - 1, ib = (ii == NR - 1) ? NR - 1 : ii + 1;
      const float dr = 0.5f * ff_diff(ff_split(m.re[ia]), ff_split(m.re[ib]));
      R.wt[ii] = d2f(r) * dr * wt_c;
    }
    rr.zone = (unsigned char) bsearch_asc_pos(s.rgrid, s.nz + 1, r);
    // bins of the line-profile grid touched by this radius (Relprofile.cpp:863-878)
    int ielo = -1, iehi = -1;
    if (dgt(gmx, ge0) && dgt(gen, gmn)) {
      const double egmin = dgt(ge0, gmn) ? ge0 : gmn;
      const double egmax = dgt(gmx, gen) ? gen : gmx;
      if (kind == RELX_RELLINE) {
        ielo = bsearch_asc_pos(ge, gn + 1, egmin);
        iehi = bsearch_asc_pos(ge, gn + 1, egmax);
      } else {
        ielo = conv_index(tab, egmin);
        iehi = conv_index(tab, egmax);
      }
      my_lo = min(my_lo, ielo);
      my_hi = max(my_hi, iehi);
      atomicMin(&m.zlo[rr.zone], ielo);
      atomicMax(&m.zhi[rr.zone], iehi);
    }
    rr.ielo = ielo;
    rr.iehi = iehi;
    R.rec[ii] = rr;
  }
  int wlo = block_min_i<kSetupThreads>(my_lo, m.ired);
  int whi = block_max_i<kSetupThreads>(my_hi, m.ired);
  if (tid == 0) {
    s.win_lo = (whi >= 0) ? wlo : 0;
    s.win_hi = (whi >= 0) ? whi + 1 : 0;
  }
  for (int z = tid; z < s.nz; z += kSetupThreads) {
    // profile bins outside a zone's window stay exactly zero
    s.zw_lo[z] = (m.zhi[z] >= 0) ? m.zlo[z] : s.win_lo;
    s.zw_hi[z] = (m.zhi[z] >= 0) ? m.zhi[z] + 1 : s.win_lo;
  }

  // ---- emissivity
  if (s.emis_type == RELX_EMIS_BKN) {
    // get_emis_bkn + norm_emis_profile (Rellp.cpp:91-109,421-437)
    // the power law in FP32 (r / Rbr as a float product), the normalisation integral sum(e 4 wt)
    // as a float-float sum per thread (wt = r dr pi / 2 from the records above)
    const float inv_rbr = m.inv_rbr;
    const float a1 = d2f(-m.emis1), a2 = d2f(-m.emis2);
    float2 part = make_float2(0.0f, 0.0f);
    for (int ii = tid; ii < NR; ii += kSetupThreads) {
      const double r = m.re[ii];
      const float e = powf(d2f(r) * inv_rbr, dgt(r, m.rbr) ? a2 : a1);
      m.pr.emis[ii] = e;
      m.pr.del_emit[ii] = -1.0f;
      m.pr.del_inc[ii] = -1.0f;
      part = ff_add(part, ff_mulf(make_float2(e, 0.0f), 4.0f * R.wt[ii]));
    }
    const double inv_integ = 1.0 / block_sum_d<kSetupThreads>(ff_to_double(part), m.red);
    for (int ii = tid; ii < NR; ii += kSetupThreads) m.pr.emis[ii] = d2f(f2d(m.pr.emis[ii]) * inv_integ);
    __syncthreads();
    if (tid == 0) { s.f_inf_rest = 0; s.refl_frac_lp = 0; }
  } else {
    // lamp post: interpol_lptable (Rellp.cpp:190-247)
    const int nh = tab.lp_nh, nrad = tab.lp_nrad;
    if (tid == 0) {
      float fa = d2f(s.a);
      int ia = bsearch_asc<float>(tab.lp_a, tab.lp_na, fa);
      m.lp_ind_a = ia;
      m.lp_ifac_a = (fa - tab.lp_a[ia]) / (tab.lp_a[ia + 1] - tab.lp_a[ia]);
      float fh = d2f(s.height);
      for (int q = 0; q < 2; q++) {
        const float *hg = tab.lp_h + (size_t) (ia + q) * nh;
        int ih = bsearch_asc<float>(hg, nh, fh);
        m.ind_h[q] = ih;
        m.ifac_h[q] = (fh - hg[ih]) / (hg[ih + 1] - hg[ih]);
      }
    }
    __syncthreads();
    {
      const int ia = m.lp_ind_a;
      const double fa = m.lp_ifac_a;
      const float faf = d2f(fa), f0f = d2f(m.ifac_h[0]), f1f = d2f(m.ifac_h[1]);
      for (int k = tid; k < nrad; k += kSetupThreads) {
        m.jet_rad[k] = lerp1(fa, f2d(tab.lp_rad[(size_t) ia * nrad + k]), f2d(tab.lp_rad[(size_t) (ia + 1) * nrad + k]));
#define TV(arr, q, h) (arr)[(((size_t) (ia + (q)) * nh) + (h)) * nrad + k]
        const int h0 = m.ind_h[0], h1 = m.ind_h[1];
        const double f0 = m.ifac_h[0], f1 = m.ifac_h[1];
        // the emission angle decides the radial interpolation mode and the reflection fraction: FP64;
        // the intensity and the incidence angle only enter FP32 arithmetic: FP32
        m.d_tab[k] = (1.0 - fa) * lerp1(f0, f2d(TV(tab.lp_del, 0, h0)), f2d(TV(tab.lp_del, 0, h0 + 1)))
            + fa * lerp1(f1, f2d(TV(tab.lp_del, 1, h1)), f2d(TV(tab.lp_del, 1, h1 + 1)));
        m.lp_e[k] = (1.0f - faf) * lerp1(f0f, TV(tab.lp_intens, 0, h0), TV(tab.lp_intens, 0, h0 + 1))
            + faf * lerp1(f1f, TV(tab.lp_intens, 1, h1), TV(tab.lp_intens, 1, h1 + 1));
        m.lp_di[k] = (1.0f - faf) * lerp1(f0f, TV(tab.lp_delinc, 0, h0), TV(tab.lp_delinc, 0, h0 + 1))
            + faf * lerp1(f1f, TV(tab.lp_delinc, 1, h1), TV(tab.lp_delinc, 1, h1 + 1));
#undef TV
      }
    }
    __syncthreads();
    for (int k = tid; k < nrad; k += kSetupThreads) {
      if (k < nrad - 1) {
        const float djr = d2f(m.jet_rad[k + 1] - m.jet_rad[k]);
        m.inv_drad_f[k] = 1.0f / djr;
        m.lp_dle[k] = logf(m.lp_e[k + 1] / m.lp_e[k]);                        // log e_hi - log e_lo
        m.lp_dlr[k] = log1pf(djr / d2f(m.jet_rad[k]));  // log r_hi - log r_lo (no FP64 division)
      }
      m.jet_rad_f[k] = d2f(m.jet_rad[k]);
      m.inv_jr_f[k] = 1.0f / m.jet_rad_f[k];
      m.lp_d[k] = d2f(m.d_tab[k]);
      m.lp_log[k] = dgt(m.d_tab[k], kDeg75) ? 1 : 0;  // emission angle above 75 degrees
    }
    __syncthreads();
    // rebin_emisprofile_on_radial_grid (Rellp.cpp:120-175) and the flux boost of the emissivity
    // (apply_emis_fluxboost_source_disk, Rellp.cpp:249-253, Relphysics.cpp:301-311) per fine radius.
    // gi_potential_lp with sqrt(r) = 1/u of the fine grid; r^2 - 3r + 2a sqrt(r) cancels near the
    // ISCO and stays FP64, as do r - rlo and r^1.5 + a; the rest runs in FP32.
    const double hh = s.height, aa = s.a;
    const float ut_h = m.ut_h;
    const bool moving = fabs(s.beta) >= 1e-6, boosted = s.beta > 1e-6;
    const float gam_f = d2f(s.gamma);
    const double jr_last = m.jet_rad[nrad - 1];
    for (int ii = tid; ii < NR; ii += kSetupThreads) {
      const double r = m.re[ii], sr = m.sqre[ii];
      const int kk = bsearch_asc_pos(m.jet_rad, nrad, r);
      if (dge(r, jr_last) && r - RELX_RELTABLE_MAX_R > 1e-6) atomicExch(&m.status, RELX_ERR_GRID);
      // get_ipol_factor_radius (relutility.c:407-417)
      const float dr = d2f(r - m.jet_rad[kk]);
      float inter;
      if (!m.lp_log[kk]) {
        inter = dr * m.inv_drad_f[kk];
      } else {
        inter = log1pf(dr * m.inv_jr_f[kk]) / m.lp_dlr[kk];
      }
      const float del_e = inter * m.lp_d[kk + 1] + (1.0f - inter) * m.lp_d[kk];
      m.pr.del_emit[ii] = del_e;
      m.pr.del_inc[ii] = inter * m.lp_di[kk + 1] + (1.0f - inter) * m.lp_di[kk];
      const double t = r * r - 3 * r + 2 * aa * sr;
      const float srf = d2f(sr);
      const float ut_d = fmaf(d2f(r), srf, d2f(aa)) / (srf * sqrtf(d2f(t)));
      float gi = ut_d / ut_h;
      if (moving) gi = (float) gi_potential_lp(r, aa, hh, s.beta, f2d(del_e));
      float boost = powf(gi, gam_f);
      if (boosted) {
        const float d = (float) doppler_factor(f2d(del_e), s.beta);
        boost *= d * d;
      }
      // interp_log_1d (relutility.c:41-43) as e_lo * exp(inter * (log e_hi - log e_lo)), boosted
      m.pr.emis[ii] = m.lp_e[kk] * expf(inter * m.lp_dle[kk]) * boost;
    }
    __syncthreads();
    if (tid >= kSetupThreads - 32) {
      // calc_refl_frac (Rellp.cpp:36-89) on the last warp, which joins the next loops after it (its
      // results are read at the end); the three cosines on three lanes
      double ad_max = m.d_tab[nrad - 1];
      double del_bh = f2d(m.pr.del_emit[bsearch_desc_pos(m.re, NR, s.rin)]);
      double del_ad = f2d(m.pr.del_emit[bsearch_desc_pos(m.re, NR, s.rout)]);
      if (ad_max < kPi / 2.0) ad_max = kPi / 2.0;
      double ad_obs = ad_max;
      if (s.beta > 1e-6) {
        del_bh = relat_abberation(del_bh, -1. * s.beta);
        del_ad = relat_abberation(del_ad, -1. * s.beta);
        ad_obs = relat_abberation(ad_max, -1. * s.beta);
      }
      const int lane = tid & 31;
      const double cx = cos(lane == 0 ? del_bh : lane == 1 ? del_ad : lane == 2 ? ad_max : ad_obs);
      const double c_bh = __shfl_sync(0xffffffffu, cx, 0), c_ad = __shfl_sync(0xffffffffu, cx, 1);
      const double c_max = __shfl_sync(0xffffffffu, cx, 2), c_obs = __shfl_sync(0xffffffffu, cx, 3);
      if (lane == 0) {
        double f_ad = 0.5 * (c_bh - c_ad);
        s.f_inf_rest = 0.5 * (1.0 + c_max);
        double f_inf = (s.beta > 1e-6) ? 0.5 * (1.0 + c_obs) : s.f_inf_rest;
        s.refl_frac_lp = f_ad / f_inf;
      }
    }
  }
  // (the lamp-post branch ends behind a barrier after its per-radius loop)
  // ---- returning radiation without xillver corrections (calc_emis_profile, Rellp.cpp:556-558)
  const bool rrad = m.return_rad != 0 && m.status == RELX_OK;
  if (rrad) {
    if (tid == 0) {
      const int e = (tab.rr_nspin > 0) ? rrad_bins(tab, m.rt.rr, s.a, m.rms, m.re[NR - 1], m.re[0]) : RELX_ERR_TABLE;
      if (e != RELX_OK) m.status = e;
    }
    __syncthreads();
    if (m.status == RELX_OK) rrad_centres(tab, m.rt.rr, m.re[NR - 1], m.re[0], kSetupThreads);
  }
  if (rrad && m.status == RELX_OK) {
    RradSmem &q = m.rt.rr;
    for (int j = tid; j < q.n; j += kSetupThreads) q.emis_in[j] = d2f(rebin_mean_at(m.re, m.pr.emis, NR, q.rad[j]));
    __syncthreads();
    rrad_pass(tab, q, d2f(s.gamma), false);
    __syncthreads();
    for (int k = tid; k + 1 < q.n; k += kSetupThreads) q.dl[k] = log2f(q.er[k + 1] / q.er[k]);
    __syncthreads();
    for (int ii = tid; ii < NR; ii += kSetupThreads) {
      m.rt.emis_lp[ii] = m.pr.emis[ii];
      const double r = rrad_at(q, m.re[ii]);
      m.pr.emis[ii] = d2f((m.return_rad == 1) ? f2d(m.pr.emis[ii]) + r : r);
    }
    __syncthreads();
  }
  for (int ii = tid; ii < NR; ii += kSetupThreads) R.rec[ii].ew = m.pr.emis[ii] * R.wt[ii];

  // ---- zones: fine-radius index ranges (zone is non-increasing with the radius index)
  for (int z = tid; z < s.nz; z += kSetupThreads) { s.zi0[z] = 1; s.zi1[z] = 0; }
  __syncthreads();
  for (int ii = tid; ii < NR; ii += kSetupThreads) {
    const int z = R.rec[ii].zone;
    if (ii == 0 || R.rec[ii - 1].zone != z) s.zi0[z] = ii;
    if (ii == NR - 1 || R.rec[ii + 1].zone != z) s.zi1[z] = ii;
  }
  __syncthreads();
  // conv-grid bins the final rebin to the caller's grid reads (Relxill.cpp:267-278, Relbase.cpp:281-284)
  if (tid == 0 && kind != RELX_RELLINE) {
    const double *ue = user_e + in.e_off;
    double zf = (kind != RELX_RELCONV && s.z > 0) ? (1 + s.z) : 1.0;
    double elo = ue[0] * zf, ehi = ue[in.n_ener] * zf;
    const double *ce = tab.conv_e;
    int lo = conv_index(tab, elo);  // as bsearch_asc over the N + 1 edges
    int hi = conv_index(tab, ehi);
    if (in.flags & 2) {  // RELXILL_RENORMALIZE reads the bin at 3 keV
      int k3 = bsearch_asc<double>(ce, RELX_NCONV, 3.0);
      lo = min(lo, k3);
      hi = max(hi, k3);
    }
    s.out_lo = max(0, lo - 1);
    s.out_hi = min(RELX_NCONV - 1, hi + 1);
  }
  if (!m.is_relxill) {
    __syncthreads();
    if (tid == 0) {
      if (m.status != RELX_OK) s.status = m.status;
      s.src_norm = 0;
      sout[set] = s;
    }
    return;
  }

  // ---- ionisation gradient (IonGradient.cpp:128-211, 340-390)
  const int nz = s.nz;
  if (tid < nz && (!early_shift || s.ion_grad_type == 2)) {
    int z = tid;
    if (!early_shift) {
      m.zdel_emit[z] = rebin_mean_at(m.re, m.pr.del_emit, NR, m.rmean[z]);
      m.shift[z] = gi_potential_lp(m.rmean[z], s.a, s.height, s.beta, m.zdel_emit[z]);
    }
    if (s.ion_grad_type == 2) {
      double rin = s.rgrid[0];
      double irr = rebin_mean_at(m.re, m.pr.emis, NR, m.rmean[z]);
      double dinc = rebin_mean_at(m.re, m.pr.del_inc, NR, m.rmean[z]);
      double rad_lxi = (11. / 9.) * (11. / 9.) * rin;
      int kk = bsearch_desc(m.re, NR, rad_lxi);
      double ip = (rad_lxi - m.re[kk + 1]) / (m.re[kk] - m.re[kk + 1]);
      double emis_r = lerp1(ip, f2d(m.pr.emis[kk + 1]), f2d(m.pr.emis[kk]));
      double dinc_r = lerp1(ip, f2d(m.pr.del_inc[kk + 1]), f2d(m.pr.del_inc[kk]));
      double lxi_max = log10(4.0 * kPi * emis_r / density_ss73_zone_a(rad_lxi, rin) * (cos(kPi / 4) / cos(dinc_r)));
      double fac = m.lxi - lxi_max;
      double dmin = density_ss73_zone_a((25. / 9.) * rin, rin);
      double dn = (m.flags & 4) ? 1.0 : density_ss73_zone_a(m.rmean[z], rin) / dmin;
      m.zdens[z] = log10(dn) + m.dens;
      m.zlxi[z] = log10(4.0 * kPi * irr / dn * (cos(kPi / 4) / cos(dinc))) + fac;
      if (m.zlxi[z] < 0.0) m.zlxi[z] = 0.0;
      else if (m.zlxi[z] > 4.7) m.zlxi[z] = 4.7;
    }
  }
  __syncthreads();

  // ---- xillver brackets and factors per zone (xilltable.c:278-323, 1090-1142)
  const int npar = tab.x_npar;
  if (tid < nz) {
    int z = tid;
    double ect_z = s.ect_src * m.shift[z];
    float inp[10];
    for (int q = 0; q < 10; q++) inp[q] = 0.0f;
    inp[0] = d2f(s.gam);
    inp[1] = d2f(m.afe);
    inp[2] = d2f(m.zlxi[z]);
    inp[3] = d2f(ect_z);
    inp[4] = d2f(m.zdens[z]);
    inp[7] = (float) (s.incl * 180 / kPi);
    for (int q = 0; q < npar; q++) {
      const float *pv = tab.x_vals + q * tab.x_maxvals;
      int nv = tab.x_nvals[q];
      int pi = tab.x_pindex[q];
      int ind = bsearch_asc<float>(pv, nv, inp[pi]);
      if (ind < 0) ind = 0;
      else if (ind > nv - 2) ind = nv - 2;
      m.zind[z][q] = ind;
      float val = inp[pi];
      if (pi != 7) {
        if (val < pv[0]) val = pv[0];
        else if (val > pv[nv - 1]) val = pv[nv - 1];
      }
      float f = (val - pv[ind]) / (pv[ind + 1] - pv[ind]);
      m.zfac[z][q] = f2d(f);
      if (pi == 3) {  // ensure_ecut_within_boundarys (xilltable.c:1054-1067)
        if (!dgt(ect_z, f2d(pv[0]))) m.zfac[z][q] = 0.0;  // the Ecut grid is positive
        if (dge(ect_z, f2d(pv[nv - 1]))) m.zfac[z][q] = 1.0;
      }
    }
  }
  // ---- normalisation of the primary continuum (Xillspec.cpp:179-205, 302-332, 408-440): one warp
  // per continuum (source, then every zone), float-float sums of FP32 terms times the bin centre
  // The nthcomp continuum of the Cp models is normalised by nthcomp_kernel after this kernel
  // (nthcomp.cu), which also applies the zones' normalisation changes to their corner weights.
  for (int z = tid; z < nz; z += kSetupThreads) s.zshift[z] = m.shift[z];
  if (s.prim == 1) {
    if (tid == 0) s.src_norm = 0.0;
    for (int z = tid; z < nz; z += kSetupThreads) m.xscale[z] = 1.0;
  } else {
    const float gam = d2f(s.gam);
    const int lane = tid & 31, warp = tid >> 5;
    for (int b = tid; b < RELX_NCOARSE; b += kSetupThreads) m.cpow[b] = powf(tab.coarse_t[b].x, -gam);
    for (int qq = tid; qq <= nz; qq += kSetupThreads) m.qecut[qq] = d2f(s.ect_src * (qq == 0 ? 1.0 : m.shift[qq - 1]));
    __syncthreads();
    // the continua (the source, then the zones) in groups of kQGroup over the whole block: every
    // thread sums the terms of its coarse bins for each continuum of the group (independent sums),
    // the warps reduce with shuffles and one thread per continuum adds the warps' sums in warp order;
    // float-float sums of FP32 terms (calcNormWrtXillverTableSpec, Xillspec.cpp:179-233)
    for (int q0 = 0; q0 <= nz; q0 += kQGroup) {
      const int nq = min(kQGroup, nz + 1 - q0);
      float2 part[kQGroup];
      float ecut[kQGroup], e0[kQGroup];
#pragma unroll
      for (int k = 0; k < kQGroup; k++) {
        part[k] = make_float2(0.0f, 0.0f);
        ecut[k] = m.qecut[q0 + min(k, nq - 1)];
        e0[k] = expf(1.0f / ecut[k]);
      }
      for (int b = tid; b < RELX_NCOARSE; b += kSetupThreads) {
        const float4 t = tab.coarse_t[b];  // bin centre, width, centre as float-float (0 outside the band)
        const float pw = m.cpow[b];
#pragma unroll
        for (int k = 0; k < kQGroup; k++) {
          if (k < nq) {  // uniform over the block
            const float term = e0[k] * pw * expf(-t.x / ecut[k]) * t.y;
            part[k] = ff_add(part[k], ff_mulf(make_float2(t.z, t.w), term));
          }
        }
      }
#pragma unroll
      for (int k = 0; k < kQGroup; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          float2 u;
          u.x = __shfl_xor_sync(0xffffffffu, part[k].x, o);
          u.y = __shfl_xor_sync(0xffffffffu, part[k].y, o);
          part[k] = ff_add(part[k], u);
        }
        if (lane == 0) m.qpart[warp][k] = part[k];
      }
      __syncthreads();
      if (tid < nq) {
        float2 a = m.qpart[0][tid];
        for (int w = 1; w < kSetupThreads / 32; w++) a = ff_add(a, m.qpart[w][tid]);
        m.qsum[q0 + tid] = (f2d(a.x) + f2d(a.y)) * kQsumScale;
      }
      __syncthreads();
    }
    if (tid < 32) {  // one warp: the reciprocal is a chain of FP64 operations
      const double src_norm = 1.0 / m.qsum[0];
      if (tid == 0) s.src_norm = src_norm;
      for (int z = tid; z < nz; z += 32)
        m.xscale[z] = (m.shift[z] == 1.0) ? 1.0 : m.qsum[z + 1] * src_norm;  // 1 / (disk factor / source factor)
    }
  }
  __syncthreads();
  const int ni = tab.x_nincl;
  const bool six = tab.x_npar == 6;
  // corners per zone: 16 over parameters 0..3 of the 5-parameter table (interp_5d_tab_incl,
  // xilltable.c:812-876); 32 over parameters 0..4 of the 6-parameter table (the two 16-corner
  // blocks of interp_6d_tab_incl, xilltable.c:999-1020), which has a density parameter and so no
  // density division
  const int ncz = six ? 32 : 16, nbits = six ? 5 : 4;
  if (six && !tab.x_has_dens && tid == 0) m.status = RELX_ERR_TABLE;
  const bool listed = nz * ncz <= RELX_NZMAX * 16;  // the entries fit the de-duplication arrays
  if (!listed) {  // 6-parameter table and more than 25 zones: per-zone lists, no de-duplication
    for (int e = tid; e < nz * 32; e += kSetupThreads) {
      const int z = e >> 5, c = e & 31;
      long row = 0;
      double w = 1.0;
      for (int q = 0; q < 5; q++) {
        const int up = (c >> q) & 1;
        row = row * tab.x_nvals[q] + m.zind[z][q] + up;
        const double f = m.zfac[z][q];
        w *= up ? f : (1.0 - f);
      }
      zcout[set].row[z][c] = (int) (row * ni);
      zcout[set].w[z][c] = d2f(w * m.xscale[z]);
    }
    if (tid == 0) {
      s.ucount = 0;
      s.xdense = 0;
    }
  }
  // ---- the corners of every zone, first-zone density scaling, de-duplication
  const int ncor = listed ? nz * ncz : 0;
  for (int e = tid; e < ncor; e += kSetupThreads) {
    const int z = e / ncz, c = e - z * ncz;
    // corner c: bit q -> upper bracket of parameter q
    long row = 0;
    for (int q = 0; q < nbits; q++) row = row * tab.x_nvals[q] + m.zind[z][q] + ((c >> q) & 1);
    row = row * ni;  // incl index 0
    m.cr.crow[e] = (int) row;
  }
  __syncthreads();
  for (int e = tid; e < ncor; e += kSetupThreads) {
    int first = e;
    for (int f = 0; f < e; f++)
      if (m.cr.crow[f] == m.cr.crow[e]) { first = f; break; }
    m.cr.cfirst[e] = (short) first;
  }
  __syncthreads();
  for (int e = tid; e < ncor; e += kSetupThreads) {
    const int z = e / ncz, c = e - z * ncz;
    double w = 1.0;
    for (int q = 0; q < nbits; q++) {
      double f = m.zfac[z][q];
      w *= ((c >> q) & 1) ? f : (1.0 - f);
    }
    // density division of the row by the zone that loads it first (xilltable.c:478-511)
    double dscale = 1.0;
    if (!tab.x_has_dens) {
      double d = m.zdens[m.cr.cfirst[e] / ncz];
      if (fabs(d - 15) > 1e-6) dscale = 1.0 / pow(10.0, d - 15);
    }
    m.cr.cw[e] = d2f(w * dscale * m.xscale[z]);
    m.cr.clive[e] = 0;
  }
  __syncthreads();
  // a row is read only if some zone gives it a non-zero weight (a parameter on a grid value
  // puts exactly zero weight on the upper bracket)
  for (int e = tid; e < ncor; e += kSetupThreads)
    if (m.cr.cw[e] != 0.0f) m.cr.clive[m.cr.cfirst[e]] = 1;
  __syncthreads();
  if (tid < 32 && listed) {  // number the live rows in entry order (warp prefix sums)
    const int lane = tid;
    int base = 0;
    for (int e0 = 0; e0 < ncor; e0 += 32) {
      const int e = e0 + lane;
      const bool first = e < ncor && m.cr.cfirst[e] == e;
      const bool live = first && m.cr.clive[e];
      const unsigned int mask = __ballot_sync(0xffffffffu, live);
      if (first) m.cr.cuniq[e] = live ? (short) (base + __popc(mask & ((1u << lane) - 1u))) : (short) -1;
      base += __popc(mask);
    }
    if (lane == 0) {
      s.ucount = base;
      m.ired[0] = base;
    }
  }
  __syncthreads();
  for (int e = tid; e < ncor; e += kSetupThreads)
    if (m.cr.cfirst[e] != e) m.cr.cuniq[e] = m.cr.cuniq[m.cr.cfirst[e]];  // the first entry is numbered above
  // dense: at most RELX_ZDENSE zones and RELX_MAX_UCORNER distinct live rows (always so for the
  // 5-parameter table: 16 corners x 16 zones)
  const bool dense = listed && nz <= RELX_ZDENSE && m.ired[0] <= RELX_MAX_UCORNER;
  __syncthreads();
  if (tid == 0 && listed) s.xdense = dense ? 1 : 0;
  if (dense) {
    RelxCorners &C = cout[set];
    for (int i = tid; i < RELX_MAX_UCORNER * RELX_ZDENSE; i += kSetupThreads) (&C.w[0][0])[i] = 0.0f;
    __syncthreads();
  }
  for (int e = tid; e < ncor; e += kSetupThreads) {
    const int z = e / ncz, c = e - z * ncz;
    if (dense) {
      RelxCorners &C = cout[set];
      const int u = m.cr.cuniq[e];
      if (u >= 0) {
        C.w[u][z] = m.cr.cw[e];  // each (u, z) pair is written by exactly one entry
        if (m.cr.cfirst[e] == e) C.row[u] = m.cr.crow[e];
      }
    } else {
      zcout[set].row[z][c] = m.cr.crow[e];
      zcout[set].w[z][c] = m.cr.cw[e];
    }
  }
  // ---- returning radiation with the xillver flux-correction factors of the zones, for relxill models
  // with a > 0 (Relxill.cpp:336-344, Relxill.h:32): the line profile uses this emissivity, the zones
  // keep the one above
  if (rrad && m.is_relxill && s.a > 0.0 && m.status == RELX_OK) {
    RradSmem &q = m.rt.rr;
    // get_xillver_fluxcorrection_factors (Xillspec.cpp:500-526) from per-corner integrals: a warp per
    // zone, a lane per corner, the corner terms summed across the lanes; the factors themselves in
    // FP32 (they enter the FP32 returning-radiation pass)
    const int nq = tab.x_npar - 1, ncorner = 1 << nq;  // parameters bracketed per corner (<= 5)
    const int lane = tid & 31, warp = tid >> 5;
    const float p15 = powf(1.5f, d2f(s.gam));
    for (int z = warp; z < nz; z += kSetupThreads / 32) {
      double ef = 0.0, pf = 0.0, pfz = 0.0;
      if (lane < ncorner) {
        const int c = lane;
        double w = 1.0;
        long corner = 0;
        for (int qq = 0; qq < nq; qq++) {
          const double f = m.zfac[z][qq];
          const int up = (c >> qq) & 1;
          w *= up ? f : (1.0 - f);
          corner = corner * tab.x_nvals[qq] + m.zind[z][qq] + up;
        }
        if (w != 0.0) {
          if (!tab.x_has_dens) {
            const double d = m.zdens[m.cr.cfirst[z * 16 + c] >> 4];
            if (fabs(d - 15) > 1e-6) w *= 1.0 / pow(10.0, d - 15);
          }
          const double *fc = tab.x_fcorr + (size_t) corner * 3;
          ef = w * fc[0];
          pf = w * fc[1];
          pfz = w * fc[2];
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ef += __shfl_xor_sync(0xffffffffu, ef, o);
        pf += __shfl_xor_sync(0xffffffffu, pf, o);
        pfz += __shfl_xor_sync(0xffffffffu, pfz, o);
      }
      if (lane == 0) {
        // energy flux of the normalised direct spectrum in 0.1-1000 keV: the table normalisation,
        // less the coarse bins outside that band (Xillspec.cpp:179-205, 344-361)
        const float ecut = d2f(s.ect_src * m.shift[z]);
        double x = 0.0;
        for (int e2 = 0; e2 < 2; e2++) {
          const int b = tab.coarse_b2_skip[e2];
          if (b < 0) continue;
          if (s.prim == 1) {  // the end-bin correction is only restated for the cut-off power law
            m.status = RELX_ERR_UNSUPPORTED;
            continue;
          }
          const float4 t = tab.coarse_t[b];
          const float term = expf(1.0f / ecut) * m.cpow[b] * expf(-t.x / ecut) * t.y;
          x += f2d(term) * (f2d(t.z) + f2d(t.w));
        }
        // the normalisation sum qz exists for the cut-off power law only (the nthcomp continuum has
        // no end bins to take off here)
        float ef_direct = (float) ((1e15 / 4.0 / kPi) / (1e20 * 1.602177e-09));
        if (x != 0.0) ef_direct -= d2f(x) / d2f((m.shift[z] == 1.0) ? m.qsum[0] : m.qsum[z + 1]);
        q.zcf_flux[z] = f2d(d2f(ef) / ef_direct);
        q.zcf_g[z] = f2d(d2f(pf) / d2f(pfz) / p15);
      }
    }
    __syncthreads();
    for (int k = tid; k < q.n; k += kSetupThreads) {  // rebin_to_grid (Relreturn_Corona.cpp:208-222)
      int zi = bsearch_asc_pos(s.rgrid, nz + 1, q.rad[k]);
      if (q.rad[k] < s.rgrid[0]) zi = 0;
      else if (q.rad[k] > s.rgrid[nz]) zi = nz - 1;
      q.cf_flux[k] = d2f(q.zcf_flux[zi]);
      q.cg_f[k] = d2f(q.zcf_g[zi]);
      q.use_corr[k] = fabs(q.zcf_g[zi] - 1) > 1e-3;
    }
    __syncthreads();
    rrad_pass(tab, q, d2f(s.gamma), true);
    __syncthreads();
    for (int k = tid; k + 1 < q.n; k += kSetupThreads) q.dl[k] = log2f(q.er[k + 1] / q.er[k]);
    __syncthreads();
    for (int ii = tid; ii < NR; ii += kSetupThreads) {
      const double r = rrad_at(q, m.re[ii]);
      const double e = (m.return_rad == 1) ? f2d(m.rt.emis_lp[ii]) + r : r;
      R.rec[ii].ew = d2f(e) * R.wt[ii];
    }
    if (tid == 0) s.rr_corr = 1;
  }
  // ---- primary and reflection factors (PrimarySource.cpp:66-125)
  if (tid == 0) {
    if (s.emis_type != RELX_EMIS_LP) {
      s.norm_fac_refl = fabs(s.refl_frac);
      s.prim_fac = 1.0;
    } else {
      double rfi = s.refl_frac;
      if (s.boost_switch) rfi *= s.refl_frac_lp;
      double pf = s.f_inf_rest / 0.5 * m.ginf_pow;
      if (s.beta > 1e-4) {
        double d = doppler_factor(kPi - s.incl, s.beta);
        pf *= d * d;
      }
      s.prim_fac = pf;
      s.norm_fac_refl = fabs(rfi) / s.refl_frac_lp;
    }
    for (int z = 0; z < nz; z++) s.inv_nc[z] = d2f(m.xscale[z]);
    if (m.status != RELX_OK) s.status = m.status;
  }
  __syncthreads();
  {  // the set state out, by all threads
    static_assert(sizeof(RelxSetState) % 8 == 0, "copied as 8-byte words");
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(&s);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(&sout[set]);
    for (int i = tid; i < (int) (sizeof(RelxSetState) / 8); i += kSetupThreads) dst[i] = src[i];
  }
}

size_t setup_smem_bytes() { return sizeof(SetupSmem); }

}  // namespace relx
