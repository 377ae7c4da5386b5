// nthcomp.cu -- the nthcomp continuum of the Cp models on the GPU.
//
// nthcomp (donthcomp.c) is thermal Comptonization of disk-blackbody seed
// photons: the Kompaneets equation with relativistic corrections, discretised
// on a logarithmic photon-energy grid (0.02 dex) and solved as one tridiagonal
// system (Lightman & Zdziarski 1987; Zdziarski, Johnson & Magdziarz 1996;
// Zycki, Done & Smith 1999).  The Cp models evaluate it with a seed
// temperature of 0.05 keV (get_nthcomp_param, relutility.c:625-631) for the
// primary continuum and for the normalisation of every zone's continuum
// (kTe times the zone's energy shift, Xillspec.cpp:243-253, 408-440).
//
// With the seed temperature fixed, the photon grid, Cooper's coefficient, the
// Klein-Nishina factor and the disk-blackbody seed spectrum do not depend on
// kTe or Gamma: they are computed once on the host in FP64 (NthGrid), as are
// the weights that turn an E F_E table into its normalisation on the 500-bin
// coarse grid (calcNormWrtXillverTableSpec, Xillspec.cpp:179-205): that
// normalisation is linear in the table, sum_j G_j sp_j times the inverse of the
// table at the 1 keV point.
//
// nthcomp_kernel: one thread per continuum (the source, and each zone whose
// energy shift differs from 1).  The tridiagonal coefficients are formed on
// the fly from the grid and the continuum's tautom and theta, and the system
// is solved by the Thomas algorithm (thermlc, donthcomp.c:194-280) in
// float-float arithmetic on the FP32 pipe (about 48 significant bits; the FP64
// pipe of this part runs at 1/64 of the FP32 rate).  The forward sweep keeps
// its two recurrences per point in a scratch laid out [point][continuum], so a
// warp's accesses are contiguous; the back sweep recovers the solution, forms
// E F_E (donthcomp.c:603-610) and accumulates the normalisation.  The source
// continuum also writes its table for the primary spectrum (c_donthcomp,
// donthcomp.c:640-793).
// nthcomp_apply_kernel: the normalisation changes of the zones on their corner
// weights and the source normalisation of the primary.
#include <cmath>
#include <vector>

#include "relx_device.cuh"
#include "relx_kernels.h"

namespace relx {

constexpr int kNthThreads = 128;
constexpr int kNthMaxJ = 899;  // the reference's largest grid index (donthcomp.c:360)

static double lg10_h(double x) { return 0.43429448190325182765 * std::log(x); }

// residuals of the multi-colour disk interpolation formula in 0.06 dex steps from E/T = 1e-3
// (Mitsuda et al. 1984; the table of donthcomp.c:57-79)
static const double kMcdRes[98] = {
    9.6198382e-4, .0010901181, .0012310012, .0013841352, .0015481583, .0017210036, .0018988943, .002076939,
    .0022484281, .0024049483, .0025366202, .0026316255, .0026774985, .0026613059, .0025708784, .0023962965,
    .002130655, .0017725174, .0013268656, 8.0657672e-4, 2.3337584e-4, -3.6291778e-4, -9.4443569e-4,
    -.0014678875, -.0018873741, -.0021588493, -.0022448371, -.0021198179, -.0017754602, -.0012246034,
    -5.0414167e-4, 3.2507078e-4, .0011811065, .0019673402, .0025827094, .0029342526, .0029517083, .0026012166,
    .0018959062, 9.0128649e-4, -2.6757144e-4, -.0014567885, -.002492855, -.0032079776, -.0034678637,
    -.0031988217, -.0024080969, -.001193624, 2.6134145e-4, .0017117758, .0028906898, .0035614435, .0035711778,
    .0028921374, .0016385898, 4.9857464e-5, -.0015572671, -.0028578151, -.0035924212, -.0036253044,
    -.002975086, -.0018044436, -3.7796664e-4, .0010076215, .0020937327, .0027090854, .0028031667, .0024276576,
    .0017175597, 8.1030795e-4, -1.2592304e-4, -9.4888491e-4, -.0015544816, -.0018831972, -.0019203142,
    -.0016905849, -.0012487737, -6.6789911e-4, -2.7079461e-5, 5.9931935e-4, .0011499748, .0015816521,
    .0018709224, .0020129966, .0020184702, .0019089181, .0017122289, .001458377, .0011760717, 8.9046768e-4,
    6.2190822e-4, 3.8553762e-4, 1.9155022e-4, 4.5837109e-5, -4.9177834e-5, -9.3670762e-5, -8.9622968e-5,
    -4.01538532e-5};

// multi-colour disk integrand (mcdint, donthcomp.c:52-103)
static double mcdint_h(double et) {
  static const double gc[3] = {.078196667, -1.066202, 1.192418};
  static const double gw[3] = {.5207874, .513457, .4077983};
  static const double gn[3] = {.3728691, .039775528, .037766505};
  const double loget = lg10_h(et);
  double pos = (loget - lg10_h(0.001)) / .06 + 1;
  const int j = (int) pos;
  double resfact;
  if (j < 1) {
    resfact = kMcdRes[0];
  } else if (j >= 98) {
    resfact = kMcdRes[97];
  } else {
    pos -= j;
    resfact = kMcdRes[j - 1] * (1 - pos) + kMcdRes[j] * pos;
  }
  double gaufact = 1.0;
  for (int k = 0; k < 3; k++) {
    const double zz = (loget - gc[k]) / gw[k];
    gaufact += gn[k] * std::exp(-zz * zz / 2.);
  }
  return std::pow(et / .001, -.66666666666666663) * 193.21556 * (std::pow(et, 1.663753) * .52876731 + 1.) *
         std::exp(-et) * gaufact * (resfact + 1.);
}

static float2 ff_h(double d) {
  const float hi = (float) d;
  return make_float2(hi, (float) (d - (double) hi));
}

int nth_grid_build(const std::vector<double> &co, double band_lo, double band_hi, NthGrid &G) {
  const double tempbb = .05 / 511., delta = .02, deltal = delta * std::log(10.);
  const double xmin = tempbb * 1e-4;
  std::vector<double> x(RELX_NTH_N + 3, 0.0), seed(RELX_NTH_N + 2, 0.0);
  for (int j = 1; j <= RELX_NTH_N + 2; j++) x[j] = xmin * std::pow(10., (j - 1) * delta);
  // seed photons: the disk blackbody per bin of the grid's geometric midpoints (xsdskb,
  // donthcomp.c:137-191, five-point Gauss-Legendre), as a rate per unit energy
  int jmaxth = (int) (lg10_h(tempbb * 50. / xmin) / delta);
  if (jmaxth > 900) jmaxth = 900;
  const int ne = jmaxth - 2;
  const double tin = tempbb * 511.;
  static const double gw5[5] = {.236926885, .47862867, .568888888, .47862867, .236926885};
  static const double gx5[5] = {-.906179846, -.53846931, 0., .53846931, .906179846};
  for (int i = 1; i <= ne; i++) {
    const double elo = std::sqrt(x[i] * x[i + 1]) * 511., ehi = std::sqrt(x[i + 1] * x[i + 2]) * 511.;
    const double xn = (ehi - elo) / 2.f, xh = xn + elo;
    double acc = 0.;
    for (int k = 0; k < 5; k++) acc += gw5[k] * (mcdint_h((xn * gx5[k] + xh) / tin) * tin * tin * 1. / 361.);
    seed[i] = acc * xn * 511. / (ehi - elo);
  }
  seed[0] = seed[1];
  // normalisation weights: p(E) at the coarse edges is linear in the table (interpolation of
  // donthcomp.c:768-786, the reference's search over x * 511), the bin photon flux is the
  // trapezoid of p / E^2, weighted by the bin centre inside the band
  const int nb = (int) co.size() - 1;
  std::vector<double> W(co.size(), 0.0), Gw(RELX_NTH_N + 2, 0.0);
  for (int b = 0; b < nb; b++) {
    const bool in_band = co[b] >= band_lo && co[b] <= band_hi;
    if (!in_band) continue;
    const double em = 0.5 * (co[b] + co[b + 1]), hw = .5 * (co[b + 1] - co[b]) * em;
    W[b] += hw / (co[b] * co[b]);
    W[b + 1] += hw / (co[b + 1] * co[b + 1]);
  }
  for (size_t k = 0; k < co.size(); k++) {
    if (W[k] == 0.0) continue;
    int j = 1;
    while (j <= RELX_NTH_N - 1 && x[j] * 511. < co[k]) ++j;
    if (j == 1) {
      Gw[1] += W[k];
    } else {
      const int jl = j - 1;
      const double w = (co[k] / 511. - x[jl]) / (x[jl + 1] - x[jl]);
      Gw[jl] += W[k] * (1 - w);
      Gw[jl + 1] += W[k] * w;
    }
  }
  for (int j = 1; j <= RELX_NTH_N; j++) {
    const double w = x[j], w1 = std::sqrt(x[j] * x[j + 1]);
    const double c2 = std::pow(w1, 4.) / (w1 * 4.6 + 1. + w1 * 1.1 * w1);  // Cooper (donthcomp.c:511-521)
    double rel;                                                           // (donthcomp.c:557-570)
    if (w <= .05) {
      rel = 1 - w * 2 + w * 26 * w / 5;
    } else {
      const double z1 = (w + 1) / (w * (w * w)), z2 = w * 2 + 1, z3 = std::log(z2), z4 = w * 2 * (w + 1) / z2,
                   z5 = z3 / 2 / w, z6 = (w * 3 + 1) / z2 / z2;
      rel = (z1 * (z4 - z3) + z5 - z6) * .75;
    }
    NthPoint &P = G.p[j];
    P.cd = ff_h(c2 / deltal);
    P.iw = ff_h(1. / (deltal * w1));
    P.rel3 = ff_h(rel / 3.);
    P.x3 = ff_h(w * w * w);
    P.xd = ff_h(w * ((j - 1 <= ne) ? seed[j - 1] : 0.0));
    P.x4 = ff_h(w * w * w * w);
    P.g = ff_h(Gw[j]);
    P.x = ff_h(w);
  }
  G.p[0] = NthPoint{};
  for (int j = 0; j <= RELX_NTH_N + 1; j++) G.x[j] = x[j];
  G.jnr0 = (int) (lg10_h(.1 / xmin) / delta + 1);
  G.jrel0 = (int) (lg10_h(1. / xmin) / delta + 1);
  const double xx = 1 / (1 / (1. / 511.));
  int ih = 2;
  while (ih < kNthMaxJ && xx > x[ih]) ++ih;
  G.ih0 = ih;
  G.l2x511 = (float) std::log2(x[1] * 511.);
  G.inv_l2step = (float) (1.0 / (delta * std::log2(10.)));
  return 0;
}

__device__ __forceinline__ double nth_lg10(double x) { return 0.43429448190325182765 * log(x); }

// reciprocal in float-float: the float reciprocal and one Newton step
__device__ __forceinline__ float2 ff_rcp(float2 a) {
  const float r = __frcp_rn(a.x);
  const float p = __fmul_rn(a.x, r);
  const float pe = fmaf(a.x, r, -p);
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), pe), __fmul_rn(a.y, r));
  return qts(r, __fmul_rn(r, e));
}

// tautom times the escape probability at point j (donthcomp.c:572-585): 1 / (taukn / 3 + 1) below
// the non-relativistic bound, the same with taukn tapered linearly up to the relativistic one, 1 above
__device__ __forceinline__ float2 nth_bt(const NthPoint &P, int j, float2 tau, int jnr, int jrel, float2 xnr,
                                         float2 invdx) {
  if (j > jrel) return make_float2(1.0f, 0.0f);
  float2 y = ff_mul(tau, P.rel3);
  if (j >= jnr) y = ff_mul(y, ff_addf(ff_neg(ff_mul(ff_add(P.x, ff_neg(xnr)), invdx)), 1.0f));
  return ff_rcp(ff_addf(y, 1.0f));
}

// continuum c of the launch: set = c / per, k = c % per; k = 0 the source (kTe), k = z + 1 zone z
// (kTe times the zone's energy shift).  params: the xillver model reads Gamma and kTe from its
// parameters (p[0], p[2]).  scr: [point][continuum] with stride ncont_all, this launch's
// continua from c_off.
__global__ void __launch_bounds__(kNthThreads) nthcomp_kernel(const NthGrid *__restrict__ G,
                                                              const RelxSetIn *__restrict__ sin,
                                                              const RelxSetState *__restrict__ sst, bool params,
                                                              int per, int n_sets, int nq, double *__restrict__ qout,
                                                              NthTable *__restrict__ tabs, float4 *__restrict__ scr,
                                                              int64_t ncont_all, int64_t c_off) {
  // the photon grid in shared memory (58 KB, read at every point of both sweeps)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  NthPoint *Pg = reinterpret_cast<NthPoint *>(smem_raw);
  {
    const float4 *src = reinterpret_cast<const float4 *>(G->p);
    float4 *dst = reinterpret_cast<float4 *>(Pg);
    for (int i = threadIdx.x; i < (RELX_NTH_N + 1) * 4; i += kNthThreads) dst[i] = src[i];
  }
  __syncthreads();
  const int64_t c = (int64_t) blockIdx.x * kNthThreads + threadIdx.x;
  if (c >= (int64_t) n_sets * per) return;
  const int set = (int) (c / per), k = (int) (c - (int64_t) set * per);
  double gam, kte;
  if (params) {
    gam = sin[set].p[0];
    kte = sin[set].p[2];
  } else {
    const RelxSetState &s = sst[set];
    if (s.status != RELX_OK || s.prim != 1 || k > s.nz) return;
    const double shift = k == 0 ? 1.0 : s.zshift[k - 1];
    if (k > 0 && shift == 1.0) return;  // the zone keeps the source normalisation
    gam = s.gam;
    kte = s.ect_src * shift;
  }
  double *q = qout + (size_t) set * nq + k;
  NthTable *T = (k == 0) ? &tabs[set] : nullptr;
  // grid length and scalars (donthcomp.c:320-375); a kTe that leaves fewer than 4 points (kTe <= 0 or
  // far below the seed temperature) has no spectrum: a non-finite normalisation marks the set
  const double tempbb = .05 / 511., theta = kte / 511.;
  const double d1 = gam + .5;
  const double tautom = sqrt(3. / (theta * (d1 * d1 - 2.25)) + 2.25) - 1.5;
  const double xmin = tempbb * 1e-4, xmax = theta * 40.;
  const double r = nth_lg10(xmax / xmin) / .02;
  if (!(r >= 3.0)) {
    *q = __longlong_as_double(0x7ff8000000000000ll);
    if (T) T->n = 0;
    return;
  }
  const int jmax = r >= (double) kNthMaxJ ? kNthMaxJ : min((int) r + 1, kNthMaxJ);
  const int jnr = min(G->jnr0, jmax - 1), jrel = min(G->jrel0, jmax);
  const float2 tau = ff_from_double(tautom), th = ff_from_double(theta);
  const float2 xnr = Pg[jnr].x, invdx = ff_from_double(1.0 / (G->x[jrel] - G->x[jnr]));
  float4 *sc = scr + c_off + c;

  // forward sweep: a u(j+1) + b u(j) + c u(j-1) = d for j = 2 .. jmax - 1, u(1) = aa u(2), u(jmax) = 0
  // a_j = -A_j, c_j = T_{j-1}, b_j = A_{j-1} - T_j + x_j^3 bt_j with
  // A_j = tautom cd_j (theta iw_j + 1/2), T_j = tautom cd_j (1/2 - theta iw_j)
  const float2 u1 = ff_mul(th, Pg[1].iw);
  const float2 aa = ff_mul(ff_addf(u1, .5f), ff_rcp(ff_addf(u1, -.5f)));
  float2 Ap, Tp;
  {
    const float2 P1 = ff_mul(tau, Pg[1].cd);
    Ap = ff_mul(P1, ff_addf(u1, .5f));
    Tp = ff_mul(P1, ff_addf(ff_neg(u1), .5f));
  }
  float2 gm = make_float2(0.f, 0.f), dd = make_float2(0.f, 0.f);
  for (int j = 2; j <= jmax - 1; j++) {
    const NthPoint P = Pg[j];
    const float2 u = ff_mul(th, P.iw);
    const float2 Pj = ff_mul(tau, P.cd);
    const float2 A = ff_mul(Pj, ff_addf(u, .5f)), Tj = ff_mul(Pj, ff_addf(ff_neg(u), .5f));
    const float2 bt = nth_bt(P, j, tau, jnr, jrel, xnr, invdx);
    const float2 b = ff_add(ff_add(Ap, ff_neg(Tj)), ff_mul(P.x3, bt));
    float2 alp, num;
    if (j == 2) {
      alp = ff_add(b, ff_mul(Tp, aa));
      num = P.xd;
    } else {
      alp = ff_add(b, ff_neg(ff_mul(Tp, gm)));
      num = ff_add(P.xd, ff_neg(ff_mul(Tp, dd)));
    }
    const float2 ia = ff_rcp(alp);
    gm = ff_mul(ff_neg(A), ia);
    dd = ff_mul(num, ia);
    sc[(size_t) j * ncont_all] = make_float4(gm.x, gm.y, dd.x, dd.y);
    Ap = A;
    Tp = Tj;
  }
  // back sweep: u, E F_E = x^4 u bt (donthcomp.c:603-610), the normalisation sum and the table
  const int ih = min(G->ih0, jmax), il = ih - 1;
  float2 un = make_float2(0.f, 0.f), qs = make_float2(0.f, 0.f), s_il = un, s_ih = un;
  // the scratch is read 8 points at a time (independent loads in flight together)
  for (int j0 = jmax - 1; j0 >= 1; j0 -= 8) {
    float4 vb[8];
#pragma unroll
    for (int q = 0; q < 8; q++)
      if (j0 - q >= 2) vb[q] = sc[(size_t) (j0 - q) * ncont_all];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int j = j0 - q;
      if (j < 1) break;
      float2 uj;
      if (j >= 2) {
        uj = ff_add(make_float2(vb[q].z, vb[q].w), ff_neg(ff_mul(make_float2(vb[q].x, vb[q].y), un)));
      } else {
        uj = ff_mul(aa, un);
      }
      const NthPoint P = Pg[j];
      const float2 sp = ff_mul(ff_mul(P.x4, uj), nth_bt(P, j, tau, jnr, jrel, xnr, invdx));
      qs = ff_add(qs, ff_mul(P.g, sp));
      if (j == il) s_il = sp;
      if (j == ih) s_ih = sp;
      if (T) {
        T->sp[j] = ff_to_double(sp);
        T->spf[j] = __fadd_rn(sp.x, sp.y);
      }
      un = uj;
    }
  }
  if (T) {
    T->sp[jmax] = 0.0;
    T->spf[jmax] = 0.0f;
    T->n = jmax;
  }
  // 1 / E F_E at the 1 keV point (donthcomp.c:617-638, 754-758) and the normalisation on the coarse grid
  const double xx = 1 / (1 / (1. / 511.));
  const double sil = ff_to_double(s_il), sih = ff_to_double(s_ih);
  const double normfac = 1 / (sil + (sih - sil) * (xx - G->x[il]) / (G->x[ih] - G->x[il]));
  *q = ff_to_double(qs) * normfac * (1e20 * 1.602177e-09 / (1e15 / 4.0 / kPi));
}

// The same continua for few sets, one CTA per continuum: the per-point quantities (the tridiagonal
// coefficients A and T, tautom times the escape probability, x^3 / seed / x^4 / weight of the grid)
// are formed by all threads at once into shared memory, and thread 0 runs only the two recurrences
// and the normalisation sum, with the operations and the order of nthcomp_kernel: the same numbers,
// with a serial chain a few times shorter.
struct NthCoopSmem {
  float2 A[RELX_NTH_N + 1], T[RELX_NTH_N + 1], bt[RELX_NTH_N + 1], b[RELX_NTH_N + 1];
  float2 xd[RELX_NTH_N + 1], x4[RELX_NTH_N + 1], g[RELX_NTH_N + 1];
  float2 gm[RELX_NTH_N + 1], dd[RELX_NTH_N + 1], sp[RELX_NTH_N + 1];
  int skip;
};

constexpr int kNthCoopThreads = 256;

__global__ void __launch_bounds__(kNthCoopThreads) nthcomp_coop_kernel(const NthGrid *__restrict__ G,
                                                                       const RelxSetIn *__restrict__ sin,
                                                                       const RelxSetState *__restrict__ sst,
                                                                       bool params, int per, int nq,
                                                                       double *__restrict__ qout,
                                                                       NthTable *__restrict__ tabs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  NthCoopSmem &m = *reinterpret_cast<NthCoopSmem *>(smem_raw);
  const int set = blockIdx.x / per, k = blockIdx.x - set * per, tid = threadIdx.x;
  double gam, kte;
  if (params) {
    gam = sin[set].p[0];
    kte = sin[set].p[2];
  } else {
    const RelxSetState &s = sst[set];
    if (s.status != RELX_OK || s.prim != 1 || k > s.nz) return;  // block-uniform
    const double shift = k == 0 ? 1.0 : s.zshift[k - 1];
    if (k > 0 && shift == 1.0) return;
    gam = s.gam;
    kte = s.ect_src * shift;
  }
  double *q = qout + (size_t) set * nq + k;
  NthTable *Tt = (k == 0) ? &tabs[set] : nullptr;
  const double tempbb = .05 / 511., theta = kte / 511.;
  const double d1 = gam + .5;
  const double tautom = sqrt(3. / (theta * (d1 * d1 - 2.25)) + 2.25) - 1.5;
  const double xmin = tempbb * 1e-4, xmax = theta * 40.;
  const double r = nth_lg10(xmax / xmin) / .02;
  if (!(r >= 3.0)) {
    if (tid == 0) {
      *q = __longlong_as_double(0x7ff8000000000000ll);
      if (Tt) Tt->n = 0;
    }
    return;
  }
  const int jmax = r >= (double) kNthMaxJ ? kNthMaxJ : min((int) r + 1, kNthMaxJ);
  const int jnr = min(G->jnr0, jmax - 1), jrel = min(G->jrel0, jmax);
  const float2 tau = ff_from_double(tautom), th = ff_from_double(theta);
  const float2 xnr = G->p[jnr].x, invdx = ff_from_double(1.0 / (G->x[jrel] - G->x[jnr]));
  // per point, in parallel
  for (int j = 1 + tid; j <= jmax - 1; j += kNthCoopThreads) {
    const NthPoint P = G->p[j];
    const float2 u = ff_mul(th, P.iw);
    const float2 Pj = ff_mul(tau, P.cd);
    m.A[j] = ff_mul(Pj, ff_addf(u, .5f));
    m.T[j] = ff_mul(Pj, ff_addf(ff_neg(u), .5f));
    m.bt[j] = nth_bt(P, j, tau, jnr, jrel, xnr, invdx);
    m.xd[j] = P.xd;
    m.x4[j] = P.x4;
    m.g[j] = P.g;
  }
  __syncthreads();
  for (int j = 2 + tid; j <= jmax - 1; j += kNthCoopThreads)
    m.b[j] = ff_add(ff_add(m.A[j - 1], ff_neg(m.T[j])), ff_mul(G->p[j].x3, m.bt[j]));
  __syncthreads();
  const int ih = min(G->ih0, jmax), il = ih - 1;
  if (tid == 0) {
    const float2 u1 = ff_mul(th, G->p[1].iw);
    const float2 aa = ff_mul(ff_addf(u1, .5f), ff_rcp(ff_addf(u1, -.5f)));
    float2 gm = make_float2(0.f, 0.f), dd = make_float2(0.f, 0.f);
    for (int j = 2; j <= jmax - 1; j++) {
      const float2 Tp = m.T[j - 1];
      float2 alp, num;
      if (j == 2) {
        alp = ff_add(m.b[j], ff_mul(Tp, aa));
        num = m.xd[j];
      } else {
        alp = ff_add(m.b[j], ff_neg(ff_mul(Tp, gm)));
        num = ff_add(m.xd[j], ff_neg(ff_mul(Tp, dd)));
      }
      const float2 ia = ff_rcp(alp);
      gm = ff_mul(ff_neg(m.A[j]), ia);
      dd = ff_mul(num, ia);
      m.gm[j] = gm;
      m.dd[j] = dd;
    }
    float2 un = make_float2(0.f, 0.f), qs = make_float2(0.f, 0.f), s_il = un, s_ih = un;
    for (int j = jmax - 1; j >= 1; j--) {
      const float2 uj = (j >= 2) ? ff_add(m.dd[j], ff_neg(ff_mul(m.gm[j], un))) : ff_mul(aa, un);
      const float2 spj = ff_mul(ff_mul(m.x4[j], uj), m.bt[j]);
      qs = ff_add(qs, ff_mul(m.g[j], spj));
      if (j == il) s_il = spj;
      if (j == ih) s_ih = spj;
      m.sp[j] = spj;
      un = uj;
    }
    const double xx = 1 / (1 / (1. / 511.));
    const double sil = ff_to_double(s_il), sih = ff_to_double(s_ih);
    const double normfac = 1 / (sil + (sih - sil) * (xx - G->x[il]) / (G->x[ih] - G->x[il]));
    *q = ff_to_double(qs) * normfac * (1e20 * 1.602177e-09 / (1e15 / 4.0 / kPi));
  }
  if (Tt) {
    __syncthreads();
    for (int j = 1 + tid; j <= jmax - 1; j += kNthCoopThreads) {
      Tt->sp[j] = ff_to_double(m.sp[j]);
      Tt->spf[j] = __fadd_rn(m.sp[j].x, m.sp[j].y);
    }
    if (tid == 0) {
      Tt->sp[jmax] = 0.0;
      Tt->spf[jmax] = 0.0f;
      Tt->n = jmax;
    }
  }
}

// normalisation changes of the zones on their corner weights (the de-duplicated list or the per-zone
// lists), source normalisation of the primary
__global__ void nthcomp_apply_kernel(RelxSetState *__restrict__ sst, const double *__restrict__ q, int nq,
                                     RelxCorners *__restrict__ cor, RelxZoneCorners *__restrict__ zcor) {
  const int set = blockIdx.x, tid = threadIdx.x;
  RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.prim != 1) return;
  const double q0 = q[(size_t) set * nq];
  bool bad = !isfinite(q0) || !(q0 > 0.0);
  for (int z = 0; z < s.nz && !bad; z++)
    if (s.zshift[z] != 1.0 && !isfinite(q[(size_t) set * nq + z + 1])) bad = true;
  if (bad) {  // no nthcomp spectrum for the set's kTe (every thread sees the same)
    if (tid == 0) s.status = RELX_ERR_PARAM;
    return;
  }
  const int nz = s.nz;
  if (s.xdense) {
    for (int e = tid; e < s.ucount * nz; e += blockDim.x) {
      const int u = e / nz, z = e - u * nz;
      const double xs = (s.zshift[z] == 1.0) ? 1.0 : q[(size_t) set * nq + z + 1] * (1.0 / q0);
      cor[set].w[u][z] = (float) ((double) cor[set].w[u][z] * xs);
    }
  } else {
    for (int e = tid; e < nz * 32; e += blockDim.x) {
      const int z = e >> 5, c = e & 31;
      const double xs = (s.zshift[z] == 1.0) ? 1.0 : q[(size_t) set * nq + z + 1] * (1.0 / q0);
      zcor[set].w[z][c] = (float) ((double) zcor[set].w[z][c] * xs);
    }
  }
  for (int z = tid; z < nz; z += blockDim.x)
    s.inv_nc[z] = (float) ((s.zshift[z] == 1.0) ? 1.0 : q[(size_t) set * nq + z + 1] * (1.0 / q0));
  if (tid == 0) s.src_norm = 1.0 / q0;
}

cudaError_t nthcomp_set_smem() {
  cudaError_t e = cudaFuncSetAttribute(nthcomp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int) (sizeof(NthPoint) * (RELX_NTH_N + 1)));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(nthcomp_coop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int) sizeof(NthCoopSmem));
}

size_t nthcomp_scratch_bytes(int n_sets, int nza, bool params) {
  return (size_t) n_sets * (params ? 1 : nza + 1) * (kNthMaxJ + 1) * sizeof(float4);
}

cudaError_t launch_nthcomp(cudaStream_t s, const RelxTables &tab, const RelxSetIn *sin, RelxSetState *sst, int n_sets,
                           int nza, bool params, double *q, NthTable *tabs, RelxCorners *cor, RelxZoneCorners *zcor,
                           float4 *scr, int64_t ncont_all, int64_t c_off) {
  if (n_sets <= 0) return cudaSuccess;
  const int nq = RELX_NZMAX + 1;
  const int per = params ? 1 : nza + 1;
  const int64_t ncont = (int64_t) n_sets * per;
  if (ncont <= 2 * 152) {  // few continua: one CTA each, the per-point work spread over its threads
    nthcomp_coop_kernel<<<(unsigned) ncont, kNthCoopThreads, sizeof(NthCoopSmem), s>>>(tab.nth_grid, sin, sst, params,
                                                                                     per, nq, q, tabs);
  } else {
    nthcomp_kernel<<<(unsigned) ((ncont + kNthThreads - 1) / kNthThreads), kNthThreads,
                     sizeof(NthPoint) * (RELX_NTH_N + 1), s>>>(tab.nth_grid, sin, sst, params, per, n_sets, nq, q,
                                                              tabs, scr, ncont_all, c_off);
  }
  if (!params) nthcomp_apply_kernel<<<n_sets, 128, 0, s>>>(sst, q, nq, cor, zcor);
  return cudaGetLastError();
}

}  // namespace relx
