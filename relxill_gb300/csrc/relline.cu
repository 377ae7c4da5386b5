// relline.cu -- line profile kernel: transfer-function interpolation, g*
// integration of every (radius, energy bin) pair and binning into radial zones
// and the emission-angle histogram (Relprofile.cpp:39-80, 141-303, 489-958).
//
// line_table_kernel writes each set's (a, mu0)-interpolated transfer functions on
// all table radii once (two float2 planes: trff1/trff2, cosne1/cosne2); the line
// profile stages the rows a chunk of radii reads in shared memory, the histogram
// reads them through the read-only cache.
//
// Line profile: one CTA per (512-bin tile, parameter set), 8 warps, four CTAs per SM.
//  * Zone by zone, warps take fine radii round robin; per radius a warp builds
//    the radial interpolation trf(g*) (40 points) from the set's table and its
//    lanes integrate consecutive energy bins (Romberg with the reference's prec
//    0.02 / itermax 5, midpoint below 0.95 keV, sqrt edge terms within 5e-3 of
//    g* = 0 and 1).  Each warp adds into its own shared row; at the end of
//    the zone the rows are summed in warp order: no atomics, so every bin is
//    the same number in every run and in every batch composition.
//  * Arithmetic is FP32.  Bin edges and gmin/gmax enter as float-float so
//    that g* is accurate to an ulp.  Two decisions of the reference are
//    discrete and are taken in higher precision where the FP32 value lies close
//    to the decision point: the side of a transfer-function grid point (the
//    reference's interpolation weights are reversed, so the interpolant jumps
//    there; decided in float-float from the reference's own energy abscissa
//    within 2e-5 grid units of the point), and Romberg's convergence test
//    obtprec > 0.02 (a bin whose FP32 test came within 2e-6 of 0.02 is
//    integrated again with FP64 Romberg: one level more or less changes the bin
//    by up to about 2%).  Such bins are marked in a per-lane mask and redone
//    after the radius's other bins by one out-of-line call, so that the bin
//    loop holds no call (a call there makes the compiler spill its registers).
#include "relx_device.cuh"
#include "relx_kernels.h"

namespace relx {

constexpr int kLineWarps = 8;
constexpr int kLineThreads = kLineWarps * 32;
constexpr int kSumBins = 256;    // profile sums are kept per block of 256 bins (two per tile)
static_assert(kSumBins == kLineThreads, "one bin per thread and block in the sums");
constexpr float kH = 5e-3f;
constexpr float kSideBand = 2e-5f;  // grid units within which the side of a g* point is taken in float-float
// |obtprec - 0.02| within which a bin is integrated again in FP64: about five times the error of the
// FP32 obtprec (the level sums carry a few ulp each, 2-5e-7 of the integral)
constexpr float kConvBand = 2e-6f;
constexpr int kLineTile = 512;      // energy bins per CTA

// per-radius constants (warp uniform)
struct RadC {
  float2 gmin, gmax, dg;  // float-float
  float gminf, dgf, inv_dg;
  float edge_lo, edge_hi; // 2 sqrt(H) sum_k F_k(H), same at 1-H (emissivity factored out)
  float2 eH, e1H;         // gstar2ener(H), gstar2ener(1-H) in float-float
  bool red_H;             // gstar2ener(H) >= 0.95
  int ng, limb;
  float inv_dgs;          // (ng-1) / (1-2H)
  const float2 *gs;       // table g* points as float-float (shared memory)
};

// abscissa of the reference in energy (for the grid-point side decision, read only there)
struct Absc {
  const float2 *eb;  // the bin's edges E_lo, E_hi (float-float, shared memory)
  bool lo_H, hi_H;   // the lower / upper end is replaced by gstar2ener(H) / gstar2ener(1-H)
  int n, i;          // Romberg level and index (n = -1: midpoint)
};

// transfer functions at one radius: trff (and cosne for limb laws) at the table g* points
template <bool LIMB> struct TW;
template <> struct TW<false> { float2 t; };
template <> struct TW<true> { float4 t; };

// integrand F_k(x) = E^3 trf_k(x) [limb] / sqrt(x (1-x)), k = 0, 1  (relb_func,
// Relprofile.cpp:489-521 times (gmax - gmin) / emis)
template <bool LIMB>
__device__ __forceinline__ float2 eval_F(float x, float y, const RadC &rc, const TW<LIMB> *__restrict__ tw,
                                         const Absc &ab) {
  const int ng = rc.ng;
  float t = (x - kH) * rc.inv_dgs;
  float tr = rintf(t);
  int ind;
  if (fabsf(t - tr) < kSideBand && tr >= 1.0f && tr <= (float) (ng - 2)) {
    // side of grid point k from the reference's abscissa (float-float)
    int k = (int) tr;
    const float2 alo = ab.lo_H ? rc.eH : ab.eb[0];
    const float2 ahi = ab.hi_H ? rc.e1H : ab.eb[1];
    float2 eg;
    if (ab.n < 0) {
      eg = ff_mulf(ff_add(alo, ahi), 0.5f);
    } else if (ab.i == (1 << ab.n)) {
      eg = ahi;
    } else {
      float2 w = ff_add(ahi, ff_neg(alo));
      eg = ff_add(alo, ff_mulf(w, ldexpf((float) ab.i, -ab.n)));
    }
    float2 G = ff_add(rc.gmin, ff_mul(rc.gs[k], rc.dg));
    ind = ff_ge(eg, G) ? k : k - 1;
  } else {
    ind = (int) floorf(t);
    ind = max(0, min(ind, ng - 2));
  }
  const float inte = t - (float) ind;
  const float inte1 = 1.0f - inte;
  const float e = rc.gminf + x * rc.dgf;
  const float e3 = e * e * e * rsqrtf(x * y);
  if constexpr (!LIMB) {
    const float2 A = tw[ind].t, B = tw[ind + 1].t;
    return make_float2(e3 * (inte * A.x + inte1 * B.x), e3 * (inte * A.y + inte1 * B.y));
  } else {
    const float4 A = tw[ind].t, B = tw[ind + 1].t;
    float f0 = e3 * (inte * A.x + inte1 * B.x);
    float f1 = e3 * (inte * A.y + inte1 * B.y);
    float m0 = inte * A.z + inte1 * B.z, m1 = inte * A.w + inte1 * B.w;
    if (rc.limb == 1) { f0 *= (1.0f + 2.06f * m0); f1 *= (1.0f + 2.06f * m1); }
    else if (rc.limb == 2) { f0 *= logf(1.0f + 1.0f / m0); f1 *= logf(1.0f + 1.0f / m1); }
    return make_float2(f0, f1);
  }
}

// romberg_integration (Relprofile.cpp:524-579) over [ga, gb] in g*, both branches in
// lock step; interior sums reuse the previous level's points; the Romberg table is
// updated in place (p[ii] holds t[ii][n-ii] of the last completed level).
// *rare is set when a tested FP32 obtprec lies within kConvBand of 0.02.
template <bool LIMB>
__device__ __forceinline__ float romberg2(float ga, float ca, float gb, float cb, const RadC &rc,
                                          const TW<LIMB> *__restrict__ tw, Absc ab, bool *rare) {
  const float pas0 = gb - ga;
  ab.n = 0;
  ab.i = 0;
  const float2 fa = eval_F<LIMB>(ga, ca, rc, tw, ab);
  ab.i = 1;
  const float2 fb = eval_F<LIMB>(gb, cb, rc, tw, ab);
  const float ta0 = (fa.x + fb.x) * 0.5f, ta1 = (fa.y + fb.y) * 0.5f;
  float p0[7], p1[7];
  p0[0] = ta0 * pas0;
  p1[0] = ta1 * pas0;
  float s0 = 0.0f, s1 = 0.0f;
  bool c0 = false, c1 = false;
  float r0 = 0.0f, r1 = 0.0f;
  constexpr float inv4m1[7] = {0.f, 1.f / 3.f, 1.f / 15.f, 1.f / 63.f, 1.f / 255.f, 1.f / 1023.f, 1.f / 4095.f};
#pragma unroll
  for (int n = 1; n <= 6; n++) {
    const float sc = ldexpf(1.0f, -n);
    const float pas = pas0 * sc;
    float a0 = 0.0f, a1 = 0.0f;
    ab.n = n;
    for (int i = 1; i < (1 << n); i += 2) {
      const float u = pas0 * ((float) i * sc);
      ab.i = i;
      const float2 f = eval_F<LIMB>(ga + u, ca - u, rc, tw, ab);
      a0 += f.x;
      a1 += f.y;
    }
    s0 += a0;
    s1 += a1;
    const float old0 = p0[n - 1], old1 = p1[n - 1];
    float t0 = (ta0 + s0) * pas, t1 = (ta1 + s1) * pas;
    float r = 1.0f;
#pragma unroll
    for (int ii = 1; ii <= n; ii++) {
      r *= 4.0f;
      const float n0 = (r * t0 - p0[ii - 1]) * inv4m1[ii];
      const float n1 = (r * t1 - p1[ii - 1]) * inv4m1[ii];
      p0[ii - 1] = t0;
      p1[ii - 1] = t1;
      t0 = n0;
      t1 = n1;
    }
    p0[n] = t0;
    p1[n] = t1;
    const float o0 = fabsf(t0 - old0) / t0;
    const float o1 = fabsf(t1 - old1) / t1;
    if (!c0) {
      r0 = t0;
      if (fabsf(o0 - 0.02f) < kConvBand) *rare = true;
      if (!(o0 > 0.02f)) c0 = true;
    }
    if (!c1) {
      r1 = t1;
      if (fabsf(o1 - 0.02f) < kConvBand) *rare = true;
      if (!(o1 > 0.02f)) c1 = true;
    }
    if (c0 && c1) break;
  }
  return r0 + r1;
}

// sqrt(hi) - sqrt(lo) without cancellation
__device__ __forceinline__ float sqrt_diff(float hi, float lo) {
  float d = hi - lo;
  float sh = sqrtf(hi), sl = sqrtf(lo);
  float den = sh + sl;
  return den > 0.0f ? d / den : 0.0f;
}

// g* and 1 - g* of a bin edge, clamped to [0, 1] (integ_relline_bin, Relprofile.cpp:653-666).
// The side of gmin and gmax is taken from the signs of the float-float differences: the two
// rounded quotients alone can give g <= 1 with 1 - g < 0 for an edge just above gmax.
// (ff_diff: near gmin and gmax the sign is right and the value within about an ulp)
__device__ __forceinline__ float2 edge_gc(float2 E, const RadC &rc) {
  const float dlo = ff_diff(E, rc.gmin), dhi = ff_diff(rc.gmax, E);
  if (dlo <= 0.0f) return make_float2(0.0f, 1.0f);
  if (dhi <= 0.0f) return make_float2(1.0f, 0.0f);
  return make_float2(fminf(dlo * rc.inv_dg, 1.0f), fminf(dhi * rc.inv_dg, 1.0f));
}

// what the FP64 Romberg integration needs (read only on the rare path)
struct RareCtx {
  const RelxTables *tab;
  const RelxSetState *s;
  const double *ge;      // the set's line-profile grid (FP64)
  const double *ifac_p;  // FP64 radial factor of the radius (RelxRadial::ifac)
  int itab;              // table radius index
};

// the radius's transfer functions in FP64 at the table's g* points g0 .. g1 (trf1, trf2, cosne1,
// cosne2), and its gmin, gmax
struct Rad64 {
  double tf[RELX_MAX_NG][4];
  double gmn, gmx;
  int ng, g0, g1;
};

// gmin or gmax of the radius in FP64, as the set-up kernel computes it (Relprofile.cpp:295-300)
__device__ double gext_fp64(const RelxTables &tab, const RelxSetState &s, int itab, double ifac, bool is_max) {
  const int nr = tab.rel_nr, nm = tab.rel_nmu0;
  const size_t b00 = (size_t) s.ind_a * nm + s.ind_mu0, b10 = (size_t) (s.ind_a + 1) * nm + s.ind_mu0;
  const size_t b01 = b00 + 1, b11 = b10 + 1;
  const float *a = is_max ? tab.rel_gmax : tab.rel_gmin;
  const double fa = s.ifac_a, fm = s.ifac_mu0;
  double v[2];
  for (int q = 0; q < 2; q++) {
    const int i = itab + q;
    v[q] = lerp2(fa, fm, a[b00 * nr + i], a[b10 * nr + i], a[b01 * nr + i], a[b11 * nr + i]);
  }
  return lerp1(ifac, v[1], v[0]);
}

// gmin and gmax of the radius in FP64
__device__ void rad64_gext(const RareCtx &q, Rad64 &r) {
  const double ifac = *q.ifac_p;
  r.ng = q.tab->rel_ng;
  r.gmn = gext_fp64(*q.tab, *q.s, q.itab, ifac, false);
  r.gmx = gext_fp64(*q.tab, *q.s, q.itab, ifac, true);
}

// the last table point g with gstar[g] <= x (binary_search, relutility.c:155-170)
__device__ __forceinline__ int gstar_index(int ng, double x) {
  const double h = 5e-3, step = (1.0 - 2 * 5e-3) / (ng - 1);
  int klo = 0, khi = ng - 1;
  while (khi - klo > 1) {
    const int m = (khi + klo) >> 1;
    if (h + step * (double) (float) m > x) khi = m; else klo = m;
  }
  return klo;
}

// the radius's FP64 transfer functions (interp_lin_2d_float, then interp_lin_1d of the two table
// rows, Relprofile.cpp:67-77, 280-293) at the table points an integration over [a, b] (energies)
// reads; limb: the cosne columns as well
__device__ void rad64_build(const RareCtx &q, Rad64 &r, double a, double b, int limb) {
  const RelxTables &tab = *q.tab;
  const RelxSetState &s = *q.s;
  const int nr = tab.rel_nr, nm = tab.rel_nmu0, ng = tab.rel_ng;
  const double ifac = *q.ifac_p;
  const size_t b00 = (size_t) s.ind_a * nm + s.ind_mu0, b10 = (size_t) (s.ind_a + 1) * nm + s.ind_mu0;
  const size_t b01 = b00 + 1, b11 = b10 + 1;
  const double fa = s.ifac_a, fm = s.ifac_mu0;
  const double del_g = 1.0 / (r.gmx - r.gmn);
  r.g0 = gstar_index(ng, (a - r.gmn) * del_g);
  r.g1 = gstar_index(ng, (b - r.gmn) * del_g) + 1;
  const int nc = limb ? 4 : 2;
  for (int g = r.g0; g <= r.g1; g++) {
    float4 v[2][4];
#pragma unroll
    for (int q2 = 0; q2 < 2; q2++) {  // rows itab (q2 = 0) and itab + 1
      const size_t row = (size_t) (q.itab + q2) * ng + g;
      v[q2][0] = __ldg(&tab.rel_tc[b00 * nr * ng + row]);
      v[q2][1] = __ldg(&tab.rel_tc[b10 * nr * ng + row]);
      v[q2][2] = __ldg(&tab.rel_tc[b01 * nr * ng + row]);
      v[q2][3] = __ldg(&tab.rel_tc[b11 * nr * ng + row]);
    }
    for (int c = 0; c < nc; c++) {
      auto comp = [c](float4 x) { return c == 0 ? x.x : c == 1 ? x.y : c == 2 ? x.z : x.w; };
      const double hi = lerp2(fa, fm, comp(v[0][0]), comp(v[0][1]), comp(v[0][2]), comp(v[0][3]));
      const double lo = lerp2(fa, fm, comp(v[1][0]), comp(v[1][1]), comp(v[1][2]), comp(v[1][3]));
      r.tf[g][c] = lerp1(ifac, lo, hi);
    }
  }
}

// relb_func (Relprofile.cpp:489-521) in FP64 without the emissivity factor (it scales every value
// of one integration alike)
__device__ double relb_fp64(const Rad64 &r, double eg, int k, int limb) {
  const int ng = r.ng;
  const double gmn = r.gmn, gmx = r.gmx;
  const double del_g = 1.0 / (gmx - gmn);
  const double egstar = (eg - gmn) * del_g;
  const double h = 5e-3, step = (1.0 - 2 * 5e-3) / (ng - 1);
  const int klo = min(max(gstar_index(ng, egstar), r.g0), r.g1 - 1);  // within [g0, g1] up to rounding
  const double g0 = h + step * (double) (float) klo, g1 = h + step * (double) (float) (klo + 1);
  const double inte = (egstar - g0) / (g1 - g0), inte1 = 1.0 - inte;
  const double ftrf = inte * r.tf[klo][k] + inte1 * r.tf[klo + 1][k];
  double val = eg * eg * eg / ((gmx - gmn) * sqrt(egstar - egstar * egstar)) * ftrf;
  if (limb != 0) {
    const double mu = inte * r.tf[klo][2 + k] + inte1 * r.tf[klo + 1][2 + k];
    val *= (limb == 1) ? (1.0 + 2.06 * mu) : log(1.0 + 1.0 / mu);
  }
  return val;
}

// romberg_integration (Relprofile.cpp:524-579) of branch k in FP64 over the reference's interval
// (bin j's edges, or gstar2ener(H) / gstar2ener(1 - H) where the edge terms take over), with the
// emissivity factored out
__device__ double romberg_fp64(const Rad64 &r, double a, double b, int k, int limb) {
  double t[7][7];
  const double ta = (relb_fp64(r, a, k, limb) + relb_fp64(r, b, k, limb)) / 2.0;
  double pas = b - a;
  t[0][0] = ta * pas;
  double obtprec = 1.0;
  int niter = 0;
  while (obtprec > 0.02 && niter <= 5) {
    niter++;
    pas = pas / 2.0;
    double sum = ta;
    for (int ii = 1; ii <= (1 << niter) - 1; ii++) sum += relb_fp64(r, a + pas * ii, k, limb);
    t[0][niter] = sum * pas;
    double rr = 1.0;
    for (int ii = 1; ii <= niter; ii++) {
      rr *= 4.0;
      const int jj = niter - ii;
      t[ii][jj] = (rr * t[ii - 1][jj + 1] - t[ii - 1][jj]) / (rr - 1.0);
    }
    obtprec = fabs(t[niter][0] - t[niter - 1][0]) / t[niter][0];
  }
  return t[niter][0];
}

// integ_relline_bin (Relprofile.cpp:650-726) with the emissivity factored out, from the clamped
// g* of the bin's edges; eb: the bin's edges (for the rare grid-point side decision).  FP64: the
// Romberg part through romberg_fp64 (rq, bin j); otherwise through romberg2, which sets *rare.
template <bool LIMB, bool FP64>
__device__ __forceinline__ float integ_bin(float glo, float clo, float ghi, float chi, const float2 *eb, bool red_lo,
                                           const RadC &rc, const TW<LIMB> *__restrict__ tw, bool *rare,
                                           Rad64 *r64, const RareCtx *rq64, const double *ge, int j) {
  if (ghi == 0.0f) return 0.0f;
  float flu = 0.0f;
  bool has_lo = true, has_hi = true;
  float ga = glo, ca = clo, gb = ghi, cb = chi;
  bool red = red_lo;
  Absc ab;
  ab.eb = eb;
  ab.lo_H = false;
  ab.hi_H = false;
  if (glo <= kH) {
    float hhi = kH;
    ga = kH;
    ca = 1.0f - kH;
    red = rc.red_H;
    ab.lo_H = true;
    if (ghi <= kH) { hhi = ghi; has_lo = false; }
    flu += rc.edge_lo * sqrt_diff(hhi, glo);
  }
  if (ghi >= 1.0f - kH) {
    float hi_c = kH;  // 1 - hlo
    gb = 1.0f - kH;
    cb = kH;
    ab.hi_H = true;
    if (glo >= 1.0f - kH) { hi_c = clo; has_hi = false; }
    flu += rc.edge_hi * sqrt_diff(hi_c, chi);
  }
  if (has_lo && has_hi) {
    if (red) {
      if constexpr (FP64) {
        // the reference's interval: the bin's edges, or gstar2ener(H) / gstar2ener(1 - H)
        Rad64 &r = *r64;
        const double a = ab.lo_H ? (RELX_GFAC_H * (r.gmx - r.gmn) + r.gmn) : ge[j];
        const double b = ab.hi_H ? ((1 - RELX_GFAC_H) * (r.gmx - r.gmn) + r.gmn) : ge[j + 1];
        rad64_build(*rq64, r, a, b, rc.limb);
        flu += (float) (romberg_fp64(r, a, b, 0, rc.limb) + romberg_fp64(r, a, b, 1, rc.limb));
      } else {
        flu += romberg2<LIMB>(ga, ca, gb, cb, rc, tw, ab, rare);
      }
    } else {
      ab.n = -1;
      const float2 f = eval_F<LIMB>(0.5f * (ga + gb), 0.5f * (ca + cb), rc, tw, ab);
      flu += (f.x + f.y) * (gb - ga);
    }
  }
  return flu;
}


constexpr int kChunk = 128;  // radius records staged per chunk
static_assert(kLineTile % kSumBins == 0 && kLineTile == kLineTileH, "whole profile-sum blocks per tile");

template <bool LIMB>
struct LineSmem {
  float acc[kLineWarps][kLineTile];
  float2 eff[kLineTile + 1];
  unsigned char red[kLineTile];
  TW<LIMB> tw[kLineWarps][RELX_MAX_NG];
  RelxRadRec rec[kChunk];
  float2 gs[RELX_MAX_NG];   // table g* points (Relprofile.cpp:104-106) as float-float
  double red_sum[kLineWarps + 1];
  int row0, nrow;           // the set-table rows staged for the chunk: row0 .. row0 + nrow - 1
  TW<LIMB> rows[1];         // [line_rows<LIMB>()][ng] those rows, dynamic tail
};
// set-table rows staged per chunk at most (a zone of about 100 fine radii reads 8 rows typically,
// about 30 in the outermost zones); a chunk that reads more takes its rows from the read-only cache
template <bool LIMB> constexpr int line_rows() { return LIMB ? 16 : 32; }
static_assert(offsetof(LineSmem<false>, rec) % 16 == 0 && offsetof(LineSmem<true>, rec) % 16 == 0,
              "radius records are staged as int4 rows");
static_assert(kLineTile / 32 <= 32, "a lane's bins of one radius fit a 32-bit mask");

// the bins of one radius that romberg2 marked rare (bit i of rmask: the lane's i-th bin from jlo),
// integrated again with FP64 Romberg and added
template <bool LIMB>
__device__ __noinline__ void rare_bins(float *acc, const float2 *eff, const unsigned char *redv, int lane, int tlo,
                                       int jlo, const RadC rc, const TW<LIMB> *tw, const RareCtx rq, float ew,
                                       unsigned rmask) {
  Rad64 r64;
  rad64_gext(rq, r64);
  while (rmask) {
    const int it = __ffs(rmask) - 1;
    rmask &= rmask - 1;
    const int j = jlo + lane + 32 * it, jj = j - tlo;
    const float2 *eb = &eff[jj];
    const float2 lo = edge_gc(eb[0], rc), hi = edge_gc(eb[1], rc);
    const float v =
        integ_bin<LIMB, true>(lo.x, lo.y, hi.x, hi.y, eb, redv[jj] != 0, rc, tw, nullptr, &r64, &rq, rq.ge, j);
    acc[jj] += v * ew;
  }
}

// limb law at one table point (Relprofile.cpp:512-519)
__device__ __forceinline__ float limb_factor(int limb, float mu) {
  if (limb == 1) return 1.0f + 2.06f * mu;
  if (limb == 2) return logf(1.0f + 1.0f / mu);
  return 1.0f;
}

// tsum holds the profile sum of every (256-bin block, zone), nblk blocks per set.  htab: the sets'
// (a, mu0)-interpolated transfer functions (line_table_kernel).
template <bool LIMB>
__global__ void __launch_bounds__(kLineThreads, 4) relline_kernel(
    RelxTables tab, const RelxSetIn *__restrict__ sin, const RelxSetState *__restrict__ sst,
    const RelxRadial *__restrict__ srad, const double *__restrict__ line_e, const float4 *__restrict__ htab, int nza,
    float *__restrict__ prof, double *__restrict__ tsum, int nblk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  LineSmem<LIMB> &m = *reinterpret_cast<LineSmem<LIMB> *>(smem_raw);
  const int set = blockIdx.y, tile = blockIdx.x;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.cached) return;
  if ((s.limb != 0) != LIMB) return;
  const int tlo = s.win_lo + tile * kLineTile;
  const int thi = min(s.win_hi, tlo + kLineTile);
  if (tlo >= thi) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const RelxRadial &R = srad[set];
  const int nr = tab.rel_nr, ng = tab.rel_ng;
  const int nz = s.nz;
  if ((int) blockIdx.z >= nz) return;
  const bool is_line = (s.model == RELX_RELLINE);
  const double *ge = is_line ? (line_e + sin[set].e_off) : tab.conv_e;
  const size_t pbase = is_line ? (size_t) sin[set].e_off : (size_t) set * nza * RELX_NCONV;
  const size_t zstride = is_line ? 0 : RELX_NCONV;
  // the set's interpolated table: (trff1, trff2) plane, then (cosne1, cosne2)
  const float2 *__restrict__ T = reinterpret_cast<const float2 *>(htab + (size_t) set * nr * ng);
  const float2 *__restrict__ C = T + nr * ng;

  {
    for (int j = tid; j <= thi - tlo; j += kLineThreads) m.eff[j] = ff_split(ge[tlo + j]);
    for (int j = tid; j < thi - tlo; j += kLineThreads) m.red[j] = ge[tlo + j] >= 0.95 ? 1 : 0;
    for (int i = tid; i < kLineWarps * kLineTile; i += kLineThreads) (&m.acc[0][0])[i] = 0.0f;
    for (int g = tid; g < ng; g += kLineThreads)
      m.gs[g] = ff_from_double(5e-3 + (1.0 - 2 * 5e-3) / (ng - 1) * ((float) g));
  }
  __syncthreads();

  const float inv_dgs = (float) ((ng - 1) / (1.0 - 2 * 5e-3));
  const float sH = sqrtf(kH), isq = rsqrtf(kH * (1.0f - kH));
  // with a zone axis in the grid (few sets) each CTA takes one zone; a zone's sums do not depend
  // on the other zones, so the numbers are the same either way
  const int zb = gridDim.z > 1 ? (int) blockIdx.z : 0, ze = gridDim.z > 1 ? min((int) blockIdx.z + 1, nz) : nz;
  for (int z = zb; z < ze; z++) {
    const int i0 = s.zi0[z], i1 = s.zi1[z];
    for (int c0 = i0; c0 <= i1; c0 += kChunk) {
      const int cn = min(kChunk, i1 + 1 - c0);
      // stage the chunk's radius records (64-byte rows, coalesced)
      {
        const int4 *src = reinterpret_cast<const int4 *>(&R.rec[c0]);
        int4 *dst = reinterpret_cast<int4 *>(m.rec);
        for (int q = tid; q < cn * 4; q += kLineThreads) dst[q] = src[q];
      }
      __syncthreads();
      if (warp == 0) {
        // the set-table rows the chunk's radii read (itab and itab + 1 of each)
        int lo = 1 << 30, hi = -1;
        for (int q = lane; q < cn; q += 32) {
          const RelxRadRec &r = m.rec[q];
          if (r.ielo >= 0 && r.ielo < thi && r.iehi >= tlo) {
            lo = min(lo, (int) r.itab);
            hi = max(hi, (int) r.itab);
          }
        }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        if (lane == 0) {
          m.row0 = lo;
          m.nrow = hi >= lo ? hi + 2 - lo : 0;
        }
      }
      __syncthreads();
      const int row0 = m.row0;
      const bool staged = m.nrow <= line_rows<LIMB>();
      if (staged) {
        for (int q = tid; q < m.nrow * ng; q += kLineThreads) {
          if constexpr (!LIMB) {
            m.rows[q].t = __ldg(&T[row0 * ng + q]);
          } else {
            const float2 t = __ldg(&T[row0 * ng + q]), c = __ldg(&C[row0 * ng + q]);
            m.rows[q].t = make_float4(t.x, t.y, c.x, c.y);
          }
        }
      }
      __syncthreads();
      for (int ci = warp; ci < cn; ci += kLineWarps) {
        const RelxRadRec &rr = m.rec[ci];
        const int ielo = rr.ielo, iehi = rr.iehi;
        if (!(ielo >= 0 && ielo < thi && iehi >= tlo)) continue;
        // trf(g*) at this radius: interp_lin_1d(ifac_r, T[ind+1], T[ind]) (Relprofile.cpp:280-293)
        const int it = rr.itab;
        const float fr = rr.ifac;
        for (int g = lane; g < ng; g += 32) {
          if constexpr (!LIMB) {
            const float2 lo = staged ? m.rows[(it + 1 - row0) * ng + g].t : __ldg(&T[(it + 1) * ng + g]);
            const float2 hi = staged ? m.rows[(it - row0) * ng + g].t : __ldg(&T[it * ng + g]);
            m.tw[warp][g].t = make_float2(fr * hi.x + (1.0f - fr) * lo.x, fr * hi.y + (1.0f - fr) * lo.y);
          } else {
            float4 lo, hi;
            if (staged) {
              lo = m.rows[(it + 1 - row0) * ng + g].t;
              hi = m.rows[(it - row0) * ng + g].t;
            } else {
              const float2 tl = __ldg(&T[(it + 1) * ng + g]), th = __ldg(&T[it * ng + g]);
              const float2 cl = __ldg(&C[(it + 1) * ng + g]), ch = __ldg(&C[it * ng + g]);
              lo = make_float4(tl.x, tl.y, cl.x, cl.y);
              hi = make_float4(th.x, th.y, ch.x, ch.y);
            }
            m.tw[warp][g].t = make_float4(fr * hi.x + (1.0f - fr) * lo.x, fr * hi.y + (1.0f - fr) * lo.y,
                                          fr * hi.z + (1.0f - fr) * lo.z, fr * hi.w + (1.0f - fr) * lo.w);
          }
        }
        __syncwarp();
        const TW<LIMB> *tw = m.tw[warp];
        RadC rc;
        rc.gmin = rr.gmin;
        rc.gmax = rr.gmax;
        rc.dg = rr.dg;
        rc.gminf = rc.gmin.x;
        rc.dgf = rc.dg.x;
        rc.inv_dg = rr.inv_dg;
        rc.ng = ng;
        rc.limb = s.limb;
        rc.inv_dgs = inv_dgs;
        rc.eH = rr.eH;
        rc.e1H = rr.e1H;
        rc.red_H = rr.red_H != 0;
        rc.gs = m.gs;
        {
          // int_edge norms (Relprofile.cpp:585-621): trf at g* = H is T[1], at 1 - H is T[ng-2]
          float e = rc.gminf + kH * rc.dgf;
          float e3 = e * e * e * isq;
          float f0, f1;
          if constexpr (!LIMB) {
            f0 = tw[1].t.x;
            f1 = tw[1].t.y;
          } else {
            f0 = tw[1].t.x * limb_factor(rc.limb, tw[1].t.z);
            f1 = tw[1].t.y * limb_factor(rc.limb, tw[1].t.w);
          }
          rc.edge_lo = 2.0f * sH * e3 * (f0 + f1);
          e = rc.gminf + (1.0f - kH) * rc.dgf;
          e3 = e * e * e * isq;
          if constexpr (!LIMB) {
            f0 = tw[ng - 2].t.x;
            f1 = tw[ng - 2].t.y;
          } else {
            f0 = tw[ng - 2].t.x * limb_factor(rc.limb, tw[ng - 2].t.z);
            f1 = tw[ng - 2].t.y * limb_factor(rc.limb, tw[ng - 2].t.w);
          }
          rc.edge_hi = 2.0f * sH * e3 * (f0 + f1);
        }
        const float ew = rr.ew;
        const int jlo = max(ielo, tlo), jhi = min(iehi, thi - 1);
        // bins whose FP32 Romberg test came close to 0.02 are skipped here (bit it of rmask) and
        // added by rare_bins, before this warp's next radius: each bin still receives this
        // radius's value at the same place in its sum
        unsigned rmask = 0;
        int bi = 0;
        for (int j = jlo + lane; j <= jhi; j += 32, bi++) {
          const int jj = j - tlo;
          const float2 lo = edge_gc(m.eff[jj], rc), hi = edge_gc(m.eff[jj + 1], rc);
          bool rare = false;
          const float v =
              integ_bin<LIMB, false>(lo.x, lo.y, hi.x, hi.y, &m.eff[jj], m.red[jj] != 0, rc, tw, &rare, nullptr,
                                     nullptr, ge, j);
          if (rare) rmask |= 1u << bi;
          else m.acc[warp][jj] += v * ew;
        }
        if (rmask) {
          RareCtx rq;
          rq.tab = &tab;
          rq.s = &s;
          rq.ge = ge;
          rq.ifac_p = &R.ifac[c0 + ci];
          rq.itab = it;
          rare_bins<LIMB>(m.acc[warp], m.eff, m.red, lane, tlo, jlo, rc, tw, rq, ew, rmask);
        }
        __syncwarp();
      }
      __syncthreads();
    }
    // zone end: sum the warp rows in order, divide by the bin centre (renorm_relline_profile, Relprofile.cpp:753-762)
    for (int b = 0; b < kLineTile / kSumBins; b++) {
      const int jj = b * kSumBins + tid;
      double part = 0.0;
      if (jj < thi - tlo) {
        float v = 0.0f;
#pragma unroll
        for (int w = 0; w < kLineWarps; w++) { v += m.acc[w][jj]; m.acc[w][jj] = 0.0f; }
        const float emid = 0.5f * (m.eff[jj].x + m.eff[jj + 1].x);
        const float pv = v / emid;
        prof[pbase + z * zstride + tlo + jj] = pv;
        part = (double) pv;
      }
      const double zs = block_sum_d<kLineThreads>(part, m.red_sum);
      if (tid == 0 && b * kSumBins < thi - tlo) tsum[((size_t) set * nblk + tile * (kLineTile / kSumBins) + b) * nza + z] = zs;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// emission-angle distribution per zone (Relprofile.cpp:908-938), one CTA per set.  The set's
// (a, mu0)-interpolated transfer functions and emission-angle cosines on all table radii are
// written once per set by line_table_kernel (which the line profile reads as well) and read
// through the read-only cache, so that the histogram CTA's shared memory stays small; five CTAs
// per SM (48 registers: 0.82 -> 0.77 ms per 4096-set step against four; six spill).
// ---------------------------------------------------------------------------
struct HistSmem {
  RelxRadRec rec[kChunk];    // radius records of the current chunk
  float re[kChunk];
  float lh[kLineWarps][RELX_MAX_INCL][32];  // per-lane histograms, lane fastest (no bank conflicts)
  float hist[kLineWarps][RELX_MAX_INCL];
  float gfac[RELX_MAX_NG];   // d_gstar / sqrt(g*(1-g*))
  float gsf[RELX_MAX_NG];
};

// interpol_a_mu0 (Relprofile.cpp:39-80) of (trff1, trff2, cosne1, cosne2) at every (table radius,
// g*) of a set, for the line profile and the histogram: grid (chunks of kLineThreads entries, sets).
// A set's rel_nr x rel_ng float4 slot holds two planes of float2: (trff1, trff2), then (cosne1,
// cosne2), so that the line profile without a limb law reads half the bytes.
__global__ void __launch_bounds__(kLineThreads) line_table_kernel(RelxTables tab, const RelxSetState *__restrict__ sst,
                                                                  float4 *__restrict__ htab) {
  const int set = blockIdx.y;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.cached) return;
  const int nr = tab.rel_nr, nm = tab.rel_nmu0, ng = tab.rel_ng;
  const int q = blockIdx.x * kLineThreads + threadIdx.x;
  if (q >= nr * ng) return;
  const size_t b00 = (size_t) s.ind_a * nm + s.ind_mu0, b10 = (size_t) (s.ind_a + 1) * nm + s.ind_mu0;
  const size_t b01 = b00 + 1, b11 = b10 + 1;
  const float f1 = s.ifac_a, f2 = s.ifac_mu0;
  const float w00 = (1.0f - f1) * (1.0f - f2), w10 = f1 * (1.0f - f2), w01 = (1.0f - f1) * f2, w11 = f1 * f2;
  const float4 a = __ldg(&tab.rel_tc[b00 * nr * ng + q]), b = __ldg(&tab.rel_tc[b10 * nr * ng + q]);
  const float4 c = __ldg(&tab.rel_tc[b01 * nr * ng + q]), d = __ldg(&tab.rel_tc[b11 * nr * ng + q]);
  float2 *ht = reinterpret_cast<float2 *>(htab + (size_t) set * nr * ng);
  ht[q] = make_float2(w00 * a.x + w10 * b.x + w01 * c.x + w11 * d.x, w00 * a.y + w10 * b.y + w01 * c.y + w11 * d.y);
  ht[nr * ng + q] =
      make_float2(w00 * a.z + w10 * b.z + w01 * c.z + w11 * d.z, w00 * a.w + w10 * b.w + w01 * c.w + w11 * d.w);
}
static_assert(offsetof(HistSmem, rec) % 16 == 0, "radius records are staged as int4 rows");

// FP64 emission-angle cosine of one fine radius, table point g, branch k
// (interp_lin_2d_float then interp_lin_1d as Relprofile.cpp:67-77, 287-290)
__device__ double cosne_fp64(const RelxTables &tab, const RelxSetState &s, int itab, double ifac, int g, int k) {
  const int nr = tab.rel_nr, nm = tab.rel_nmu0, ng = tab.rel_ng;
  const size_t b00 = (size_t) s.ind_a * nm + s.ind_mu0, b10 = (size_t) (s.ind_a + 1) * nm + s.ind_mu0;
  const size_t b01 = b00 + 1, b11 = b10 + 1;
  double v[2];
  for (int q = 0; q < 2; q++) {
    int i = itab + 1 - q;  // q=0: lower radius (ind+1), q=1: upper (ind)
    float4 c00 = tab.rel_tc[(b00 * nr + i) * ng + g], c10 = tab.rel_tc[(b10 * nr + i) * ng + g];
    float4 c01 = tab.rel_tc[(b01 * nr + i) * ng + g], c11 = tab.rel_tc[(b11 * nr + i) * ng + g];
    double a = k ? c00.w : c00.z, b = k ? c10.w : c10.z, c = k ? c01.w : c01.z, d = k ? c11.w : c11.z;
    v[q] = lerp2((double) s.ifac_a, (double) s.ifac_mu0, a, b, c, d);
  }
  return lerp1(ifac, v[0], v[1]);
}

__global__ void __launch_bounds__(kLineThreads, 5) hist_kernel(RelxTables tab, const RelxSetState *__restrict__ sst,
                                                            const RelxRadial *__restrict__ srad, int nza,
                                                            const float4 *__restrict__ htab, float *__restrict__ dist) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HistSmem &m = *reinterpret_cast<HistSmem *>(smem_raw);
  const int set = blockIdx.x;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.model < RELX_RELXILL || s.cached || (int) blockIdx.y >= s.nz) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const RelxRadial &R = srad[set];
  const int nr = tab.rel_nr, ng = tab.rel_ng, n_incl = tab.x_nincl;
  // the set's interpolated table: (trff1, trff2) plane, then (cosne1, cosne2)
  const float2 *__restrict__ T = reinterpret_cast<const float2 *>(htab + (size_t) set * nr * ng);
  const float2 *__restrict__ C = T + nr * ng;
  {
    for (int g = tid; g < ng; g += kLineThreads) {
      double gs = 5e-3 + (1.0 - 2 * 5e-3) / (ng - 1) * ((float) g);
      double gs1 = 5e-3 + (1.0 - 2 * 5e-3) / (ng - 1) * ((float) 1);
      double dgs = (g == 0 || g == ng - 1) ? 0.5 * (gs1 - 5e-3) + 5e-3 : gs1 - 5e-3;
      m.gfac[g] = (float) (dgs / sqrt(gs - gs * gs));
      m.gsf[g] = (float) gs;
    }
  }
  __syncthreads();
  // Each lane owns (g*, branch) pairs q = lane, lane + 32, ... and keeps a private histogram in
  // shared memory; at the end of a zone the lanes are added by a shuffle tree and the warps in order.
  float(*lh)[32] = m.lh[warp];
  for (int j = 0; j < RELX_MAX_INCL; j++) lh[j][lane] = 0.0f;
  const float c4pi2 = (float) (4.0 * kPi * kPi);
  const int zb = gridDim.y > 1 ? (int) blockIdx.y : 0, ze = gridDim.y > 1 ? min((int) blockIdx.y + 1, s.nz) : s.nz;
  for (int z = zb; z < ze; z++) {
    const int i0 = s.zi0[z], i1 = s.zi1[z];
    for (int c0 = i0; c0 <= i1; c0 += kChunk) {
      const int cn = min(kChunk, i1 + 1 - c0);
      {
        const int4 *src = reinterpret_cast<const int4 *>(&R.rec[c0]);
        int4 *dst = reinterpret_cast<int4 *>(m.rec);
        for (int q = tid; q < cn * 4; q += kLineThreads) dst[q] = src[q];
        for (int q = tid; q < cn; q += kLineThreads) m.re[q] = (float) R.re[c0 + q];
      }
      __syncthreads();
      // four radii per warp: 8 lanes per radius, each lane takes a block of consecutive table points
      const int grp = lane >> 3, sub = lane & 7;
      for (int cb = warp * 4; cb < cn; cb += kLineWarps * 4) {
        const int ci = cb + grp;
        if (ci >= cn) continue;
        const RelxRadRec &rr = m.rec[ci];
        if (rr.ielo < 0) continue;  // radius outside the line-profile grid (Relprofile.cpp:863)
        const int it = rr.itab;
        const float fr = rr.ifac;
        const float re = m.re[ci];
        const float c = re * re * re * c4pi2 * rr.ew;
        const float dg = rr.dg.x, gmn = rr.gmin.x;
        // consecutive table points mostly fall into the same angle bin: each lane takes a block of
        // consecutive points, adds runs and flushes a run on a change of bin
        int cur0 = -1, cur1 = -1;
        float run0 = 0.0f, run1 = 0.0f;
        const int gper = (ng + 7) >> 3, g_end = min(ng, (sub + 1) * gper);
        for (int g = sub * gper; g < g_end; g++) {
          // trf(g*) and cosne(g*) at this radius: interp_lin_1d(ifac_r, T[ind+1], T[ind]) (Relprofile.cpp:280-293)
          const float2 lo = __ldg(&T[(it + 1) * ng + g]), hi = __ldg(&T[it * ng + g]);
          const float2 clo = __ldg(&C[(it + 1) * ng + g]), chi = __ldg(&C[it * ng + g]);
          const float ge_ = m.gsf[g] * dg + gmn;
          const float cg = c * ge_ * ge_ * m.gfac[g];
#pragma unroll
          for (int k = 0; k < 2; k++) {
            const float trf = k ? fr * hi.y + (1.0f - fr) * lo.y : fr * hi.x + (1.0f - fr) * lo.x;
            const float mu = k ? fr * chi.y + (1.0f - fr) * clo.y : fr * chi.x + (1.0f - fr) * clo.x;
            const float xb = (float) n_incl * (1.0f - mu);
            int b;
            if (fabsf(xb - rintf(xb)) < 1e-5f) {
              const double mud = cosne_fp64(tab, s, it, R.ifac[c0 + ci], g, k);
              b = ((int) (n_incl * (1 - mud) + 1)) - 1;  // get_cosne_bin, Relprofile.cpp:799-801
            } else {
              b = ((int) (xb + 1.0f)) - 1;
            }
            b = max(0, min(b, n_incl - 1));
            const float term = cg * trf;
            int &cur = k ? cur1 : cur0;
            float &run = k ? run1 : run0;
            if (b != cur) {
              if (cur >= 0) lh[cur][lane] += run;
              cur = b;
              run = 0.0f;
            }
            run += term;
          }
        }
        if (cur0 >= 0) lh[cur0][lane] += run0;
        if (cur1 >= 0) lh[cur1][lane] += run1;
      }
      __syncthreads();
    }
    // zone end: lanes by a shuffle tree, warps in order
    for (int j = 0; j < n_incl; j++) {
      float v = lh[j][lane];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) m.hist[warp][j] = v;
      lh[j][lane] = 0.0f;
    }
    __syncthreads();
    if (tid < n_incl) {
      float h = 0.0f;
      for (int w = 0; w < kLineWarps; w++) h += m.hist[w][tid];
      dist[((size_t) set * nza + z) * RELX_MAX_INCL + tid] = h;
    }
    __syncthreads();
  }
}

template <bool LIMB>
static size_t line_smem_t(int ng) {
  return sizeof(LineSmem<LIMB>) + sizeof(TW<LIMB>) * (size_t) (line_rows<LIMB>() * ng - 1);
}
size_t line_smem_bytes(int nr, int ng, bool limb, int tile) {
  (void) nr;
  (void) tile;
  return limb ? line_smem_t<true>(ng) : line_smem_t<false>(ng);
}
size_t hist_smem_bytes(int nr, int ng) {
  (void) nr;
  (void) ng;
  return sizeof(HistSmem);
}

cudaError_t relline_set_smem(int nr, int ng) {
  (void) nr;
  cudaError_t e;
#define SET(L)                                                                                             \
  e = cudaFuncSetAttribute(relline_kernel<L>, cudaFuncAttributeMaxDynamicSharedMemorySize,                \
                           (int) line_smem_t<L>(ng));                                                      \
  if (e != cudaSuccess) return e;
  SET(false) SET(true)
#undef SET
  return cudaFuncSetAttribute(hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) hist_smem_bytes(nr, ng));
}

cudaError_t launch_line_table(int n_sets, cudaStream_t s, const RelxTables &tab, const RelxSetState *sst,
                              float4 *htab) {
  const int nq = tab.rel_nr * tab.rel_ng;
  line_table_kernel<<<dim3((nq + kLineThreads - 1) / kLineThreads, n_sets), kLineThreads, 0, s>>>(tab, sst, htab);
  return cudaGetLastError();
}

// launches the line profile (both variants: a set runs in the one matching its limb law) in tiles of
// kLineTile bins and, for relxill models, the emission-angle histogram; htab: written by
// launch_line_table
cudaError_t launch_relline(bool hist, int n_sets, int nblk, cudaStream_t s, const RelxTables &tab,
                           const RelxSetIn *sin, const RelxSetState *sst, const RelxRadial *srad, const double *line_e,
                           int nza, float *prof, float *dist, double *tsum, bool any_limb, bool zsplit,
                           const float4 *htab) {
  const int ng = tab.rel_ng;
  const int ntile = (nblk * kSumBins + kLineTile - 1) / kLineTile;
  const dim3 grid(ntile, n_sets, zsplit ? nza : 1);
  relline_kernel<false><<<grid, kLineThreads, line_smem_t<false>(ng), s>>>(tab, sin, sst, srad, line_e, htab, nza, prof,
                                                                           tsum, nblk);
  if (any_limb)
    relline_kernel<true><<<grid, kLineThreads, line_smem_t<true>(ng), s>>>(tab, sin, sst, srad, line_e, htab, nza, prof,
                                                                           tsum, nblk);
  if (hist) return launch_hist(n_sets, s, tab, sst, srad, nza, dist, zsplit, htab);
  return cudaGetLastError();
}

cudaError_t launch_hist(int n_sets, cudaStream_t s, const RelxTables &tab, const RelxSetState *sst,
                        const RelxRadial *srad, int nza, float *dist, bool zsplit, const float4 *htab) {
  hist_kernel<<<dim3(n_sets, zsplit ? nza : 1), kLineThreads, hist_smem_bytes(tab.rel_nr, tab.rel_ng), s>>>(
      tab, sst, srad, nza, htab, dist);
  return cudaGetLastError();
}

}  // namespace relx
