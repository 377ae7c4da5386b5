// relline.cu -- line profile kernel: transfer-function interpolation, g*
// integration of every (radius, energy bin) pair and binning into radial zones
// and the emission-angle histogram (Relprofile.cpp:39-80, 141-303, 489-958).
//
// Launch: one CTA per (energy-bin tile, parameter set), 8 warps.
//  * The (a, mu0)-interpolated transfer functions of the set on all table radii
//    are staged once in shared memory (float4 trff1, trff2, cosne1, cosne2).
//  * Zone by zone, warps take fine radii round robin; per radius a warp builds
//    the radial interpolation trf(g*) (40 x float4) and its lanes integrate
//    consecutive energy bins (Romberg with the reference's prec 0.02 /
//    itermax 5, midpoint below 0.95 keV, sqrt edge terms within 5e-3 of
//    g* = 0 and 1).  Each warp adds into its own shared row; at the end of
//    the zone the rows are summed in warp order: no atomics, so every bin is
//    the same number in every run and in every batch composition.
//  * Arithmetic is FP32.  Bin edges and gmin/gmax enter as float-float so
//    that g* is accurate to an ulp.  Where an abscissa lies within 4e-6 grid
//    units of a transfer-function grid point (the reference's interpolation
//    weights are reversed, so the interpolant jumps there) the side is decided
//    in float-float arithmetic from the reference's own energy abscissa.
#include "relx_device.cuh"

namespace relx {

constexpr int kLineWarps = 8;
constexpr int kLineThreads = kLineWarps * 32;
constexpr int kLineTile = 512;   // energy bins per CTA
constexpr float kH = 5e-3f;

// ---- float-float arithmetic ---------------------------------------------
__device__ __forceinline__ float2 two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}
__device__ __forceinline__ float2 qts(float a, float b) {
  float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  float2 s = two_sum(a.x, b.x);
  return qts(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = __fadd_rn(e, __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
  return qts(p, e);
}
__device__ __forceinline__ float2 ff_mulf(float2 a, float b) {
  float p = __fmul_rn(a.x, b);
  float e = fmaf(a.x, b, -p);
  e = __fadd_rn(e, __fmul_rn(a.y, b));
  return qts(p, e);
}
__device__ __forceinline__ bool ff_ge(float2 a, float2 b) {
  float2 d = ff_add(a, ff_neg(b));
  return d.x > 0.0f || (d.x == 0.0f && d.y >= 0.0f);
}

// per-radius constants (warp uniform)
struct RadC {
  float2 gmin, gmax, dg;  // float-float
  float gminf, dgf, inv_dg;
  float edge_lo, edge_hi; // 2 sqrt(H) sum_k F_k(H), same at 1-H (emissivity factored out)
  float2 eH, e1H;         // gstar2ener(H), gstar2ener(1-H) in float-float
  bool red_H;             // gstar2ener(H) >= 0.95
  float ew;               // emissivity * weight
  int ng, limb;
  float inv_dgs;          // (ng-1) / (1-2H)
  const float2 *gs;       // table g* points as float-float (shared memory)
};

// abscissa of the reference in energy (for the grid-point side decision)
struct Absc {
  float2 lo, hi;  // rlo, rhi of the real integration
  int n, i;       // Romberg level and index (n = -1: midpoint)
};

// integrand F_k(x) = E^3 trf_k(x) [limb] / sqrt(x (1-x)), k = 0, 1  (relb_func,
// Relprofile.cpp:489-521 times (gmax - gmin) / emis)
__device__ __forceinline__ float2 eval_F(float x, float y, const RadC &rc, const float4 *__restrict__ tw,
                                         const Absc &ab) {
  const int ng = rc.ng;
  float t = (x - kH) * rc.inv_dgs;
  float tr = rintf(t);
  int ind;
  if (fabsf(t - tr) < 4e-6f && tr >= 1.0f && tr <= (float) (ng - 2)) {
    // side of grid point k from the reference's abscissa (float-float)
    int k = (int) tr;
    float2 eg;
    if (ab.n < 0) {
      eg = ff_mulf(ff_add(ab.lo, ab.hi), 0.5f);
    } else if (ab.i == (1 << ab.n)) {
      eg = ab.hi;
    } else {
      float2 w = ff_add(ab.hi, ff_neg(ab.lo));
      eg = ff_add(ab.lo, ff_mulf(w, ldexpf((float) ab.i, -ab.n)));
    }
    float2 G = ff_add(rc.gmin, ff_mul(rc.gs[k], rc.dg));
    ind = ff_ge(eg, G) ? k : k - 1;
  } else {
    ind = (int) floorf(t);
    ind = max(0, min(ind, ng - 2));
  }
  float inte = t - (float) ind;
  float inte1 = 1.0f - inte;
  float4 A = tw[ind], B = tw[ind + 1];
  float e = rc.gminf + x * rc.dgf;
  float e3 = e * e * e * rsqrtf(x * y);
  float f0 = e3 * (inte * A.x + inte1 * B.x);
  float f1 = e3 * (inte * A.y + inte1 * B.y);
  if (rc.limb) {
    float m0 = inte * A.z + inte1 * B.z, m1 = inte * A.w + inte1 * B.w;
    if (rc.limb == 1) { f0 *= (1.0f + 2.06f * m0); f1 *= (1.0f + 2.06f * m1); }
    else { f0 *= logf(1.0f + 1.0f / m0); f1 *= logf(1.0f + 1.0f / m1); }
  }
  return make_float2(f0, f1);
}

// romberg_integration (Relprofile.cpp:524-579) over [ga, gb] in g*, both
// branches in lock step; interior sums reuse the previous level's points.
__device__ __forceinline__ float romberg2(float ga, float ca, float gb, float cb, const RadC &rc,
                                          const float4 *__restrict__ tw, Absc ab) {
  const float pas0 = gb - ga;
  ab.n = 0;
  ab.i = 0;
  float2 fa = eval_F(ga, ca, rc, tw, ab);
  ab.i = 1;
  float2 fb = eval_F(gb, cb, rc, tw, ab);
  float ta0 = (fa.x + fb.x) * 0.5f, ta1 = (fa.y + fb.y) * 0.5f;
  float p0[7], p1[7];
  p0[0] = ta0 * pas0;
  p1[0] = ta1 * pas0;
  float s0 = 0.0f, s1 = 0.0f;
  bool c0 = false, c1 = false;
  float r0 = 0.0f, r1 = 0.0f;
#pragma unroll
  for (int n = 1; n <= 6; n++) {
    const float sc = ldexpf(1.0f, -n);
    const float pas = pas0 * sc;
    float a0 = 0.0f, a1 = 0.0f;
    ab.n = n;
    for (int i = 1; i < (1 << n); i += 2) {
      float u = pas0 * ((float) i * sc);
      ab.i = i;
      float2 f = eval_F(ga + u, ca - u, rc, tw, ab);
      a0 += f.x;
      a1 += f.y;
    }
    s0 += a0;
    s1 += a1;
    float q0[7], q1[7];
    q0[0] = (ta0 + s0) * pas;
    q1[0] = (ta1 + s1) * pas;
    float r = 1.0f;
#pragma unroll
    for (int ii = 1; ii <= n; ii++) {
      r *= 4.0f;
      q0[ii] = (r * q0[ii - 1] - p0[ii - 1]) / (r - 1.0f);
      q1[ii] = (r * q1[ii - 1] - p1[ii - 1]) / (r - 1.0f);
    }
    float o0 = fabsf(q0[n] - p0[n - 1]) / q0[n];
    float o1 = fabsf(q1[n] - p1[n - 1]) / q1[n];
    if (!c0) { r0 = q0[n]; if (!(o0 > 0.02f)) c0 = true; }
    if (!c1) { r1 = q1[n]; if (!(o1 > 0.02f)) c1 = true; }
#pragma unroll
    for (int ii = 0; ii <= n; ii++) { p0[ii] = q0[ii]; p1[ii] = q1[ii]; }
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

// integ_relline_bin (Relprofile.cpp:650-726) with the emissivity factored out
__device__ __forceinline__ float integ_bin(float2 Elo, float2 Ehi, bool red_lo, const RadC &rc,
                                           const float4 *__restrict__ tw) {
  float glo = ff_sub_to_float(Elo, rc.gmin) * rc.inv_dg;
  float clo = ff_sub_to_float(rc.gmax, Elo) * rc.inv_dg;
  if (glo < 0.0f) { glo = 0.0f; clo = 1.0f; } else if (glo > 1.0f) { glo = 1.0f; clo = 0.0f; }
  float ghi = ff_sub_to_float(Ehi, rc.gmin) * rc.inv_dg;
  float chi = ff_sub_to_float(rc.gmax, Ehi) * rc.inv_dg;
  if (ghi < 0.0f) { ghi = 0.0f; chi = 1.0f; } else if (ghi > 1.0f) { ghi = 1.0f; chi = 0.0f; }
  if (ghi == 0.0f) return 0.0f;
  float flu = 0.0f;
  bool has_lo = true, has_hi = true;
  float ga = glo, ca = clo, gb = ghi, cb = chi;
  bool red = red_lo;
  Absc ab;
  ab.lo = Elo;
  ab.hi = Ehi;
  if (glo <= kH) {
    float hhi = kH;
    ga = kH;
    ca = 1.0f - kH;
    red = rc.red_H;
    ab.lo = rc.eH;
    if (ghi <= kH) { hhi = ghi; has_lo = false; }
    flu += rc.edge_lo * sqrt_diff(hhi, glo);
  }
  if (ghi >= 1.0f - kH) {
    float hi_c = kH;  // 1 - hlo
    gb = 1.0f - kH;
    cb = kH;
    ab.hi = rc.e1H;
    if (glo >= 1.0f - kH) { hi_c = clo; has_hi = false; }
    flu += rc.edge_hi * sqrt_diff(hi_c, chi);
  }
  if (has_lo && has_hi) {
    if (red) {
      flu += romberg2(ga, ca, gb, cb, rc, tw, ab);
    } else {
      ab.n = -1;
      float2 f = eval_F(0.5f * (ga + gb), 0.5f * (ca + cb), rc, tw, ab);
      flu += (f.x + f.y) * (gb - ga);
    }
  }
  return flu;
}

struct LineSmem {
  float acc[kLineWarps][kLineTile];
  float2 eff[kLineTile + 1];
  unsigned char red[kLineTile];
  float4 tw[kLineWarps][RELX_MAX_NG];
  float hterm[kLineWarps][2 * RELX_MAX_NG];
  unsigned char hbin[kLineWarps][2 * RELX_MAX_NG];
  float hist[kLineWarps][RELX_MAX_INCL];
  float gfac[RELX_MAX_NG];  // d_gstar / sqrt(g*(1-g*)) at the table g* points
  float2 gs[RELX_MAX_NG];   // table g* points (Relprofile.cpp:104-106) as float-float
  double red_sum[kLineWarps + 1];
  // the (a, mu0)-interpolated table, [n_r][n_g]
  float4 tab[1];  // dynamic tail
};

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

template <bool HIST>
__global__ void __launch_bounds__(kLineThreads) relline_kernel(RelxTables tab, const RelxSetIn *__restrict__ sin,
                                                               const RelxSetState *__restrict__ sst,
                                                               const RelxRadial *__restrict__ srad,
                                                               const double *__restrict__ line_e, int nza,
                                                               float *__restrict__ prof, float *__restrict__ dist,
                                                               double *__restrict__ tsum, int ntile_max) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  LineSmem &m = *reinterpret_cast<LineSmem *>(smem_raw);
  const int set = blockIdx.y, tile = blockIdx.x;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK) return;
  const int tlo = s.win_lo + tile * kLineTile;
  const int thi = min(s.win_hi, tlo + kLineTile);
  const bool do_hist = HIST && tile == 0;
  if (tlo >= thi && !do_hist) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const RelxRadial &R = srad[set];
  const int nr = tab.rel_nr, nm = tab.rel_nmu0, ng = tab.rel_ng;
  const int nz = s.nz;
  const bool is_line = (s.model == RELX_RELLINE);
  const double *ge = is_line ? (line_e + sin[set].e_off) : tab.conv_e;
  const size_t pbase = is_line ? (size_t) sin[set].e_off : (size_t) set * nza * RELX_NCONV;
  const size_t zstride = is_line ? 0 : RELX_NCONV;
  float4 *tabI = m.tab;

  // stage the (a, mu0) interpolation of the transfer functions (interpol_a_mu0, Relprofile.cpp:39-80)
  {
    const size_t b00 = (size_t) s.ind_a * nm + s.ind_mu0, b10 = (size_t) (s.ind_a + 1) * nm + s.ind_mu0;
    const size_t b01 = b00 + 1, b11 = b10 + 1;
    const float f1 = s.ifac_a, f2 = s.ifac_mu0;
    const float w00 = (1.0f - f1) * (1.0f - f2), w10 = f1 * (1.0f - f2), w01 = (1.0f - f1) * f2, w11 = f1 * f2;
    for (int q = tid; q < nr * ng; q += kLineThreads) {
      float4 a = __ldg(&tab.rel_tc[b00 * nr * ng + q]), b = __ldg(&tab.rel_tc[b10 * nr * ng + q]);
      float4 c = __ldg(&tab.rel_tc[b01 * nr * ng + q]), d = __ldg(&tab.rel_tc[b11 * nr * ng + q]);
      float4 r;
      r.x = w00 * a.x + w10 * b.x + w01 * c.x + w11 * d.x;
      r.y = w00 * a.y + w10 * b.y + w01 * c.y + w11 * d.y;
      r.z = w00 * a.z + w10 * b.z + w01 * c.z + w11 * d.z;
      r.w = w00 * a.w + w10 * b.w + w01 * c.w + w11 * d.w;
      tabI[q] = r;
    }
    for (int j = tid; j <= thi - tlo && tlo < thi; j += kLineThreads) m.eff[j] = ff_from_double(ge[tlo + j]);
    for (int j = tid; j < thi - tlo; j += kLineThreads) m.red[j] = ge[tlo + j] >= 0.95 ? 1 : 0;
    for (int i = tid; i < kLineWarps * kLineTile; i += kLineThreads) (&m.acc[0][0])[i] = 0.0f;
    for (int g = tid; g < ng; g += kLineThreads)
      m.gs[g] = ff_from_double(5e-3 + (1.0 - 2 * 5e-3) / (ng - 1) * ((float) g));
    if (do_hist) {
      for (int g = tid; g < ng; g += kLineThreads) {
        double gs = 5e-3 + (1.0 - 2 * 5e-3) / (ng - 1) * ((float) g);
        double gs1 = 5e-3 + (1.0 - 2 * 5e-3) / (ng - 1) * ((float) 1);
        double gs0 = 5e-3;
        double dgs = (g == 0 || g == ng - 1) ? 0.5 * (gs1 - gs0) + 5e-3 : gs1 - gs0;
        m.gfac[g] = (float) (dgs / sqrt(gs - gs * gs));
      }
      for (int i = tid; i < kLineWarps * RELX_MAX_INCL; i += kLineThreads) (&m.hist[0][0])[i] = 0.0f;
    }
  }
  __syncthreads();

  const int n_incl = tab.x_nincl;
  const float inv_dgs = (float) ((ng - 1) / (1.0 - 2 * 5e-3));
  for (int z = 0; z < nz; z++) {
    const int i0 = s.zi0[z], i1 = s.zi1[z];
    for (int ii = i0 + warp; ii <= i1; ii += kLineWarps) {
      const int ielo = R.ielo[ii], iehi = R.iehi[ii];
      const bool overlap = (ielo >= 0) && (ielo < thi) && (iehi >= tlo);
      if (!overlap && !do_hist) continue;
      // trf(g*) at this radius: interp_lin_1d(ifac_r, T[ind+1], T[ind]) (Relprofile.cpp:280-293)
      const int it = R.itab[ii];
      const float fr = (float) R.ifac[ii];
      for (int g = lane; g < ng; g += 32) {
        float4 lo = tabI[(it + 1) * ng + g], hi = tabI[it * ng + g];
        float4 r;
        r.x = fr * hi.x + (1.0f - fr) * lo.x;
        r.y = fr * hi.y + (1.0f - fr) * lo.y;
        r.z = fr * hi.z + (1.0f - fr) * lo.z;
        r.w = fr * hi.w + (1.0f - fr) * lo.w;
        m.tw[warp][g] = r;
      }
      __syncwarp();
      const float4 *tw = m.tw[warp];
      RadC rc;
      rc.gmin = R.gmin_ff[ii];
      rc.gmax = R.gmax_ff[ii];
      rc.dg = R.dg_ff[ii];
      rc.gminf = rc.gmin.x;
      rc.dgf = rc.dg.x;
      rc.inv_dg = R.inv_dg[ii];
      rc.ng = ng;
      rc.limb = s.limb;
      rc.inv_dgs = inv_dgs;
      rc.ew = R.ew[ii];
      rc.eH = R.eH_ff[ii];
      rc.e1H = R.e1H_ff[ii];
      rc.red_H = R.red_H[ii] != 0;
      rc.gs = m.gs;
      {
        // int_edge norms (Relprofile.cpp:585-621): trf at g* = H is T[1], at 1 - H is T[ng-2]
        const float sH = sqrtf(kH), isq = rsqrtf(kH * (1.0f - kH));
        float e = rc.gminf + kH * rc.dgf;
        float e3 = e * e * e * isq;
        float4 A = tw[1];
        float f0 = A.x, f1 = A.y;
        if (rc.limb == 1) { f0 *= 1.0f + 2.06f * A.z; f1 *= 1.0f + 2.06f * A.w; }
        else if (rc.limb == 2) { f0 *= logf(1.0f + 1.0f / A.z); f1 *= logf(1.0f + 1.0f / A.w); }
        rc.edge_lo = 2.0f * sH * e3 * (f0 + f1);
        e = rc.gminf + (1.0f - kH) * rc.dgf;
        e3 = e * e * e * isq;
        A = tw[ng - 2];
        f0 = A.x;
        f1 = A.y;
        if (rc.limb == 1) { f0 *= 1.0f + 2.06f * A.z; f1 *= 1.0f + 2.06f * A.w; }
        else if (rc.limb == 2) { f0 *= logf(1.0f + 1.0f / A.z); f1 *= logf(1.0f + 1.0f / A.w); }
        rc.edge_hi = 2.0f * sH * e3 * (f0 + f1);
      }
      if (overlap) {
        const int jlo = max(ielo, tlo), jhi = min(iehi, thi - 1);
        for (int j = jlo + lane; j <= jhi; j += 32) {
          const int jj = j - tlo;
          float v = integ_bin(m.eff[jj], m.eff[jj + 1], m.red[jj] != 0, rc, tw);
          m.acc[warp][jj] += v * rc.ew;
        }
      }
      if (do_hist) {
        // emission-angle distribution (Relprofile.cpp:908-938)
        const float re = (float) R.re[ii];
        const float c = re * re * re * (float) (4.0 * kPi * kPi) * rc.ew;
        for (int q = lane; q < 2 * ng; q += 32) {
          const int g = q >> 1, k = q & 1;
          const float4 T = tw[g];
          const float ge_ = m.gs[g].x * rc.dgf + rc.gminf;
          const float trf = k ? T.y : T.x;
          m.hterm[warp][q] = c * ge_ * ge_ * m.gfac[g] * trf;
          float mu = k ? T.w : T.z;
          float xb = (float) n_incl * (1.0f - mu);
          float xr = rintf(xb);
          if (fabsf(xb - xr) < 1e-5f) {
            double mud = cosne_fp64(tab, s, it, R.ifac[ii], g, k);
            int b = ((int) (n_incl * (1 - mud) + 1)) - 1;
            m.hbin[warp][q] = (unsigned char) max(0, min(b, n_incl - 1));
          } else {
            int b = ((int) (xb + 1.0f)) - 1;
            m.hbin[warp][q] = (unsigned char) max(0, min(b, n_incl - 1));
          }
        }
        __syncwarp();
        if (lane < n_incl) {
          float acc = 0.0f;
          for (int q = 0; q < 2 * ng; q++)
            if (m.hbin[warp][q] == lane) acc += m.hterm[warp][q];
          m.hist[warp][lane] += acc;
        }
      }
      __syncwarp();
    }
    __syncthreads();
    // zone end: sum the warp rows in order, divide by the bin centre (renorm_relline_profile, Relprofile.cpp:753-762)
    double part = 0.0;
    for (int jj = tid; jj < thi - tlo; jj += kLineThreads) {
      float v = 0.0f;
#pragma unroll
      for (int w = 0; w < kLineWarps; w++) { v += m.acc[w][jj]; m.acc[w][jj] = 0.0f; }
      const float emid = 0.5f * (m.eff[jj].x + m.eff[jj + 1].x);
      float pv = v / emid;
      prof[pbase + z * zstride + tlo + jj] = pv;
      part += (double) pv;
    }
    double zs = block_sum_d<kLineThreads>(part, m.red_sum);
    if (tid == 0) tsum[((size_t) set * ntile_max + tile) * nza + z] = zs;
    if (do_hist && tid < n_incl) {
      float h = 0.0f;
      for (int w = 0; w < kLineWarps; w++) { h += m.hist[w][tid]; m.hist[w][tid] = 0.0f; }
      dist[((size_t) set * nza + z) * RELX_MAX_INCL + tid] = h;
    }
    __syncthreads();
  }
}

size_t line_smem_bytes(int nr, int ng) { return sizeof(LineSmem) + sizeof(float4) * (size_t) (nr * ng - 1); }

cudaError_t relline_set_smem(size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(relline_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(relline_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
}

cudaError_t launch_relline(bool hist, dim3 grid, size_t smem, cudaStream_t s, const RelxTables &tab,
                           const RelxSetIn *sin, const RelxSetState *sst, const RelxRadial *srad, const double *line_e,
                           int nza, float *prof, float *dist, double *tsum, int ntile_max) {
  if (hist)
    relline_kernel<true><<<grid, kLineThreads, smem, s>>>(tab, sin, sst, srad, line_e, nza, prof, dist, tsum, ntile_max);
  else
    relline_kernel<false><<<grid, kLineThreads, smem, s>>>(tab, sin, sst, srad, line_e, nza, prof, dist, tsum, ntile_max);
  return cudaGetLastError();
}

}  // namespace relx
