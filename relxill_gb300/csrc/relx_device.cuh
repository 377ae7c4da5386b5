// relx_device.cuh -- device helpers shared by the relxill kernels: the
// reference's search and interpolation conventions, Kerr-metric formulas in
// FP64, and float-float (double-single) helpers for bin edges.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "relx_common.h"
#include "relx_fpconv.cuh"

namespace relx {

constexpr double kPi = 3.14159265358979323846;

// ---- searches with the conventions of relutility.c:135-211 ----------------
// ascending arr: returns k with arr[k] <= val < arr[k+1], clamped to [0, n-2]
template <typename T>
__device__ __forceinline__ int bsearch_asc(const T *arr, int n, T val) {
  int klo = 0, khi = n - 1;
  while (khi - klo > 1) {
    int k = (khi + klo) >> 1;
    if (arr[k] > val) khi = k; else klo = k;
  }
  return klo;
}
// bsearch_asc of an ascending array of positive values (largest k in [0, n-2] with a[k] <= v)
__device__ __forceinline__ int bsearch_asc_pos(const double *a, int n, double v) {
  int lo = 0, hi = n;  // count of entries <= v
  while (lo < hi) {
    const int k = (lo + hi) >> 1;
    if (!dgt(a[k], v)) lo = k + 1; else hi = k;
  }
  return max(0, min(lo - 1, n - 2));
}
// number of entries > v of a descending array of positive values
__device__ __forceinline__ int count_gt_desc_pos(const double *a, int n, double v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int k = (lo + hi) >> 1;
    if (dgt(a[k], v)) lo = k + 1; else hi = k;
  }
  return lo;
}
// bsearch_desc of a descending array of positive values (largest k in [0, n-2] with a[k] >= v)
__device__ __forceinline__ int bsearch_desc_pos(const double *a, int n, double v) {
  int lo = 0, hi = n;  // count of entries >= v
  while (lo < hi) {
    const int k = (lo + hi) >> 1;
    if (dge(a[k], v)) lo = k + 1; else hi = k;
  }
  return max(0, min(lo - 1, n - 2));
}

// index k of the log conv grid with ge[k] <= e < ge[k+1] (clamped to [0, N-1]), as
// binary_search would return it: a first guess from the logarithm, then exact comparisons
__device__ __forceinline__ int conv_index(const RelxTables &tab, double e) {
  const double *ge = tab.conv_e;
  const float2 *gf = tab.conv_eff;  // .x = (float) ge
  const float ef = d2f(e);
  // the grid is logarithmic (edge k at exp(log E_0 + k step)), so the float position kf is the bin
  // up to about 1e-3 of a bin (logf, the rounding of e, of the two constants and of the product);
  // more than 4e-3 of a bin away from an edge the bin is certain without reading the grid
  const float kf = (logf(ef) - tab.conv_lg0) * tab.conv_ilg;
  const float kfl = floorf(kf), fr = kf - kfl;
  int k = (int) kfl;
  if (fr > 4e-3f && fr < 1.0f - 4e-3f && kfl >= 0.0f && kfl <= (float) (RELX_NCONV - 1)) return k;
  k = max(0, min(k, RELX_NCONV - 1));
  // ge[k] > e, decided in float unless the float values tie
  while (k > 0 && (gf[k].x > ef || (gf[k].x == ef && dgt(ge[k], e)))) k--;
  while (k < RELX_NCONV - 1 && (gf[k + 1].x < ef || (gf[k + 1].x == ef && !dgt(ge[k + 1], e)))) k++;
  return k;
}

// Searches over FP64 arrays guided by float copies.  Rounding to float is monotone, so a strict
// float comparison decides the FP64 one; only float ties are compared in FP64 (FP64 compares
// share the narrow FP64 pipe).
// number of entries of the descending array a that are > v
__device__ __forceinline__ int count_gt_desc(const double *a, const float *af, int n, double v, float vf) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int k = (lo + hi) >> 1;
    if (af[k] > vf) lo = k + 1; else hi = k;
  }
  while (lo < n && af[lo] == vf && a[lo] > v) lo++;
  return lo;
}
// bsearch_asc (largest k in [0, n-2] with a[k] <= v, 0 below the range) of an ascending array
__device__ __forceinline__ int bsearch_asc_exact(const double *a, const float *af, int n, double v, float vf) {
  int lo = 0, hi = n;  // count of entries < v in float
  while (lo < hi) {
    const int k = (lo + hi) >> 1;
    if (af[k] < vf) lo = k + 1; else hi = k;
  }
  while (lo < n && af[lo] == vf && a[lo] <= v) lo++;  // lo = count of entries <= v
  return max(0, min(lo - 1, n - 2));
}
// bsearch_desc of a strictly descending array (the largest k in [0, n-2] with a[k] >= v, 0 when
// there is none), guided by the float copy af
__device__ __forceinline__ int bsearch_desc_exact(const double *a, const float *af, int n, double v, float vf) {
  int lo = 0, hi = n;  // count of entries > v in float
  while (lo < hi) {
    const int k = (lo + hi) >> 1;
    if (af[k] > vf) lo = k + 1; else hi = k;
  }
  while (lo < n && af[lo] == vf && a[lo] >= v) lo++;  // lo = count of entries >= v
  return max(0, min(lo - 1, n - 2));
}
// descending arr (inv_binary_search, relutility.c:195-211)
__device__ __forceinline__ int bsearch_desc(const double *arr, int n, double val) {
  int klo = 0, khi = n - 1;
  while (khi - klo > 1) {
    int k = (khi + klo) >> 1;
    if (arr[k] < val) khi = k; else klo = k;
  }
  return klo;
}

// relutility.c:24-26 and :46-58
__device__ __forceinline__ double lerp1(double f, double lo, double hi) { return f * hi + (1.0 - f) * lo; }
__device__ __forceinline__ float lerp1(float f, float lo, float hi) { return f * hi + (1.0f - f) * lo; }
__device__ __forceinline__ double lerp2(double f1, double f2, double r11, double r12, double r21, double r22) {
  return (1.0 - f1) * (1.0 - f2) * r11 + (f1) * (1.0 - f2) * r12 + (1.0 - f1) * (f2) * r21 + (f1) * (f2) * r22;
}

// ---- Kerr metric (Relphysics.cpp), FP64 -------------------------------------
__device__ __forceinline__ double kerr_rms(double a) {
  double sign = (a < 0) ? -1.0 : 1.0;
  // cube roots as cbrt (the reference writes pow(x, 1.0/3.0); the two differ by about an ulp)
  double z1 = 1.0 + cbrt(1.0 - a * a) * (cbrt(1.0 + a) + cbrt(1.0 - a));
  double z2 = sqrt((3.0 * a * a) + (z1 * z1));
  return 3.0 + z2 - sign * sqrt((3.0 - z1) * (3.0 + z1 + (2 * z2)));
}
__device__ __forceinline__ double kerr_rplus(double a) { return 1 + sqrt(1 - a * a); }
__device__ __forceinline__ double relat_abberation(double del, double beta) {
  return acos((cos(del) - beta) / (1 - beta * cos(del)));
}
__device__ __forceinline__ double calc_g_inf(double h, double a) { return sqrt(1.0 - (2 * h / (h * h + a * a))); }
__device__ __forceinline__ double doppler_factor(double del, double bet) {
  return sqrt(1.0 - bet * bet) / (1.0 + bet * cos(del));
}
// gi_potential_lp, Relphysics.cpp:163-207
__device__ __forceinline__ double gi_potential_lp(double r, double a, double h, double bet, double del) {
  double sr = sqrt(r);
  double ut_d = ((r * sr + a) / (sr * sqrt(r * r - 3 * r + 2 * a * sr)));
  double ut_h = sqrt((h * h + a * a) / (h * h - 2 * h + a * a));
  double gi = ut_d / ut_h;
  if (fabs(bet) < 1e-6) return gi;
  double gam = 1.0 / sqrt(1.0 - bet * bet);
  double sign = (del > kPi / 2) ? -1.0 : 1.0;
  double delta_eq = h * h - 2 * h + a * a;
  double sd = sin(del);
  double h2a2 = h * h + a * a;
  double q2 = (sd * sd) * (h2a2 * h2a2 / delta_eq) - a * a;
  double beta_fac = sqrt(h2a2 * h2a2 - delta_eq * (q2 + a * a));
  beta_fac = gam * (1.0 + sign * beta_fac / h2a2 * bet);
  return gi / beta_fac;
}
// Relphysics.cpp:123-125
__device__ __forceinline__ double density_ss73_zone_a(double radius, double rms) {
  double q = 1 - sqrt(rms / radius);
  return pow(radius / rms, 1.5) / (q * q);
}

// ---- float-float (value = hi + lo) ------------------------------------------
__device__ __forceinline__ float2 ff_from_double(double d) {
  float hi = __double2float_rn(d);
  float lo = __double2float_rn(d - (double) hi);
  return make_float2(hi, lo);
}
// double -> float-float without the FP64 pipe (which runs at 2 lanes/clk/SM): hi keeps the
// leading 24 significant bits of d (truncated), lo is the rest rounded to float, so hi + lo = d to
// about 2^-48 relative.  For |d| in [2^-60, 2^61); other values give (float) d and 0 (integer
// operations throughout: a conversion instruction on a rare path is if-converted into every call).
__device__ __forceinline__ float2 ff_split(double d) {
  const unsigned long long b = (unsigned long long) __double_as_longlong(d);
  const unsigned long long ab = b & 0x7fffffffffffffffull;
  const int e = (int) (ab >> 52) - 1023;
  if (e < -60 || e > 60) return make_float2(d2f(d), 0.0f);  // not met by the values split here
  const unsigned int sgn = (unsigned int) (b >> 32) & 0x80000000u;
  const float hi = __uint_as_float(sgn | ((unsigned int) (e + 127) << 23) | ((unsigned int) (ab >> 29) & 0x7fffffu));
  const float r = __uint2float_rn((unsigned int) (ab & 0x1fffffffull));
  const float sc = __uint_as_float((unsigned int) (e - 52 + 127) << 23);
  const float lo = __uint_as_float(__float_as_uint(r * sc) | sgn);
  return make_float2(hi, lo);
}
// (a.hi + a.lo) - (b.hi + b.lo) in float: the difference of the high parts is exact where they are
// within a factor 2 of each other (Sterbenz), so the sign is right and the value within about an
// ulp there; elsewhere both roundings are an ulp of the result
__device__ __forceinline__ float ff_diff(float2 a, float2 b) {
  return __fadd_rn(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
}
// a > b and a >= b for doubles with their float roundings af, bf: rounding to float is monotone,
// so float copies that differ decide, and only tied copies are compared in FP64
__device__ __forceinline__ bool gt_f(double a, float af, double b, float bf) { return af != bf ? af > bf : a > b; }
__device__ __forceinline__ bool ge_f(double a, float af, double b, float bf) { return af != bf ? af > bf : a >= b; }
// (a.hi + a.lo) - (b.hi + b.lo) rounded to float, error ~1 ulp of the result
__device__ __forceinline__ float ff_sub_to_float(float2 a, float2 b) {
  float s = __fsub_rn(a.x, b.x);
  float bb = __fsub_rn(s, a.x);
  float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(-b.x, bb));  // two-sum error
  return __fadd_rn(s, __fadd_rn(err, __fsub_rn(a.y, b.y)));
}

// ---- float-float arithmetic on the FP32 pipe (FP64 runs at 1/64 of the FP32 rate on this part)
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

// a / b rounded to float from float-float operands (one correction step of the float quotient)
__device__ __forceinline__ float ff_div_to_float(float2 a, float2 b) {
  const float q1 = a.x / b.x;
  const float2 r = ff_add(a, ff_neg(ff_mulf(b, q1)));  // a - q1 b
  return q1 + r.x / b.x;
}
__device__ __forceinline__ float2 ff_addf(float2 a, float b) {
  float2 s = two_sum(a.x, b);
  return qts(s.x, __fadd_rn(s.y, a.y));
}
__device__ __forceinline__ double ff_to_double(float2 a) { return (double) a.x + (double) a.y; }

// block-wide float-float sum with a fixed reduction tree (deterministic); scratch holds NT/32 + 1
template <int NT>
__device__ __forceinline__ float2 block_sum_ff(float2 v, float2 *scratch) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float2 t;
    t.x = __shfl_xor_sync(0xffffffffu, v.x, o);
    t.y = __shfl_xor_sync(0xffffffffu, v.y, o);
    v = ff_add(v, t);
  }
  __syncthreads();
  if (lane == 0) scratch[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    float2 r = make_float2(0.0f, 0.0f);
    for (int i = 0; i < NT / 32; i++) r = ff_add(r, scratch[i]);
    scratch[NT / 32] = r;
  }
  __syncthreads();
  const float2 r = scratch[NT / 32];
  __syncthreads();
  return r;
}

// block-wide sum in FP64 with a fixed reduction tree (deterministic)
template <int NT>
__device__ __forceinline__ double block_sum_d(double v, double *scratch) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) scratch[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < NT / 32; i++) r += scratch[i];
    scratch[NT / 32] = r;
  }
  __syncthreads();
  r = scratch[NT / 32];
  __syncthreads();
  return r;
}

template <int NT>
__device__ __forceinline__ int block_min_i(int v, int *scratch) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  int r = scratch[0];
  for (int i = 1; i < NT / 32; i++) r = min(r, scratch[i]);
  __syncthreads();
  return r;
}
template <int NT>
__device__ __forceinline__ int block_max_i(int v, int *scratch) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
  __syncthreads();
  int r = scratch[0];
  for (int i = 1; i < NT / 32; i++) r = max(r, scratch[i]);
  __syncthreads();
  return r;
}

// Sum over the coarse normalisation grid of the cut-off power law times the bin centre, scaled to
// the xillver table normalisation (calcNormWrtXillverTableSpec with spec_cutoffpl,
// Xillspec.cpp:179-233): FP32 terms summed as float-float by one warp, every lane returns the
// total.  cpow: E^-Gamma per coarse bin, or null to compute it here.
__device__ __forceinline__ double primary_qsum_warp(const RelxTables &tab, float gam, float ecut, const float *cpow) {
  const int lane = threadIdx.x & 31;
  float2 part = make_float2(0.0f, 0.0f);
  for (int b = lane; b < RELX_NCOARSE; b += 32) {
    const float4 t = tab.coarse_t[b];  // bin centre, width, centre as float-float (0 outside the band)
    const float pw = cpow ? cpow[b] : powf(t.x, -gam);
    const float term = expf(1.0f / ecut) * pw * expf(-t.x / ecut) * t.y;
    part = ff_add(part, ff_mulf(make_float2(t.z, t.w), term));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float2 u;
    u.x = __shfl_xor_sync(0xffffffffu, part.x, o);
    u.y = __shfl_xor_sync(0xffffffffu, part.y, o);
    part = ff_add(part, u);
  }
  return ff_to_double(part) * (1e20 * 1.602177e-09 / (1e15 / 4.0 / kPi));  // one product, not a division
}

// E F_E of the table interpolated at photon energy e [keV] in the frame shifted by 1 + z, from the
// first grid point at or above it (c_donthcomp's walk, donthcomp.c:770-787)
__device__ __forceinline__ double nth_prim_at(const double *x, const double *sp, int nth, double e, double zp1) {
  const double t = e * zp1;
  int lo = 1, hi = nth + 1;  // first j in [1, nth] with x[j] * 511 >= t, nth + 1 if none
  while (lo < hi) {
    const int k = (lo + hi) >> 1;
    if (x[k] * 511. < t) lo = k + 1; else hi = k;
  }
  const int j = lo;
  if (j > nth) return 0.0;
  if (j == 1) return sp[1];
  const int jl = j - 1;
  return sp[jl] + (e / 511. * zp1 - x[jl]) * (sp[jl + 1] - sp[jl]) / (x[jl + 1] - x[jl]);
}

// 1 / f_spp(1 / xn): the table's E F_E at xn = (1 + z) / 511 (donthcomp.c:617-638, 754-758)
__device__ __forceinline__ double nth_normfac(const double *x, const double *sp, int nth, double zp1) {
  const double xn = zp1 / 511.;
  const double xx = 1 / (1 / xn);
  int ih = 2;
  while (ih < nth && xx > x[ih]) ++ih;
  const int il = ih - 1;
  return 1 / (sp[il] + (sp[ih] - sp[il]) * (xx - x[il]) / (x[ih] - x[il]));
}

// photon flux of the nthcomp table on the bin [e0, e1] in the frame shifted by zp1 = 1 + z
// (c_donthcomp's last loop, donthcomp.c:788-792); normfac from nth_normfac at the same shift
__device__ __forceinline__ double nth_bin(const double *x, const NthTable &T, double e0, double e1, double zp1,
                                          double normfac) {
  const double p0 = nth_prim_at(x, T.sp, T.n, e0, zp1), p1 = nth_prim_at(x, T.sp, T.n, e1, zp1);
  return (p1 / (e1 * e1) + p0 / (e0 * e0)) * .5 * (e1 - e0) * normfac;
}

// E F_E of the nthcomp table at t = E (1 + z) in keV, FP32 from the table's float copy.  The
// interpolation is continuous in t (linear between grid points, zero at the table's last point), so
// the bracketing point comes from the grid position log2(t / (x_1 511)) / step without exact
// comparisons; beyond the table 0, below its first point the first value (donthcomp.c:768-786)
__device__ __forceinline__ float nth_prim_f(const NthGrid &G, const NthTable &T, float t) {
  const float L = (log2f(t) - G.l2x511) * G.inv_l2step;
  if (!(L > 0.0f)) return T.spf[1];
  const int j = (int) ceilf(L) + 1;  // first point with x_j 511 >= t (to rounding)
  if (j > T.n) return 0.0f;
  const int jl = j - 1;
  const float xl = G.p[jl].x.x, xh = G.p[jl + 1].x.x;
  const float f = (t * (1.0f / 511.0f) - xl) / (xh - xl);
  return T.spf[jl] + f * (T.spf[jl + 1] - T.spf[jl]);
}

}  // namespace relx
