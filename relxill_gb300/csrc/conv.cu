// conv.cu -- per-zone relativistic convolution, zone sum, primary continuum
// and rebinning to the caller's energy grid.
//
// The reference convolves on the 4096-bin log grid with FFTW: the xillver
// spectrum and the relline profile rotated so that the 1 keV bin is index 0
// are both weighted by E/dE, transformed r2c, multiplied, transformed back,
// divided by E/dE and normalised to sum(rel) * sum(xill) / sum(conv) over
// 0.01-1000 keV (Relbase.cpp:119-230).  That is a circular convolution.  Here
// it is evaluated directly over the support of the relline profile: every
// output bin is a sum of non-negative products, so FP32 keeps ~1e-6 relative
// accuracy in every bin, including bins many decades below the peak where an
// FP32 FFT (absolute error ~1e-7 of the peak) would not.
//
// conv_zone_kernel: one CTA per (zone, set), 256 threads x 16 output bins,
// register-tiled (16 x 16 products per 47 shared-memory loads).
#include "relx_device.cuh"

namespace relx {

constexpr int kConvThreads = 256;
constexpr int kConvR = 16;  // output bins per thread
constexpr int kN = RELX_NCONV;
static_assert(kConvThreads * kConvR == kN, "conv tiling covers the grid");

__device__ __forceinline__ int skew(int m) { return m + (m >> 4); }

struct ConvSmem {
  float xs[kN + kN / 16];    // x * cf, skewed
  float hr[kN + kConvR];     // rel * cf over the profile window, zero padded
  double red[kConvThreads / 32 + 1];
};

// y[k0 + r] = sum_{i in [wlo, whi)} hr[i - wlo] * xs[(k0 + r + p - i) mod N]
__device__ __forceinline__ void conv_tile(const ConvSmem &m, int k0, int p, int wlo, int whi, float y[kConvR]) {
#pragma unroll
  for (int r = 0; r < kConvR; r++) y[r] = 0.0f;
  for (int i0 = wlo; i0 < whi; i0 += kConvR) {
    const int base = k0 + p - i0 - (kConvR - 1);
    float xr[2 * kConvR - 1];
#pragma unroll
    for (int c = 0; c < 2 * kConvR - 1; c++) xr[c] = m.xs[skew((base + c) & (kN - 1))];
#pragma unroll
    for (int d = 0; d < kConvR; d++) {
      const float h = m.hr[i0 - wlo + d];
#pragma unroll
      for (int r = 0; r < kConvR; r++) y[r] = fmaf(h, xr[r - d + kConvR - 1], y[r]);
    }
  }
}

// sum over tiles of the per-(tile, zone) profile sums written by the line kernel
__device__ __forceinline__ double zone_profile_sum(const double *tsum, int set, int ntile_max, int nza, int z, int ntiles) {
  double s = 0.0;
  for (int t = 0; t < ntiles; t++) s += tsum[((size_t) set * ntile_max + t) * nza + z];
  return s;
}

// relline renormalisation (renorm_relline_profile, Relprofile.cpp:766-781)
__device__ __forceinline__ double profile_scale(const RelxSetState &s, const double *tsum, int set, int ntile_max,
                                                int nza, int tile_bins) {
  if (!(s.relline_norm > 0.0)) return 1.0;
  const int ntiles = (s.win_hi - s.win_lo + tile_bins - 1) / tile_bins;
  double sum = 0.0;
  for (int z = 0; z < s.nz; z++) sum += zone_profile_sum(tsum, set, ntile_max, nza, z, ntiles);
  return s.relline_norm / sum;
}

// shared part: convolution of xs with hr, normalisation, output (fout * norm)
__device__ void conv_normalize_store(ConvSmem &m, const RelxTables &tab, int wlo, int whi, double sx, double sr,
                                     float *out) {
  const int tid = threadIdx.x;
  const int k0 = tid * kConvR;
  float y[kConvR];
  conv_tile(m, k0, tab.conv_pos1, wlo, whi, y);
  double part = 0.0;
#pragma unroll
  for (int r = 0; r < kConvR; r++) {
    const int k = k0 + r;
    y[r] = y[r] / tab.conv_cf[k];
    if (k >= tab.conv_band_lo && k <= tab.conv_band_hi) part += (double) y[r];
  }
  const double sc = block_sum_d<kConvThreads>(part, m.red);
  const float norm = (float) (sr * sx / sc);
#pragma unroll
  for (int r = 0; r < kConvR; r += 4) {
    float4 v = make_float4(y[r] * norm, y[r + 1] * norm, y[r + 2] * norm, y[r + 3] * norm);
    *reinterpret_cast<float4 *>(out + k0 + r) = v;
  }
}

__global__ void __launch_bounds__(kConvThreads) conv_zone_kernel(RelxTables tab, const RelxSetState *__restrict__ sst,
                                                                 const float *__restrict__ prof,
                                                                 const double *__restrict__ tsum, int ntile_max,
                                                                 int tile_bins, const float *__restrict__ xill, int nza,
                                                                 float *__restrict__ cout) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ConvSmem &m = *reinterpret_cast<ConvSmem *>(smem_raw);
  const int z = blockIdx.x, set = blockIdx.y, tid = threadIdx.x;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.model < RELX_RELXILL || z >= s.nz) return;
  float *out = cout + ((size_t) set * nza + z) * kN;
  const double scale = profile_scale(s, tsum, set, ntile_max, nza, tile_bins);
  const int ntiles = (s.win_hi - s.win_lo + tile_bins - 1) / tile_bins;
  // relxill_convolution_multizone skips zones without flux (Relxill.cpp:455-457)
  const double zsum = zone_profile_sum(tsum, set, ntile_max, nza, z, ntiles) * scale;
  if (zsum < 1e-12) {
    for (int k = tid; k < kN; k += kConvThreads) out[k] = 0.0f;
    return;
  }
  const int wlo = s.win_lo, whi = s.win_hi;
  const float fscale = (float) scale;
  const float *pz = prof + ((size_t) set * nza + z) * kN;
  // relline profile weighted by E/dE over its window; band sum of the profile
  double pr = 0.0;
  for (int i = tid; i < whi - wlo + kConvR; i += kConvThreads) {
    const int j = wlo + i;
    float v = 0.0f;
    if (j < whi) {
      const float fr = pz[j] * fscale;
      v = fr * tab.conv_cf[j];
      if (j >= tab.conv_band_lo && j <= tab.conv_band_hi) pr += (double) fr;
    }
    m.hr[i] = v;
  }
  // xillver spectrum of the zone rebinned onto the conv grid (_rebin_spectrum, relutility.c:549-601)
  const float *xz = xill + ((size_t) set * nza + z) * tab.x_nener_pad;
  double px = 0.0;
  for (int j = tid; j < kN; j += kConvThreads) {
    const int i0 = tab.rb_imin[j], i1 = tab.rb_imax[j];
    float v = 0.0f;
    if (i0 >= 0) {
      if (i0 == i1) {
        v = tab.rb_fmin[j] * xz[i0];
      } else {
        v = xz[i0] * tab.rb_fmin[j] + xz[i1] * tab.rb_fmax[j];
        for (int q = i0 + 1; q <= i1 - 1; q++) v += xz[q];
      }
    }
    if (j >= tab.conv_band_lo && j <= tab.conv_band_hi) px += (double) v;
    m.xs[skew(j)] = v * tab.conv_cf[j];
  }
  const double sr = block_sum_d<kConvThreads>(pr, m.red);
  const double sx = block_sum_d<kConvThreads>(px, m.red);
  conv_normalize_store(m, tab, wlo, whi, sx, sr, out);
}

// relconv (relconv_kernel, Relbase.cpp:257-289): the caller's spectrum is
// rebinned onto the conv grid, convolved with the single-zone profile and
// rebinned back; output bins outside 0.01-1000 keV are zero.
__global__ void __launch_bounds__(kConvThreads) relconv_conv_kernel(RelxTables tab, const RelxSetIn *__restrict__ sin,
                                                                    const RelxSetState *__restrict__ sst,
                                                                    const float *__restrict__ prof,
                                                                    const double *__restrict__ tsum, int ntile_max,
                                                                    int tile_bins, int nza, const double *__restrict__ user_e,
                                                                    const double *__restrict__ user_f, float *__restrict__ cout,
                                                                    int *__restrict__ sflag) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ConvSmem &m = *reinterpret_cast<ConvSmem *>(smem_raw);
  const int set = blockIdx.x, tid = threadIdx.x;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.model != RELX_RELCONV) return;
  const RelxSetIn &in = sin[set];
  const double *ue = user_e + in.e_off;
  const double *uf = user_f + in.e_off;
  const int nu = in.n_ener;
  float *out = cout + (size_t) set * nza * kN;
  // conv_model requires a positive input sum (LocalModel.cpp:84-86)
  double ps = 0.0;
  for (int i = tid; i < nu; i += kConvThreads) ps += uf[i];
  const double usum = block_sum_d<kConvThreads>(ps, m.red);
  if (!(usum > 0.0)) {
    if (tid == 0) sflag[set] = RELX_ERR_INPUT;
    return;
  }
  const double scale = profile_scale(s, tsum, set, ntile_max, nza, tile_bins);
  const int wlo = s.win_lo, whi = s.win_hi;
  const float fscale = (float) scale;
  const float *pz = prof + (size_t) set * nza * kN;
  double pr = 0.0;
  for (int i = tid; i < whi - wlo + kConvR; i += kConvThreads) {
    const int j = wlo + i;
    float v = 0.0f;
    if (j < whi) {
      const float fr = pz[j] * fscale;
      v = fr * tab.conv_cf[j];
      if (j >= tab.conv_band_lo && j <= tab.conv_band_hi) pr += (double) fr;
    }
    m.hr[i] = v;
  }
  // _rebin_spectrum(conv grid <- user grid)
  double px = 0.0;
  const double *ce = tab.conv_e;
  for (int j = tid; j < kN; j += kConvThreads) {
    const double elo0 = ce[j], ehi0 = ce[j + 1];
    float v = 0.0f;
    if (ue[0] <= ehi0 && ue[nu] >= elo0) {
      int imin = 0, imax = 0;
      {  // largest index with ue[m] <= elo0 (0 if none), capped at nu
        int lo = 0, hi = nu + 1;
        while (lo < hi) { int k = (lo + hi) >> 1; if (ue[k] <= elo0) lo = k + 1; else hi = k; }
        imin = lo > 0 ? lo - 1 : 0;
      }
      {  // largest index <= nu-1 with ue[m] <= ehi0 (0 if none)
        int lo = 0, hi = nu;
        while (lo < hi) { int k = (lo + hi) >> 1; if (ue[k] <= ehi0) lo = k + 1; else hi = k; }
        imax = lo > 0 ? lo - 1 : 0;
      }
      double elo = elo0 < ue[imin] ? ue[imin] : elo0;
      double ehi = ehi0 > ue[imax + 1] ? ue[imax + 1] : ehi0;
      if (imax == imin) {
        v = (float) ((ehi - elo) / (ue[imin + 1] - ue[imin]) * uf[imin]);
      } else {
        double dmin = (ue[imin + 1] - elo) / (ue[imin + 1] - ue[imin]);
        double dmax = (ehi - ue[imax]) / (ue[imax + 1] - ue[imax]);
        double acc = uf[imin] * dmin + uf[imax] * dmax;
        for (int q = imin + 1; q <= imax - 1; q++) acc += uf[q];
        v = (float) acc;
      }
    }
    if (j >= tab.conv_band_lo && j <= tab.conv_band_hi) px += (double) v;
    m.xs[skew(j)] = v * tab.conv_cf[j];
  }
  const double sr = block_sum_d<kConvThreads>(pr, m.red);
  const double sx = block_sum_d<kConvThreads>(px, m.red);
  conv_normalize_store(m, tab, wlo, whi, sx, sr, out);
}

// _rebin_spectrum for one output bin (relutility.c:549-601); ener0 has n0+1 edges
__device__ __forceinline__ double rebin_bin(double elo0, double ehi0, const double *__restrict__ e0, int n0,
                                           const float *__restrict__ f0) {
  if (!(e0[0] <= ehi0 && e0[n0] >= elo0)) return 0.0;
  int lo = 0, hi = n0 + 1;
  while (lo < hi) { int k = (lo + hi) >> 1; if (e0[k] <= elo0) lo = k + 1; else hi = k; }
  int imin = lo > 0 ? lo - 1 : 0;
  lo = 0;
  hi = n0;
  while (lo < hi) { int k = (lo + hi) >> 1; if (e0[k] <= ehi0) lo = k + 1; else hi = k; }
  int imax = lo > 0 ? lo - 1 : 0;
  const double elo = elo0 < e0[imin] ? e0[imin] : elo0;
  const double ehi = ehi0 > e0[imax + 1] ? e0[imax + 1] : ehi0;
  if (imax == imin) {
    float fr = (float) (ehi - elo) / (float) (e0[imin + 1] - e0[imin]);
    return (double) (fr * f0[imin]);
  }
  float dmin = (float) (e0[imin + 1] - elo) / (float) (e0[imin + 1] - e0[imin]);
  float dmax = (float) (ehi - e0[imax]) / (float) (e0[imax + 1] - e0[imax]);
  float acc = f0[imin] * dmin + f0[imax] * dmax;
  for (int q = imin + 1; q <= imax - 1; q++) acc += f0[q];
  return (double) acc;
}

struct FinSmem {
  float spec[kN];
  double red[kConvThreads / 32 + 1];
  float nrm;
};

// zone sum, primary continuum (PrimarySource.cpp:66-125), optional 3 keV
// renormalisation (Relxill.cpp:249-259) and rebin to the caller's grid
// (rebin_and_normalize_relxill_for_xspec, Relxill.cpp:267-278).
__global__ void __launch_bounds__(kConvThreads) finalize_relxill_kernel(RelxTables tab, const RelxSetIn *__restrict__ sin,
                                                                        const RelxSetState *__restrict__ sst,
                                                                        const float *__restrict__ cout, int nza,
                                                                        const double *__restrict__ user_e,
                                                                        double *__restrict__ flux) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FinSmem &m = *reinterpret_cast<FinSmem *>(smem_raw);
  const int set = blockIdx.x, tid = threadIdx.x;
  const RelxSetState &s = sst[set];
  const RelxSetIn &in = sin[set];
  const int nu = in.n_ener;
  double *fo = flux + in.e_off - set;  // flux offsets: e_off counts n+1 edges per set
  if (s.status != RELX_OK || s.model < RELX_RELXILL) {
    if (s.model != RELX_RELCONV || s.status != RELX_OK)
      for (int i = tid; i < nu; i += kConvThreads) fo[i] = 0.0;
    return;
  }
  const double *ce = tab.conv_e;
  const float gam = (float) s.gam;
  const float ecut = (float) (s.ect_src * s.g_inf);
  const float pnorm = (float) (s.src_norm * s.prim_fac);
  const float rfac = (float) s.norm_fac_refl;
  const bool add_prim = s.refl_frac >= 0;
  for (int k = tid; k < kN; k += kConvThreads) {
    float r = 0.0f;
    for (int z = 0; z < s.nz; z++) r += cout[((size_t) set * nza + z) * kN + k];
    r *= rfac;
    if (add_prim) {
      float en = (float) (0.5 * (ce[k] + ce[k + 1]));
      float pl = expf(1.0f / ecut) * powf(en, -gam) * expf(-en / ecut) * (float) (ce[k + 1] - ce[k]);
      r += pl * pnorm;
    }
    m.spec[k] = r;
  }
  __syncthreads();
  if (in.flags & 2) {  // RELXILL_RENORMALIZE: 1 cts/keV at 3 keV
    if (tid == 0) {
      int ind = bsearch_asc<double>(ce, kN, 3.0);
      m.nrm = (float) ((ce[ind + 1] - ce[ind]) / (double) m.spec[ind]);
    }
    __syncthreads();
    for (int k = tid; k < kN; k += kConvThreads) m.spec[k] *= m.nrm;
    __syncthreads();
  }
  const double *ue = user_e + in.e_off;
  const double zf = (s.z > 0) ? (1 + s.z) : 1.0;
  for (int i = tid; i < nu; i += kConvThreads) {
    double elo = ue[i], ehi = ue[i + 1];
    if (s.z > 0) { elo *= zf; ehi *= zf; }
    fo[i] = rebin_bin(elo, ehi, ce, kN, m.spec);
  }
}

// relconv: rebin the convolved spectrum back to the caller's grid, zero outside 0.01-1000 keV
__global__ void __launch_bounds__(kConvThreads) finalize_relconv_kernel(RelxTables tab, const RelxSetIn *__restrict__ sin,
                                                                        const RelxSetState *__restrict__ sst,
                                                                        const float *__restrict__ cout, int nza,
                                                                        const double *__restrict__ user_e,
                                                                        const int *__restrict__ sflag,
                                                                        double *__restrict__ flux) {
  const int set = blockIdx.x, tid = threadIdx.x;
  const RelxSetState &s = sst[set];
  const RelxSetIn &in = sin[set];
  if (s.model != RELX_RELCONV) return;
  const int nu = in.n_ener;
  double *fo = flux + in.e_off - set;
  if (s.status != RELX_OK || sflag[set] != RELX_OK) {
    for (int i = tid; i < nu; i += kConvThreads) fo[i] = 0.0;
    return;
  }
  const double *ue = user_e + in.e_off;
  const float *sp = cout + (size_t) set * nza * kN;
  for (int i = tid; i < nu; i += kConvThreads) {
    double v = rebin_bin(ue[i], ue[i + 1], tab.conv_e, kN, sp);
    if (ue[i + 1] < 0.01 || ue[i] > 1000.0) v = 0.0;  // Relbase.cpp:233-246
    fo[i] = v;
  }
}

// relline: profile on the caller's grid, normalised (Relprofile.cpp:749-781, LocalModel.cpp:43-45)
__global__ void __launch_bounds__(kConvThreads) finalize_relline_kernel(const RelxSetIn *__restrict__ sin,
                                                                        const RelxSetState *__restrict__ sst,
                                                                        const float *__restrict__ prof,
                                                                        const double *__restrict__ tsum, int ntile_max,
                                                                        int tile_bins, int nza, double *__restrict__ flux) {
  const int set = blockIdx.x, tid = threadIdx.x;
  const RelxSetState &s = sst[set];
  const RelxSetIn &in = sin[set];
  if (s.model != RELX_RELLINE) return;
  const int nu = in.n_ener;
  double *fo = flux + in.e_off - set;
  if (s.status != RELX_OK) {
    for (int i = tid; i < nu; i += kConvThreads) fo[i] = 0.0;
    return;
  }
  const double scale = profile_scale(s, tsum, set, ntile_max, nza, tile_bins);
  const float *p = prof + in.e_off;
  // bins outside the window hold 0; with an empty profile the reference's
  // renormalisation multiplies 0 by relline_norm/0 and returns NaN, as here
  for (int i = tid; i < nu; i += kConvThreads)
    fo[i] = ((i >= s.win_lo && i < s.win_hi) ? (double) p[i] : 0.0) * scale;
}

size_t conv_smem_bytes() { return sizeof(ConvSmem); }
size_t fin_smem_bytes() { return sizeof(FinSmem); }

}  // namespace relx
