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
#include "relx_tma.cuh"

namespace relx {

constexpr int kConvThreads = 256;  // convolution kernels
constexpr int kFinThreads = 128;   // finalize kernels
constexpr int kConvR = 16;         // output bins per thread and work item
constexpr int kConvD = 16;         // window bins per step of the register tile
constexpr int kN = RELX_NCONV;
constexpr int kPre = 4;            // prefix sums are kept at every kPre-th bin
constexpr int kXStage = 3072;      // xillver bins staged in shared memory (larger tables read global memory)
constexpr int kTsumStage = 256;    // (tile, zone) profile sums staged in shared memory at once        // conv bins per thread whose rebin map entries are loaded together
static_assert(kN % (kConvThreads * kPre) == 0, "scan tiling");

// xs is stored in rows of 16 bins, each followed by 4 padding floats: the 16-byte loads of the
// threads of a quarter warp (16 bins apart) then fall in distinct banks
__device__ __forceinline__ int skew(int m) { return m + ((m >> 4) << 2); }

struct ConvSmem {
  alignas(16) float xs[kN + kN / 4];  // x * cf, skewed
  float hr[kN + kConvR];       // rel * cf over the zone's profile window, zero padded (16-byte aligned)
  float2 red[kConvThreads / 32 + 2];
  float2 wsum[kConvThreads / 32];
  double dred[kConvThreads / 32 + 2];
  double zsum[RELX_NZMAX];
  double tz[kTsumStage];       // the set's per-(tile, zone) profile sums
  float bc[2];                 // broadcast scalars
  float2 sxw;                  // band sum of xs
  int abort_flag;
  uint64_t bar;                // completion of the bulk copy of the zone's xillver spectrum
  union {                      // the staged spectrum is read before the prefix sums are formed
    alignas(16) float xz[kXStage];  // the zone's xillver spectrum (bulk copy)
    float2 pre[kN / kPre + 1];   // float-float prefix sums of xs at bins 0, kPre, 2 kPre, ...
  };
};
static_assert(offsetof(ConvSmem, hr) % 16 == 0, "the profile window is read as float4");

// y[k0 + r] = sum_{i in [clo, chi)} hr[i - wlo] * xs[(k0 + r + p - i) mod N]; hr is zero padded
// past the window, so chi - clo need not be a multiple of kConvD.  Register tile: kConvR outputs x
// kConvD window bins per step, (kConvR + kConvD) / 4 float4 loads of xs and kConvD/4 float4 loads
// of hr for kConvR * kConvD FMAs.  k0 + p - clo must be a multiple of 4 (the xs loads are aligned).
__device__ __forceinline__ void conv_tile(const ConvSmem &m, int k0, int p, int wlo, int clo, int chi,
                                          float y[kConvR]) {
#pragma unroll
  for (int r = 0; r < kConvR; r++) y[r] = 0.0f;
  for (int i0 = clo; i0 < chi; i0 += kConvD) {
    const int base = k0 + p - i0 - (kConvD - 1) - 1;  // one bin lower: a multiple of 4
    float xr[kConvR + kConvD];
#pragma unroll
    for (int c4 = 0; c4 < (kConvR + kConvD) / 4; c4++) {
      const float4 v = *reinterpret_cast<const float4 *>(&m.xs[skew((base + 4 * c4) & (kN - 1))]);
      xr[4 * c4] = v.x;
      xr[4 * c4 + 1] = v.y;
      xr[4 * c4 + 2] = v.z;
      xr[4 * c4 + 3] = v.w;
    }
    const float4 *h4 = reinterpret_cast<const float4 *>(&m.hr[i0 - wlo]);
#pragma unroll
    for (int d4 = 0; d4 < kConvD / 4; d4++) {
      const float4 hv = h4[d4];
      const float hs[4] = {hv.x, hv.y, hv.z, hv.w};
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int d = d4 * 4 + e;
#pragma unroll
        for (int r = 0; r < kConvR; r++) y[r] = fmaf(hs[e], xr[r - d + kConvD], y[r]);
      }
    }
  }
}

// relline renormalisation factor (renorm_relline_profile, Relprofile.cpp:766-781) and the zone
// sums of the profile, from the per-(tile, zone) sums of the line kernel.  Warp 0: one lane per
// zone sums its tiles in order, lane 0 sums the zones in order.  Results in m.zsum (scaled) and
// m.bc[0] (scale).
__device__ void profile_sums(ConvSmem &m, const RelxSetState &s, const double *tsum, int set, int ntile_max, int nza,
                             int tile_bins) {
  const int tid = threadIdx.x;
  const int ntiles = (s.win_hi - s.win_lo + tile_bins - 1) / tile_bins;
  const bool staged = ntiles * s.nz <= kTsumStage;
  if (staged) {  // every (tile, zone) sum loaded at once
    for (int q = tid; q < ntiles * s.nz; q += kConvThreads) {
      const int t = q / s.nz, z = q - t * s.nz;
      m.tz[q] = tsum[((size_t) set * ntile_max + t) * nza + z];
    }
    __syncthreads();
  }
  if (tid < 32) {
    for (int z = tid; z < s.nz; z += 32) {
      double zs = 0.0;
      for (int t = 0; t < ntiles; t++) zs += staged ? m.tz[t * s.nz + z] : tsum[((size_t) set * ntile_max + t) * nza + z];
      m.zsum[z] = zs;
    }
    if (s.relline_norm > 0.0) {  // renormalised profile: the zones' total in zone order, then each zone scaled
      __syncwarp();
      double scale = 0.0;
      if (tid == 0) {
        double sum = 0.0;
        for (int z = 0; z < s.nz; z++) sum += m.zsum[z];
        scale = s.relline_norm / sum;
        m.bc[0] = (float) scale;
      }
      scale = __shfl_sync(0xffffffffu, scale, 0);
      for (int z = tid; z < s.nz; z += 32) m.zsum[z] *= scale;
    } else if (tid == 0) {
      m.bc[0] = 1.0f;
    }
  }
  __syncthreads();
}

// float-float prefix of xs at bin x (0 <= x <= N)
__device__ __forceinline__ float2 prefix_at(const ConvSmem &m, int x) {
  const int q = x / kPre;
  float2 v = m.pre[q];
  for (int j = q * kPre; j < x; j++) v = ff_addf(v, m.xs[skew(j)]);
  return v;
}

// cost of a split of the window into S segments: rounds of work items times segment length
__device__ __forceinline__ int split_cost(int nt, int nc, int S) {
  return ((nt * S + kConvThreads - 1) / kConvThreads) * ((nc + S - 1) / S);
}

// Convolution of xs with hr, normalised as calcFFTNormFactor (Relbase.cpp:199-222), written for the
// conv bins [olo, ohi] the caller's grid needs.  The 0.01-1000 keV sum of the convolution is
// sum_i hr_i * (window sum of xs) / cf, from prefix sums of xs, and the band sum of the xillver
// spectrum is the band's window sum of xs / cf (cf = E/dE is the same in every bin of the log grid
// up to rounding, and cancels), so bins outside [olo, ohi] are never convolved.  The sums are
// float-float (about 48 significant bits, on the FP32 pipe).
__device__ void conv_normalize_store(ConvSmem &m, const RelxTables &tab, int wlo, int whi, int olo, int ohi,
                                     float2 sr, float *out) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  // prefix sums of xs at every kPre-th bin
  {
    constexpr int per = kN / kConvThreads;
    float2 grp[per / kPre];
    float2 loc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int g = 0; g < per / kPre; g++) {
      float2 gs = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int q = 0; q < kPre; q++) gs = ff_addf(gs, m.xs[skew(tid * per + g * kPre + q)]);
      grp[g] = gs;
      loc = ff_add(loc, gs);
    }
    float2 inc = loc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      float2 t;
      t.x = __shfl_up_sync(0xffffffffu, inc.x, o);
      t.y = __shfl_up_sync(0xffffffffu, inc.y, o);
      if (lane >= o) inc = ff_add(t, inc);
    }
    float2 exc;
    exc.x = __shfl_up_sync(0xffffffffu, inc.x, 1);
    exc.y = __shfl_up_sync(0xffffffffu, inc.y, 1);
    if (lane == 0) exc = make_float2(0.0f, 0.0f);
    if (lane == 31) m.wsum[w] = inc;
    __syncthreads();
    float2 run = make_float2(0.0f, 0.0f);
    for (int q = 0; q < w; q++) run = ff_add(run, m.wsum[q]);
    run = ff_add(run, exc);
#pragma unroll
    for (int g = 0; g < per / kPre; g++) {
      m.pre[(tid * per) / kPre + g] = run;
      run = ff_add(run, grp[g]);
    }
    if (tid == kConvThreads - 1) m.pre[kN / kPre] = run;
    __syncthreads();
  }
  const int p = tab.conv_pos1;
  const int blo = tab.conv_band_lo, L = tab.conv_band_hi - tab.conv_band_lo + 1;
  if (tid == 32) m.sxw = ff_add(prefix_at(m, blo + L), ff_neg(prefix_at(m, blo)));  // band sum of xs
  float2 part = make_float2(0.0f, 0.0f);
  for (int i = wlo + tid; i < whi; i += kConvThreads) {
    const int a = (blo + p - i) & (kN - 1);
    float2 ws;
    if (a + L <= kN) ws = ff_add(prefix_at(m, a + L), ff_neg(prefix_at(m, a)));
    else ws = ff_add(ff_add(m.pre[kN / kPre], ff_neg(prefix_at(m, a))), prefix_at(m, a + L - kN));
    part = ff_add(part, ff_mulf(ws, m.hr[i - wlo]));
  }
  const float2 scf = block_sum_ff<kConvThreads>(part, m.red);
  if (tid == 0) m.bc[1] = ff_div_to_float(ff_mul(sr, m.sxw), scf);  // the barrier of block_sum_ff orders m.sxw
  __syncthreads();
  const float norm = m.bc[1];
  if (olo > ohi) return;
  const int olo_out = olo;
  olo -= (olo + p - wlo) & 3;  // tiles start where the xs loads of conv_tile are 16-byte aligned
  // work items: (16-bin output tile, window segment).  The window is split into S (a power of two)
  // segments so that narrow output ranges still occupy every thread; the S partials of a tile sit
  // in adjacent lanes and are added by a fixed shuffle tree, so the result depends only on this
  // set's own sizes.
  const int nt = (ohi - olo + 1 + kConvR - 1) / kConvR;
  const int nc = (whi - wlo + kConvD - 1) / kConvD;
  int S = 1, best = split_cost(nt, nc, 1);
  for (int c = 2; c <= 32 && c <= nc; c <<= 1) {
    const int cost = split_cost(nt, nc, c);
    if (cost < best) { best = cost; S = c; }
  }
  const int seg = ((nc + S - 1) / S) * kConvD;  // window bins per segment
  const int nitems = nt * S;
  for (int q0 = 0; q0 < nitems; q0 += kConvThreads) {
    const int q = q0 + tid;
    const int t = q / S, sg = q % S;
    float y[kConvR];
    if (q < nitems) {
      const int clo = wlo + sg * seg, chi = min(whi, clo + seg);
      conv_tile(m, olo + t * kConvR, p, wlo, clo, chi, y);
    } else {
#pragma unroll
      for (int r = 0; r < kConvR; r++) y[r] = 0.0f;
    }
    for (int o = S >> 1; o > 0; o >>= 1) {
#pragma unroll
      for (int r = 0; r < kConvR; r++) y[r] += __shfl_xor_sync(0xffffffffu, y[r], o);
    }
    if (q < nitems && sg == 0) {
#pragma unroll
      for (int r = 0; r < kConvR; r++) {
        const int k = olo + t * kConvR + r;
        if (k >= olo_out && k <= ohi) out[k] = y[r] * __frcp_rn(tab.conv_cf[k]) * norm;
      }
    }
  }
}

__global__ void __launch_bounds__(kConvThreads) conv_zone_kernel(RelxTables tab, const RelxSetState *__restrict__ sst,
                                                                 const float *__restrict__ prof,
                                                                 const double *__restrict__ tsum, int ntile_max,
                                                                 int tile_bins, const float *__restrict__ xill, int nza,
                                                                 float *__restrict__ cout, int *__restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ConvSmem &m = *reinterpret_cast<ConvSmem *>(smem_raw);
  const int z = blockIdx.x, set = blockIdx.y, tid = threadIdx.x;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.model < RELX_RELXILL || z >= s.nz) return;
  float *out = cout + ((size_t) set * nza + z) * kN;
  profile_sums(m, s, tsum, set, ntile_max, nza, tile_bins);
  // relxill_convolution_multizone skips zones without flux (Relxill.cpp:455-457)
  if (m.zsum[z] < 1e-12) {
    for (int k = s.out_lo + tid; k <= s.out_hi; k += kConvThreads) out[k] = 0.0f;
    return;
  }
  const int wlo = s.zw_lo[z], whi = s.zw_hi[z];  // the zone's profile is zero outside
  const float fscale = m.bc[0];
  const float *pz = prof + ((size_t) set * nza + z) * kN;
  // the zone's xillver spectrum on the conv grid (x E/dE): one bulk copy into shared memory,
  // overlapped with the profile loads
  const float *xz = xill + ((size_t) set * nza + z) * tab.x_cpad;
  // bulk copies need 16-byte aligned rows of a 16-byte multiple (rows are padded to 4 floats)
  const bool staged = tab.x_cpad <= kXStage && (tab.x_cpad & 3) == 0 && (((uintptr_t) xz) & 15) == 0;
  if (staged && tid == 0) {
    m.abort_flag = 0;
    mbar_init(&m.bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_expect_tx(&m.bar, (uint32_t) tab.x_cpad * 4u);
    bulk_g2s(m.xz, xz, (uint32_t) tab.x_cpad * 4u, &m.bar);
  }
  // relline profile weighted by E/dE over its window; band sum of the profile
  float2 pr = make_float2(0.0f, 0.0f);
  for (int i = tid; i < whi - wlo + kConvR; i += kConvThreads) {
    const int j = wlo + i;
    float v = 0.0f;
    if (j < whi) {
      const float fr = pz[j] * fscale;
      v = fr * tab.conv_cf[j];
      if (j >= tab.conv_band_lo && j <= tab.conv_band_hi) pr = ff_addf(pr, fr);
    }
    m.hr[i] = v;
  }
  if (staged) {
    __syncthreads();  // the barrier is initialised
    if (!mbar_wait_bounded(&m.bar, 0)) atomicExch(&m.abort_flag, 1);
    __syncthreads();
    if (m.abort_flag) {
      if (tid == 0) {
        (void) mbar_wait_bounded(&m.bar, 0);  // give the copy in flight another bounded wait
        atomicExch(err, RELX_ERR_TIMEOUT);
      }
      return;
    }
  }
  const float *xs_src = staged ? m.xz : xz;
  // the zone's spectrum, already rebinned onto the conv grid and weighted by E/dE (the table rows
  // are, and the zone spectrum is linear in them): bins outside the table's reach are zero
  const int clo = tab.x_clo, cn = tab.x_cn;
  for (int j = tid; j < kN; j += kConvThreads) {
    const int q = j - clo;
    m.xs[skew(j)] = (q >= 0 && q < cn) ? xs_src[q] : 0.0f;
  }
  const float2 sr = block_sum_ff<kConvThreads>(pr, m.red);
  conv_normalize_store(m, tab, wlo, whi, s.out_lo, s.out_hi, sr, out);
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
  const double usum = block_sum_d<kConvThreads>(ps, m.dred);
  if (!(usum > 0.0)) {
    if (tid == 0) sflag[set] = RELX_ERR_INPUT;
    return;
  }
  profile_sums(m, s, tsum, set, ntile_max, nza, tile_bins);
  const int wlo = s.win_lo, whi = s.win_hi;
  const float fscale = m.bc[0];
  const float *pz = prof + (size_t) set * nza * kN;
  float2 pr = make_float2(0.0f, 0.0f);
  for (int i = tid; i < whi - wlo + kConvR; i += kConvThreads) {
    const int j = wlo + i;
    float v = 0.0f;
    if (j < whi) {
      const float fr = pz[j] * fscale;
      v = fr * tab.conv_cf[j];
      if (j >= tab.conv_band_lo && j <= tab.conv_band_hi) pr = ff_addf(pr, fr);
    }
    m.hr[i] = v;
  }
  // _rebin_spectrum(conv grid <- user grid)
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
    m.xs[skew(j)] = v * tab.conv_cf[j];
  }
  const float2 sr = block_sum_ff<kConvThreads>(pr, m.red);
  conv_normalize_store(m, tab, wlo, whi, s.out_lo, s.out_hi, sr, out);
}

// _rebin_spectrum (relutility.c:549-601) of one output bin from the conv grid; the bin indices
// are those of the reference's walk, found from the logarithm and exact comparisons
__device__ __forceinline__ double rebin_bin(const RelxTables &tab, double elo0, double ehi0,
                                           const float *__restrict__ f0) {
  // energies are positive: comparisons of their bit patterns and conversions on the integer pipes
  // (d2f, f2d); the FP64 pipe keeps the three differences of edges
  constexpr int n0 = kN;
  const double *e0 = tab.conv_e;
  if (!(dge(ehi0, e0[0]) && dge(e0[n0], elo0))) return 0.0;
  const int imin = conv_index(tab, elo0);
  const int imax = conv_index(tab, ehi0);
  const double elo = dgt(e0[imin], elo0) ? e0[imin] : elo0;
  const double ehi = dgt(ehi0, e0[imax + 1]) ? e0[imax + 1] : ehi0;
  // bin widths of the conv grid as floats, (float) (e0[k + 1] - e0[k])
  if (imax == imin) {
    float fr = d2f(ehi - elo) / tab.conv_cw[imin].y;
    return f2d(fr * f0[imin]);
  }
  float dmin = d2f(e0[imin + 1] - elo) / tab.conv_cw[imin].y;
  float dmax = d2f(ehi - e0[imax]) / tab.conv_cw[imax].y;
  float acc = f0[imin] * dmin + f0[imax] * dmax;
  for (int q = imin + 1; q <= imax - 1; q++) acc += f0[q];
  return f2d(acc);
}

struct FinSmem {
  float spec[kN];
  double red[kFinThreads / 32 + 1];
  float nrm;
  double nth_norm;  // nthcomp: 1 / (E F_E at the shifted 1 keV point)
};

// zone sum, primary continuum (PrimarySource.cpp:66-125), optional 3 keV
// renormalisation (Relxill.cpp:249-259) and rebin to the caller's grid
// (rebin_and_normalize_relxill_for_xspec, Relxill.cpp:267-278).
template <int NT>
__global__ void __launch_bounds__(NT) finalize_relxill_kernel(RelxTables tab, const RelxSetIn *__restrict__ sin,
                                                                        const RelxSetState *__restrict__ sst,
                                                                        const float *__restrict__ cout, int nza,
                                                                        const double *__restrict__ user_e,
                                                                        double *__restrict__ flux,
                                                                        const NthTable *__restrict__ nth) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FinSmem &m = *reinterpret_cast<FinSmem *>(smem_raw);
  const int set = blockIdx.x, tid = threadIdx.x;
  const RelxSetState &s = sst[set];
  const RelxSetIn &in = sin[set];
  const int nu = in.n_ener;
  double *fo = flux + in.e_off - set;  // flux offsets: e_off counts n+1 edges per set
  if (s.status != RELX_OK || s.model < RELX_RELXILL) {
    if (s.model != RELX_RELCONV || s.status != RELX_OK)
      for (int i = tid; i < nu; i += NT) fo[i] = 0.0;
    return;
  }
  const double *ce = tab.conv_e;
  const float gam = (float) s.gam;
  const float ecut = (float) (s.ect_src * s.g_inf);
  const float pnorm = (float) (s.src_norm * s.prim_fac);
  const float rfac = (float) s.norm_fac_refl;
  const bool add_prim = s.refl_frac >= 0;
  // nthcomp primary (the Cp models): the source's E F_E table in the frame shifted by g_inf,
  // z = 1 / g_inf - 1 (spec_nthcomp, Xillspec.cpp:243-253)
  const bool cp = s.prim == 1;
  const double zp1 = (1.0 / s.g_inf - 1.0) + 1.0;
  if (cp && add_prim) {
    if (tid == 0) m.nth_norm = nth_normfac(tab.nth_grid->x, nth[set].sp, nth[set].n, zp1);
    __syncthreads();
  }
  for (int k = s.out_lo + tid; k <= s.out_hi; k += NT) {
    float r = 0.0f;
    for (int z = 0; z < s.nz; z++) r += cout[((size_t) set * nza + z) * kN + k];
    r *= rfac;
    if (add_prim && cp) {  // FP32: the bin's photon flux as the trapezoid of E F_E / E^2 (donthcomp.c:788-792)
      const float e0 = tab.conv_eff[k].x, e1 = tab.conv_eff[k + 1].x, zf1 = (float) zp1;
      const float p0 = nth_prim_f(*tab.nth_grid, nth[set], e0 * zf1);
      const float p1 = nth_prim_f(*tab.nth_grid, nth[set], e1 * zf1);
      r += (p1 / (e1 * e1) + p0 / (e0 * e0)) * 0.5f * tab.conv_cw[k].y * ((float) m.nth_norm * pnorm);
    } else if (add_prim) {
      const float2 cd = tab.conv_cw[k];  // (float) bin centre, (float) bin width
      const float en = cd.x;
      float pl = expf(1.0f / ecut) * powf(en, -gam) * expf(-en / ecut) * cd.y;
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
    for (int k = s.out_lo + tid; k <= s.out_hi; k += NT) m.spec[k] *= m.nrm;
    __syncthreads();
  }
  const double *ue = user_e + in.e_off;
  const double zf = (s.z > 0) ? (1 + s.z) : 1.0;
  for (int i = tid; i < nu; i += NT) {
    double elo = ue[i], ehi = ue[i + 1];
    if (s.z > 0) { elo *= zf; ehi *= zf; }
    fo[i] = rebin_bin(tab, elo, ehi, m.spec);
  }
}

// relconv: rebin the convolved spectrum back to the caller's grid, zero outside 0.01-1000 keV
__global__ void __launch_bounds__(kFinThreads) finalize_relconv_kernel(RelxTables tab, const RelxSetIn *__restrict__ sin,
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
    for (int i = tid; i < nu; i += kFinThreads) fo[i] = 0.0;
    return;
  }
  const double *ue = user_e + in.e_off;
  const float *sp = cout + (size_t) set * nza * kN;
  for (int i = tid; i < nu; i += kFinThreads) {
    double v = rebin_bin(tab, ue[i], ue[i + 1], sp);
    if (ue[i + 1] < 0.01 || ue[i] > 1000.0) v = 0.0;  // Relbase.cpp:233-246
    fo[i] = v;
  }
}

// relline: profile on the caller's grid, normalised (Relprofile.cpp:749-781, LocalModel.cpp:43-45)
__global__ void __launch_bounds__(kFinThreads) finalize_relline_kernel(const RelxSetIn *__restrict__ sin,
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
    for (int i = tid; i < nu; i += kFinThreads) fo[i] = 0.0;
    return;
  }
  __shared__ double scale_sh;
  if (tid == 0) {
    // renorm_relline_profile (Relprofile.cpp:766-781): zones in order, tiles in order within a zone
    double scale = 1.0;
    if (s.relline_norm > 0.0) {
      const int ntiles = (s.win_hi - s.win_lo + tile_bins - 1) / tile_bins;
      double sum = 0.0;
      for (int z = 0; z < s.nz; z++) {
        double zs = 0.0;
        for (int t = 0; t < ntiles; t++) zs += tsum[((size_t) set * ntile_max + t) * nza + z];
        sum += zs;
      }
      scale = s.relline_norm / sum;
    }
    scale_sh = scale;
  }
  __syncthreads();
  const double scale = scale_sh;
  const float *p = prof + in.e_off;
  // bins outside the window hold 0; with an empty profile the reference's
  // renormalisation multiplies 0 by relline_norm/0 and returns NaN, as here
  for (int i = tid; i < nu; i += kFinThreads)
    fo[i] = ((i >= s.win_lo && i < s.win_hi) ? (double) p[i] : 0.0) * scale;
}

size_t conv_smem_bytes() { return sizeof(ConvSmem); }
size_t fin_smem_bytes() { return sizeof(FinSmem); }

// wide: 512 threads per set (few sets: one set's bins spread over more threads); otherwise 128.
// Every output is computed by one thread with the same arithmetic, so both give the same numbers.
cudaError_t launch_finalize_relxill(cudaStream_t s, bool wide, int n_sets, const RelxTables &tab,
                                    const RelxSetIn *sin, const RelxSetState *sst, const float *cout, int nza,
                                    const double *user_e, double *flux, const NthTable *nth) {
  if (n_sets <= 0) return cudaSuccess;
  if (wide)
    finalize_relxill_kernel<512><<<n_sets, 512, sizeof(FinSmem), s>>>(tab, sin, sst, cout, nza, user_e, flux, nth);
  else
    finalize_relxill_kernel<kFinThreads><<<n_sets, kFinThreads, sizeof(FinSmem), s>>>(tab, sin, sst, cout, nza, user_e,
                                                                                     flux, nth);
  return cudaGetLastError();
}

}  // namespace relx
