// xillver_model.cu -- the non-relativistic reflection model xillver
// (xillver_model, LocalModel.cpp:103-128): the table spectrum interpolated in all
// five table parameters at the observer's inclination (interp_5d_tab,
// xilltable.c:878-995), times the semi-infinite slab factor 0.5 cos(incl)
// (Xillspec.cpp:528-545), rebinned onto the caller's grid shifted by the
// redshift (_rebin_spectrum, relutility.c:549-601), plus the primary continuum
// normalised as the table's (add_primary_component, Relbase.cpp:294-349).
//
// Launch: one CTA of 256 threads per parameter set.  Thread 0 brackets the five
// parameters and lists the corner rows with a non-zero weight (at most 32, in
// the order interp_5d_tab sums them); the CTA streams those rows, four energy
// bins per thread in float4 loads, and accumulates the weighted sum in FP32
// (all weights and spectra are non-negative, so the sum of at most 32 terms
// keeps about six significant digits).  The interpolated spectrum and the
// xillver grid (edges and widths) sit in shared memory for the rebin, which
// runs one caller bin per thread.  Bound: the table rows read, 32 rows of
// n_ener floats per set at most (fewer when a parameter sits on a grid value),
// shared with neighbouring sets through L2.
#include "relx_device.cuh"
#include "relx_kernels.h"

namespace relx {

constexpr int kXmodThreads = kXmodThreadsH;
constexpr int kXmodCorners = 64;  // 32 for a 5-parameter table, 64 for the 6-parameter one

// count of a[0..n) <= key (a ascending)
__device__ __forceinline__ int count_le_x(const float2 *a, int n, float key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid].x <= key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Corner c of interp_5d_tab's sum as a bit mask over the five table parameters (bit q: upper
// bracket of parameter q): within each group of eight, the first three parameters run through
// 000, 100, 010, 001, 110, 101, 011, 111.
__device__ __forceinline__ int corner_mask(int c) {
  const int lo3 = c & 7;
  const int perm = (lo3 == 3) ? 4 : (lo3 == 4) ? 3 : lo3;
  return (c & ~7) | perm;
}

// nthq, nth: xillverCp (the 6-parameter table and the nthcomp continuum); null for xillver
__global__ void __launch_bounds__(kXmodThreads) xillver_model_kernel(RelxTables tab, const RelxSetIn *__restrict__ sin,
                                                                      const double *__restrict__ user_e,
                                                                      RelxSetState *__restrict__ sst,
                                                                      double *__restrict__ flux,
                                                                      const double *__restrict__ nthq,
                                                                      const NthTable *__restrict__ nth) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n0 = tab.x_nener, pad = tab.x_nener_pad;
  float *spec = reinterpret_cast<float *>(smem_raw);                    // [pad]
  float2 *eb = reinterpret_cast<float2 *>(smem_raw + sizeof(float) * pad);  // [n0 + 1]
  __shared__ float w_s[kXmodCorners];
  __shared__ int row_s[kXmodCorners];
  __shared__ int ncor_s;
  __shared__ double qsum_s;
  const int set = blockIdx.x, tid = threadIdx.x;
  const RelxSetIn &in = sin[set];
  const double *v = in.p;
  // get_xill_params (ModelDefinition.cpp:339-388); the inclination stays in degrees.  xillver:
  // Gamma, A_Fe, Ecut, logxi, z, Incl, refl_frac; xillverCp: Gamma, A_Fe, kTe, logxi, logN, z, Incl,
  // refl_frac (lmodel_relxill_public.dat:77-94)
  const bool cp = nthq != nullptr;
  const double gam = v[0], afe = v[1], ect = v[2], lxi = v[3];
  const double dens = cp ? v[4] : 15.0;  // density of the xillver model (ModelDefinition.cpp:362)
  const double z = cp ? v[5] : v[4], incl = cp ? v[6] : v[5], refl_frac = cp ? v[7] : v[6];

  if (tid == 0) {
    // get_xilltab_indices_for_paramvals (xilltable.c:278-323) and the interpolation factors
    // (interp_xill_table, xilltable.c:1090-1181), the inclination reset to the table range too
    float inp[8];
    for (int q = 0; q < 8; q++) inp[q] = 0.0f;
    inp[0] = (float) gam;
    inp[1] = (float) afe;
    inp[2] = (float) lxi;
    inp[3] = (float) ect;
    inp[4] = (float) dens;
    inp[7] = (float) incl;
    const int np = tab.x_npar;
    int ind[6];
    double f[6];
    for (int q = 0; q < np; q++) {
      const float *pv = tab.x_vals + q * tab.x_maxvals;
      const int nv = tab.x_nvals[q], pi = tab.x_pindex[q];
      int k = bsearch_asc<float>(pv, nv, inp[pi]);
      if (k < 0) k = 0;
      else if (k > nv - 2) k = nv - 2;
      ind[q] = k;
      float val = inp[pi];
      if (val < pv[0]) val = pv[0];
      else if (val > pv[nv - 1]) val = pv[nv - 1];
      f[q] = (double) ((val - pv[k]) / (pv[k + 1] - pv[k]));
      if (pi == 3) {  // ensure_ecut_within_boundarys (xilltable.c:1054-1067)
        if (ect <= pv[0]) f[q] = 0.0;
        if (ect >= pv[nv - 1]) f[q] = 1.0;
      }
    }
    // 6 parameters: the 32 corners over parameters 1..5 at both brackets of parameter 0, linear in
    // parameter 0 (interp_6d_tab, xilltable.c:1022-1043)
    const int q0 = np - 5;
    int nc = 0;
    for (int c = 0; c < (32 << q0); c++) {
      const int msk = corner_mask(c & 31), half = c >> 5;
      double w = (q0 == 0) ? 1.0 : (half ? f[0] : 1.0 - f[0]);
      int64_t row = (q0 == 0) ? 0 : ind[0] + half;
      for (int q = 0; q < 5; q++) {
        const int up = (msk >> q) & 1;
        w *= up ? f[q0 + q] : (1.0 - f[q0 + q]);
        row = row * tab.x_nvals[q0 + q] + ind[q0 + q] + up;  // incl is the fastest table index
      }
      if (w != 0.0) {  // a zero weight adds exactly nothing
        w_s[nc] = (float) w;
        row_s[nc] = (int) row;
        nc++;
      }
    }
    ncor_s = nc;
  }
  for (int k = tid; k <= n0; k += kXmodThreads) eb[k] = tab.x_ew[k];
  __syncthreads();

  // the interpolated spectrum times the slab factor
  {
    const int nc = ncor_s;
    const float nf = (float) (0.5 * cos(incl * kPi / 180));
    const int n4 = pad >> 2;
    for (int i4 = tid; i4 < n4; i4 += kXmodThreads) {
      float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      for (int c = 0; c < nc; c++) {
        const float4 x = __ldg(reinterpret_cast<const float4 *>(tab.x_spec + (size_t) row_s[c] * pad) + i4);
        const float w = w_s[c];
        a.x = fmaf(w, x.x, a.x);
        a.y = fmaf(w, x.y, a.y);
        a.z = fmaf(w, x.z, a.z);
        a.w = fmaf(w, x.w, a.w);
      }
      reinterpret_cast<float4 *>(spec)[i4] = make_float4(a.x * nf, a.y * nf, a.z * nf, a.w * nf);
    }
  }
  // normalisation of the primary continuum (calc_normalized_primary_spectrum, Xillspec.cpp:302-332);
  // for the nthcomp continuum from nthcomp_kernel, with the E F_E normalisation at 1 keV
  __shared__ double nth_norm_s;
  if (cp) {
    if (tid == 0) {
      qsum_s = nthq[(size_t) set * (RELX_NZMAX + 1)];
      nth_norm_s = nth[set].n > 0 ? nth_normfac(tab.nth_grid->x, nth[set].sp, nth[set].n, 1.0) : 0.0;
    }
  } else if (tid < 32) {
    const double q = primary_qsum_warp(tab, (float) gam, (float) ect, nullptr);
    if (tid == 0) qsum_s = q;
  }
  __syncthreads();

  // xillverCp: kTe without an nthcomp grid gives no spectrum (nthcomp_kernel)
  const bool ok = !cp || (isfinite(qsum_s) && qsum_s > 0.0 && nth[set].n > 0);
  const int nu = in.n_ener;
  const double *ue = user_e + in.e_off;
  double *fo = flux + in.e_off - set;  // flux offsets: e_off counts n+1 edges per set
  const double zf = (z > 0) ? 1.0 + z : 1.0;  // shift_energy_grid_redshift (XspecSpectrum.h:70-76)
  const double arf = fabs(refl_frac);
  const bool add_prim = refl_frac >= 0;
  const float fg = (float) gam, fe = (float) ect;
  const float e1 = expf(1.0f / fe);
  const float pnorm = (float) (1.0 / qsum_s);
  const double e_first = (double) eb[0].x, e_last = (double) eb[n0].x;
  for (int i = tid; i < nu; i += kXmodThreads) {
    if (!ok) {
      fo[i] = 0.0;
      continue;
    }
    double elo = ue[i], ehi = ue[i + 1];
    if (z > 0) { elo *= zf; ehi *= zf; }
    double r = 0.0;  // a coarse caller bin sums many table bins: FP64 accumulation
    if (e_first <= ehi && e_last >= elo) {
      // the indices of the reference's walk: imin = #(edges <= elo) - 1 over all n0 + 1 edges,
      // imax = #(edges <= ehi) - 1 over the first n0; the edges are floats, so comparing with the
      // energy rounded down to a float decides exactly
      int imin = count_le_x(eb, n0 + 1, __double2float_rd(elo)) - 1;
      int imax = count_le_x(eb, n0, __double2float_rd(ehi)) - 1;
      imin = max(0, min(imin, n0 - 1));
      imax = max(0, imax);
      const double el = elo < (double) eb[imin].x ? (double) eb[imin].x : elo;
      const double eh = ehi > (double) eb[imax + 1].x ? (double) eb[imax + 1].x : ehi;
      if (imax == imin) {
        r = (double) ((float) (eh - el) / eb[imin].y * spec[imin]);
      } else {
        const float dmin = (float) ((double) eb[imin + 1].x - el) / eb[imin].y;
        const float dmax = (float) (eh - (double) eb[imax].x) / eb[imax].y;
        r = (double) (spec[imin] * dmin + spec[imax] * dmax);
        for (int q = imin + 1; q <= imax - 1; q++) r += (double) spec[q];
      }
    }
    r *= arf;
    if (add_prim && cp) {  // nthcomp on the shifted grid (spec_nthcomp with no energy shift)
      r += nth_bin(tab.nth_grid->x, nth[set], elo, ehi, 1.0, nth_norm_s) * (1.0 / qsum_s);
    } else if (add_prim) {  // spec_cutoffpl on the shifted grid (Xillspec.cpp:215-233), FP32 arithmetic
      const float en = (float) (0.5 * (elo + ehi));
      r += (double) (e1 * powf(en, -fg) * expf(-en / fe) * (float) (ehi - elo) * pnorm);
    }
    fo[i] = r;
  }
  if (tid == 0) {  // the fields the status pass and the statistics read
    RelxSetState &s = sst[set];
    s.status = ok ? RELX_OK : RELX_ERR_PARAM;
    s.model = RELX_XILLVER;
    s.pmodel = cp ? RELX_XILLVERCP : RELX_XILLVER;
    s.prim = cp ? 1 : 0;
    s.cached = 0;
    s.nz = 0;
    s.ucount = 0;
    s.win_lo = s.win_hi = 0;
  }
}

size_t xillver_model_smem_bytes(int n_ener, int n_ener_pad) {
  return sizeof(float) * (size_t) n_ener_pad + sizeof(float2) * (size_t) (n_ener + 1);
}

cudaError_t xillver_model_set_smem(int n_ener, int n_ener_pad) {
  return cudaFuncSetAttribute(xillver_model_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int) xillver_model_smem_bytes(n_ener, n_ener_pad));
}

cudaError_t launch_xillver_model(cudaStream_t s, const RelxTables &tab, int n_sets, const RelxSetIn *sin,
                                 const double *user_e, RelxSetState *sst, double *flux, const double *nthq,
                                 const NthTable *nth) {
  if (n_sets <= 0) return cudaSuccess;
  xillver_model_kernel<<<n_sets, kXmodThreads, xillver_model_smem_bytes(tab.x_nener, tab.x_nener_pad), s>>>(
      tab, sin, user_e, sst, flux, nthq, nth);
  return cudaGetLastError();
}

}  // namespace relx
