// table_ingest.cu -- the xillver table's SPECTRA rows decoded on the GPU.
//
// The reference reads one corner spectrum at a time with cfitsio on first use
// (check_xilltab_cache, xilltable.c:575-635) and divides it by 10^logXi of its
// grid point (renorm_xill_spec, xilltable.c:478-485).  Here the whole table is
// streamed once: the host reads raw FITS rows in large chunks into pinned
// memory, the chunk is copied to the device, and one CTA per row
//  * decodes the big-endian floats of the spectrum column,
//  * divides them by 10^logXi of the row and, for a table with a density
//    parameter, then by 10^(logN - 15) (the divisors are computed on the host
//    per grid value, so each quotient is the correctly rounded one the host
//    would store),
//  * writes the row padded to a multiple of four floats,
//  * integrates the row for the returning-radiation correction factors
//    (energy flux in 0.1-1000 keV, photon flux in 0.15-500 keV, and that
//    photon flux after the rebin of the spectrum shifted by g = 2/3, a fixed
//    linear map with coefficients pfz_coef; Xillspec.cpp:132-160, 457-495),
//  * and counts values that are not finite (table validation).
// A second kernel averages the row integrals over the inclinations of each
// corner with the reference's inclination weights.  A third writes every row
// rebinned onto the conv grid (_rebin_spectrum, relutility.c:549-601, in FP64)
// and weighted by E/dE of the conv bin, the form the convolution reads: the
// interpolation of the zone spectra and the weighting are linear, so the
// zones' spectra then arrive on the conv grid directly.
#include "relx_device.cuh"
#include "relx_kernels.h"

namespace relx {

constexpr int kIngestThreads = 256;

__device__ __forceinline__ float be_to_float(uint32_t w) { return __uint_as_float(__byte_perm(w, 0, 0x0123)); }

__global__ void __launch_bounds__(kIngestThreads) xill_ingest_kernel(
    const unsigned char *__restrict__ raw, int64_t width, int64_t col_off, int ne, int pad, int64_t row0,
    const double *__restrict__ lxi_div, int64_t stride_lxi, int n_lxi, const double *__restrict__ dns_div,
    int64_t stride_dns, int n_dns, const double *__restrict__ xe,
    const double *__restrict__ pfz_coef, float *__restrict__ spec, double *__restrict__ rowflux,
    unsigned long long *__restrict__ bad) {
  __shared__ double red[3][kIngestThreads / 32];
  const int r = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t row = row0 + r;
  const double div = n_lxi > 0 ? lxi_div[(row / stride_lxi) % n_lxi] : 1.0;
  const double div2 = n_dns > 0 ? dns_div[(row / stride_dns) % n_dns] : 1.0;
  const uint32_t *src = reinterpret_cast<const uint32_t *>(raw + (size_t) r * width + col_off);
  float *dst = spec + (size_t) row * pad;
  double ef = 0.0, pf = 0.0, pfz = 0.0;
  int nbad = 0;
  for (int e = tid; e < pad; e += kIngestThreads) {
    float v = 0.0f;
    if (e < ne) {
      v = (float) ((double) be_to_float(__ldg(src + e)) / div);  // float / double, stored as float
      v = (float) ((double) v / div2);                           // (xilltable.c:478-485, two steps)
      if (!isfinite(v)) nbad++;
      const double lo = xe[e], hi = xe[e + 1];
      if (lo >= 0.1 && hi <= 1000) ef += (double) v * 0.5 * (lo + hi);
      if (lo >= 0.15 && hi <= 500.0) pf += (double) v;
      pfz += pfz_coef[e] * (double) v;
    }
    dst[e] = v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ef += __shfl_xor_sync(0xffffffffu, ef, o);
    pf += __shfl_xor_sync(0xffffffffu, pf, o);
    pfz += __shfl_xor_sync(0xffffffffu, pfz, o);
    nbad += __shfl_xor_sync(0xffffffffu, nbad, o);
  }
  if (lane == 0) {
    red[0][warp] = ef;
    red[1][warp] = pf;
    red[2][warp] = pfz;
    if (nbad) atomicAdd(bad, (unsigned long long) nbad);
  }
  __syncthreads();
  if (tid < 3) {
    double t = 0.0;
    for (int w = 0; w < kIngestThreads / 32; w++) t += red[tid][w];
    rowflux[(size_t) row * 3 + tid] = t;
  }
}

// per corner (rows c * n_incl .. + n_incl - 1): sum over inclinations of f_i times the row integrals
__global__ void xill_corner_flux_kernel(const double *__restrict__ rowflux, const double *__restrict__ incl_w,
                                        int n_incl, int64_t n_corners, double *__restrict__ fcorr) {
  const int64_t c = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_corners) return;
  double a[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < n_incl; i++)
    for (int q = 0; q < 3; q++) a[q] += incl_w[i] * rowflux[(size_t) (c * n_incl + i) * 3 + q];
  for (int q = 0; q < 3; q++) fcorr[(size_t) c * 3 + q] = a[q];
}

cudaError_t launch_xill_ingest(cudaStream_t s, const XillIngest &g, const unsigned char *raw, int64_t row0,
                               int nrows) {
  if (nrows <= 0) return cudaSuccess;
  xill_ingest_kernel<<<nrows, kIngestThreads, 0, s>>>(raw, g.width, g.col_off, g.ne, g.pad, row0, g.lxi_div,
                                                      g.stride_lxi, g.n_lxi, g.dns_div, g.stride_dns, g.n_dns, g.xe,
                                                      g.pfz_coef, g.spec, g.rowflux, g.bad);
  return cudaGetLastError();
}

cudaError_t launch_xill_corner_flux(cudaStream_t s, const double *rowflux, const double *incl_w, int n_incl,
                                    int64_t n_corners, double *fcorr) {
  if (n_corners <= 0) return cudaSuccess;
  xill_corner_flux_kernel<<<(unsigned) ((n_corners + 127) / 128), 128, 0, s>>>(rowflux, incl_w, n_incl, n_corners,
                                                                             fcorr);
  return cudaGetLastError();
}

// one CTA per table row
__global__ void __launch_bounds__(kIngestThreads) xill_conv_rows_kernel(const float *__restrict__ spec, int pitch,
                                                                     const int4 *__restrict__ rb_pack,
                                                                     const float *__restrict__ cf, int clo, int cn,
                                                                     int cpad, float *__restrict__ out) {
  const float *x = spec + (size_t) blockIdx.x * pitch;
  float *o = out + (size_t) blockIdx.x * cpad;
  for (int q = threadIdx.x; q < cpad; q += kIngestThreads) {
    float v = 0.0f;
    if (q < cn) {
      const int4 rb = rb_pack[clo + q];  // first and last xillver bin, end fractions
      const int i0 = rb.x, i1 = rb.y;
      double a = 0.0;
      if (i0 >= 0) {
        const double fmin = __int_as_float(rb.z), fmax = __int_as_float(rb.w);
        if (i0 == i1) {
          a = fmin * x[i0];
        } else {
          a = x[i0] * fmin + x[i1] * fmax;
          for (int k = i0 + 1; k <= i1 - 1; k++) a += x[k];
        }
      }
      v = (float) (a * (double) cf[clo + q]);
    }
    o[q] = v;
  }
}

cudaError_t launch_xill_conv_rows(cudaStream_t s, const float *spec, int pitch, int64_t rows, const int4 *rb_pack,
                                  const float *cf, int clo, int cn, int cpad, float *out) {
  if (rows <= 0) return cudaSuccess;
  xill_conv_rows_kernel<<<(unsigned) rows, kIngestThreads, 0, s>>>(spec, pitch, rb_pack, cf, clo, cn, cpad, out);
  return cudaGetLastError();
}

}  // namespace relx
