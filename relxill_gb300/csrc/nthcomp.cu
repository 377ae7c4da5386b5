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
// nthcomp_kernel: one CTA of 128 threads per (continuum, set).  The grid, the
// Kompaneets coefficients and the escape probabilities are FP64, computed in
// parallel; the disk-blackbody seed spectrum (five-point Gauss-Legendre per
// bin of the multi-colour disk formula, donthcomp.c:52-191) is FP32, its
// relative error of about 1e-7 carries linearly into the spectrum; the
// tridiagonal system is solved by one thread in FP64.  Outputs: the
// continuum's normalisation with respect to the xillver table
// (calcNormWrtXillverTableSpec on the 500-bin coarse grid, Xillspec.cpp:179-205)
// and, for the source continuum, the E F_E table that the primary spectrum is
// interpolated from (c_donthcomp, donthcomp.c:640-793).
// nthcomp_apply_kernel: the normalisation changes of the zones on their corner
// weights and the source normalisation of the primary.
#include "relx_device.cuh"
#include "relx_kernels.h"

namespace relx {

constexpr int kNthThreads = 128;
constexpr int kNthMax = 900;

struct NthSmem {
  double x[kNthMax + 1];     // photon energies / m_e c^2, index 1..jmax+1
  double c2[kNthMax];        // Cooper's coefficient, then E F_E (sptot), index j-1 -> j
  double bet[kNthMax];       // escape probability per Thomson time
  double dph[kNthMax];       // seed photon production rate
  double a[kNthMax], b[kNthMax], c[kNthMax], d[kNthMax];
  double red[kNthThreads / 32];
  int jmax, jmaxth, ne_seed;
};

__device__ __forceinline__ double nth_lg10(double x) { return 0.43429448190325182765 * log(x); }

// residuals of the multi-colour disk interpolation formula in 0.06 dex steps from E/T = 1e-3
// (Mitsuda et al. 1984; the table of donthcomp.c:57-79)
__constant__ float c_mcd_res[98] = {
    9.6198382e-4f, .0010901181f, .0012310012f, .0013841352f, .0015481583f, .0017210036f, .0018988943f,
    .002076939f, .0022484281f, .0024049483f, .0025366202f, .0026316255f, .0026774985f, .0026613059f,
    .0025708784f, .0023962965f, .002130655f, .0017725174f, .0013268656f, 8.0657672e-4f, 2.3337584e-4f,
    -3.6291778e-4f, -9.4443569e-4f, -.0014678875f, -.0018873741f, -.0021588493f, -.0022448371f, -.0021198179f,
    -.0017754602f, -.0012246034f, -5.0414167e-4f, 3.2507078e-4f, .0011811065f, .0019673402f, .0025827094f,
    .0029342526f, .0029517083f, .0026012166f, .0018959062f, 9.0128649e-4f, -2.6757144e-4f, -.0014567885f,
    -.002492855f, -.0032079776f, -.0034678637f, -.0031988217f, -.0024080969f, -.001193624f, 2.6134145e-4f,
    .0017117758f, .0028906898f, .0035614435f, .0035711778f, .0028921374f, .0016385898f, 4.9857464e-5f,
    -.0015572671f, -.0028578151f, -.0035924212f, -.0036253044f, -.002975086f, -.0018044436f, -3.7796664e-4f,
    .0010076215f, .0020937327f, .0027090854f, .0028031667f, .0024276576f, .0017175597f, 8.1030795e-4f,
    -1.2592304e-4f, -9.4888491e-4f, -.0015544816f, -.0018831972f, -.0019203142f, -.0016905849f, -.0012487737f,
    -6.6789911e-4f, -2.7079461e-5f, 5.9931935e-4f, .0011499748f, .0015816521f, .0018709224f, .0020129966f,
    .0020184702f, .0019089181f, .0017122289f, .001458377f, .0011760717f, 8.9046768e-4f, 6.2190822e-4f,
    3.8553762e-4f, 1.9155022e-4f, 4.5837109e-5f, -4.9177834e-5f, -9.3670762e-5f, -8.9622968e-5f,
    -4.01538532e-5f};

// multi-colour disk integrand (donthcomp.c:52-103), FP32
__device__ __forceinline__ float nth_mcdint_f(float et) {
  const float gc[3] = {.078196667f, -1.066202f, 1.192418f};
  const float gw[3] = {.5207874f, .513457f, .4077983f};
  const float gn[3] = {.3728691f, .039775528f, .037766505f};
  const float loget = log10f(et);
  float pos = (loget + 3.0f) / .06f + 1.0f;  // log10(et) - log10(0.001), in 0.06 dex steps
  const int j = (int) pos;
  float resfact;
  if (j < 1) {
    resfact = c_mcd_res[0];
  } else if (j >= 98) {
    resfact = c_mcd_res[97];
  } else {
    pos -= (float) j;
    resfact = c_mcd_res[j - 1] * (1.0f - pos) + c_mcd_res[j] * pos;
  }
  float gaufact = 1.0f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float zz = (loget - gc[k]) / gw[k];
    gaufact += gn[k] * expf(-zz * zz * 0.5f);
  }
  return powf(et * 1000.0f, -2.0f / 3.0f) * 193.21556f * (powf(et, 1.663753f) * .52876731f + 1.0f) * expf(-et) *
         gaufact * (resfact + 1.0f);
}

// Comptonized spectrum of one (theta, gamma): fills m.x[1..jmax+1] and m.c2[j] = sptot[j] for
// j = 1..jmax (sptot[jmax] = 0, as the reference's cleared array), returns jmax, or 0 when kTe gives
// fewer than 4 grid points (kTe <= 0 or far below the seed temperature): nothing is computed then
__device__ int nth_compton(NthSmem &m, double tempbb, double theta, double gamma) {
  const int tid = threadIdx.x;
  const double d1 = gamma + .5;
  const double tautom = sqrt(3. / (theta * (d1 * d1 - 2.25)) + 2.25) - 1.5;
  const double delta = .02, deltal = delta * log(10.);
  const double xmin = tempbb * 1e-4, xmax = theta * 40.;
  if (tid == 0) {
    int jmax = (int) (nth_lg10(xmax / xmin) / delta) + 1;
    if (jmax > 899) jmax = 899;
    int jmaxth = (int) (nth_lg10(tempbb * 50. / xmin) / delta);
    if (jmaxth > 900) jmaxth = 900;
    if (jmaxth > jmax) jmaxth = jmax;
    m.jmax = jmax;
    m.jmaxth = jmaxth;
    m.ne_seed = jmaxth - 2;
  }
  __syncthreads();
  const int jmax = m.jmax, ne = m.ne_seed;
  if (!(jmax >= 4 && jmax <= 899)) return 0;  // block-uniform
  for (int j = 1 + tid; j <= jmax + 1; j += kNthThreads) m.x[j] = xmin * exp((double) (j - 1) * deltal);
  for (int j = tid; j < kNthMax; j += kNthThreads) m.dph[j] = 0.0;
  __syncthreads();
  // Cooper's coefficient and the Klein-Nishina escape probability (donthcomp.c:511-585)
  const int jnr = min((int) (nth_lg10(.1 / xmin) / delta + 1), jmax - 1);
  const int jrel = min((int) (nth_lg10(1. / xmin) / delta + 1), jmax);
  const double xnr = m.x[jnr], xr = m.x[jrel];
  for (int j = 1 + tid; j <= jmax; j += kNthThreads) {
    const double w = m.x[j], w1 = sqrt(m.x[j] * m.x[j + 1]);
    const double w12 = w1 * w1;
    m.c2[j - 1] = w12 * w12 / (w1 * 4.6 + 1. + w1 * 1.1 * w1);
    double rel;
    if (w <= .05) {
      rel = 1 - w * 2 + w * 26 * w / 5;
    } else {
      const double z1 = (w + 1) / (w * (w * w)), z2 = w * 2 + 1, z3 = log(z2), z4 = w * 2 * (w + 1) / z2,
                   z5 = z3 / 2 / w, z6 = (w * 3 + 1) / z2 / z2;
      rel = (z1 * (z4 - z3) + z5 - z6) * .75;
    }
    const double taukn = tautom * rel;
    double bet;
    if (j <= jnr - 1) bet = 1 / tautom / (taukn / 3 + 1);
    else if (j <= jrel) bet = 1 / tautom / (taukn / 3 * (1 - (w - xnr) / (xr - xnr)) + 1);
    else bet = 1 / tautom;
    m.bet[j - 1] = bet;
  }
  // seed photons: the disk-blackbody spectrum per bin (xsdskb, donthcomp.c:137-191), FP32
  {
    const float gw5[5] = {.236926885f, .47862867f, .568888888f, .47862867f, .236926885f};
    const float gx5[5] = {-.906179846f, -.53846931f, 0.f, .53846931f, .906179846f};
    const float tin = (float) (tempbb * 511.);
    for (int i = 1 + tid; i <= ne; i += kNthThreads) {
      const double elo = sqrt(m.x[i] * m.x[i + 1]) * 511., ehi = sqrt(m.x[i + 1] * m.x[i + 2]) * 511.;
      const float xn = (float) ((ehi - elo) / 2.), xh = xn + (float) elo;
      float acc = 0.0f;
#pragma unroll
      for (int k = 0; k < 5; k++) {
        const float e = xn * gx5[k] + xh;
        acc += gw5[k] * (nth_mcdint_f(e / tin) * tin * tin / 361.0f);
      }
      m.dph[i] = (double) (acc * xn) * 511. / (ehi - elo);
    }
  }
  __syncthreads();
  if (tid == 0) m.dph[0] = m.dph[1];
  __syncthreads();
  // tridiagonal coefficients a u(j+1) + b u(j) + c u(j-1) = d (thermlc, donthcomp.c:194-280)
  const double c20 = tautom / deltal, td = theta / deltal;
  for (int j = 2 + tid; j <= jmax - 1; j += kNthThreads) {
    const double w1 = sqrt(m.x[j] * m.x[j + 1]), w2 = sqrt(m.x[j - 1] * m.x[j]);
    m.a[j - 1] = -c20 * m.c2[j - 1] * (td / w1 + .5);
    const double t1 = -c20 * m.c2[j - 1] * (.5 - td / w1);
    const double t2 = c20 * m.c2[j - 2] * (td / w2 + .5);
    const double xj = m.x[j];
    const double t3 = xj * xj * xj * (tautom * m.bet[j - 1]);
    m.b[j - 1] = t1 + t2 + t3;
    m.c[j - 1] = c20 * m.c2[j - 2] * (.5 - td / w2);
    m.d[j - 1] = xj * m.dph[j - 1];
  }
  __syncthreads();
  if (tid == 0) {  // Thomas algorithm: gam in a, alp in b, g then u in d
    const double x32 = sqrt(m.x[1] * m.x[2]);
    const double aa = (td / x32 + .5) / (td / x32 - .5);
    double alp = m.b[1] + m.c[1] * aa;
    m.a[1] = m.a[1] / alp;
    m.d[1] = m.d[1] / alp;
    for (int j = 3; j <= jmax - 1; j++) {
      alp = m.b[j - 1] - m.c[j - 1] * m.a[j - 2];
      const double ia = 1.0 / alp;
      m.a[j - 1] = m.a[j - 1] * ia;
      m.d[j - 1] = (m.d[j - 1] - m.c[j - 1] * m.d[j - 2]) * ia;
    }
    // u(jmax) = 0: the last row is the same recurrence
    m.d[jmax - 1] = 0.0;
    for (int jj = jmax - 2; jj >= 2; jj--) m.d[jj - 1] = m.d[jj - 1] - m.a[jj - 1] * m.d[jj];
    m.d[0] = aa * m.d[1];
  }
  __syncthreads();
  // E F_E of the escaping photons (donthcomp.c:603-610); c2 is free now
  for (int j = 1 + tid; j <= jmax; j += kNthThreads) {
    const double xj = m.x[j];
    const double dphesc = xj * xj * m.d[j - 1] * m.bet[j - 1] * tautom;
    m.c2[j] = (j <= jmax - 1) ? dphesc * (xj * xj) : 0.0;
  }
  __syncthreads();
  return jmax;
}

// continuum k of set: k = 0 the source (kTe), k = z + 1 zone z (kTe times the zone's energy shift);
// params: the xillver model reads Gamma and kTe from its parameters (p[0], p[2])
__global__ void __launch_bounds__(kNthThreads) nthcomp_kernel(RelxTables tab, const RelxSetIn *__restrict__ sin,
                                                              const RelxSetState *__restrict__ sst, bool params,
                                                              int nq, double *__restrict__ qout,
                                                              NthTable *__restrict__ tabs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  NthSmem &m = *reinterpret_cast<NthSmem *>(smem_raw);
  const int k = blockIdx.x, set = blockIdx.y, tid = threadIdx.x;
  double gam, kte;
  if (params) {
    if (k > 0) return;
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
  const int jmax = nth_compton(m, .05 / 511., kte / 511., gam);
  if (jmax == 0) {  // no spectrum: a non-finite normalisation marks the set as failed
    if (tid == 0) {
      qout[(size_t) set * nq + k] = __longlong_as_double(0x7ff8000000000000ll);
      if (k == 0) tabs[set].n = 0;
    }
    return;
  }
  const double *x = m.x, *sp = m.c2;
  // normalisation on the coarse grid (calcNormWrtXillverTableSpec, Xillspec.cpp:179-205): the
  // E F_E table at the 501 edges in FP32, the per-bin photon flux times the bin centre summed in FP64
  const double normfac = nth_normfac(x, sp, jmax, 1.0);
  double part = 0.0;
  for (int bn = tid; bn < RELX_NCOARSE; bn += kNthThreads) {
    const double e0 = tab.coarse_e[bn], e1 = tab.coarse_e[bn + 1];
    const float4 t = tab.coarse_t[bn];  // zero centre weight outside the normalisation band
    if (t.z == 0.0f) continue;
    const double p0 = nth_prim_at(x, sp, jmax, e0, 1.0), p1 = nth_prim_at(x, sp, jmax, e1, 1.0);
    const double ph = (p1 / (e1 * e1) + p0 / (e0 * e0)) * .5 * (e1 - e0) * normfac;
    part += ph * ((double) t.z + (double) t.w);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((tid & 31) == 0) m.red[tid >> 5] = part;
  __syncthreads();
  if (tid == 0) {
    double sum = 0.0;
    for (int w = 0; w < kNthThreads / 32; w++) sum += m.red[w];
    qout[(size_t) set * nq + k] = sum * 1e20 * 1.602177e-09 / (1e15 / 4.0 / kPi);
  }
  if (k == 0) {  // the source's table for the primary spectrum
    NthTable &T = tabs[set];
    for (int j = tid; j <= jmax + 1; j += kNthThreads) {
      T.x[j] = x[j];
      T.sp[j] = (j >= 1 && j <= jmax) ? sp[j] : 0.0;
    }
    if (tid == 0) T.n = jmax;
  }
}

// normalisation changes of the zones on their corner weights, source normalisation of the primary
__global__ void nthcomp_apply_kernel(RelxSetState *__restrict__ sst, const double *__restrict__ q, int nq,
                                     RelxZoneCorners *__restrict__ zcor) {
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
  for (int e = tid; e < s.nz * 32; e += blockDim.x) {
    const int z = e >> 5, c = e & 31;
    const double xs = (s.zshift[z] == 1.0) ? 1.0 : q[(size_t) set * nq + z + 1] * (1.0 / q0);
    zcor[set].w[z][c] = (float) ((double) zcor[set].w[z][c] * xs);
    if (c == 0) s.inv_nc[z] = (float) xs;
  }
  if (tid == 0) s.src_norm = 1.0 / q0;
}

size_t nthcomp_smem_bytes() { return sizeof(NthSmem); }

cudaError_t nthcomp_set_smem() {
  return cudaFuncSetAttribute(nthcomp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sizeof(NthSmem));
}

cudaError_t launch_nthcomp(cudaStream_t s, const RelxTables &tab, const RelxSetIn *sin, RelxSetState *sst, int n_sets,
                           int nza, bool params, double *q, NthTable *tabs, RelxZoneCorners *zcor) {
  if (n_sets <= 0) return cudaSuccess;
  const int nq = RELX_NZMAX + 1;
  nthcomp_kernel<<<dim3(params ? 1 : nza + 1, n_sets), kNthThreads, sizeof(NthSmem), s>>>(tab, sin, sst, params, nq,
                                                                                        q, tabs);
  if (!params && zcor) nthcomp_apply_kernel<<<n_sets, 128, 0, s>>>(sst, q, nq, zcor);
  return cudaGetLastError();
}

}  // namespace relx
