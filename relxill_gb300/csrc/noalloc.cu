// noalloc.cu -- evaluation of one parameter set without any device allocation.
//
// Who needs this: callers that must not allocate device memory while they
// evaluate the model.  A sampler or fit that runs next to a framework whose
// caching allocator has taken the rest of the device memory cannot get a new
// buffer; a caller on a latency-critical loop cannot afford cudaMalloc and
// cudaFree, which take a driver lock and can synchronise the device, stalling
// its other streams; code that runs under a fixed, planned memory budget may
// not grow.  The batched entry points grow a workspace on demand, so they are
// not usable there.  relx_eval_one_noalloc evaluates one parameter set with
// every intermediate array carved from one static device array of fixed size;
// the caller passes the inputs and the output buffer.
//
// Limits (checked, status RELX_ERR_ARG with a message otherwise):
//   * one parameter set per call, at most RELX_NZMAX radial zones;
//   * relline: at most kMaxLineBins bins in the caller's grid (the line profile
//     is computed on that grid); the other models use the fixed conv grid;
//   * xillver tables with at most kMaxXillBins energy bins;
//   * the Cp models need the xillverCp table (status RELX_ERR_NOTABLE without it); relxilllpCp
//     reserves the zones of an ionisation gradient, since its gradient type is a parameter;
//   * the tables must have been loaded by relx_init on the current device
//     before the call (loading allocates).
//
// Set-up: the first call on a device looks up the device address of the
// static array (cudaGetSymbolAddress, which can load the module lazily).  Make
// that first call before any stream capture.  relx_release forgets the
// addresses, so that the first call after it (for instance after the caller
// reset the device) looks them up again.
//
// Tables: each call copies the table descriptor under the runtime's lock and
// its kernels read the tables until they finish.  relx_init with another table
// path, relx_release and a device reset free the tables: do not run them while
// calls of this entry point are in flight on the device.
//
// Sharing: every call on every stream uses the same static array, which keeps
// the contents of the last call.  Calls whose device work overlaps race on it:
// issue them on one stream or synchronise between them.  Each call clears what
// must start at zero (the per-set error flags); every other intermediate array
// is written in full before it is read.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "../../include/relxill_gb300.h"
#include "relx_common.h"
#include "relx_kernels.h"
#include "relx_runtime.h"

namespace relx {

constexpr int kMaxLineBins = 16384;  // relline grid limit of this entry point
constexpr int kMaxXillBins = 4096;   // padded xillver bins per spectrum
constexpr size_t kAlign = 256;

constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// the largest carve: every array at its limit
constexpr size_t kScratchBytes =
    align_up(sizeof(RelxSetIn)) + align_up(sizeof(RelxSetState)) + align_up(sizeof(RelxRadial)) +
    align_up(sizeof(RelxCorners)) + align_up(sizeof(RelxZoneCorners)) +
    align_up(sizeof(double) * (kMaxLineBins + 1)) +                                          // line grid
    align_up(sizeof(float) * (size_t) (RELX_NZMAX * RELX_NCONV > kMaxLineBins ? RELX_NZMAX * RELX_NCONV
                                                                               : kMaxLineBins)) +  // profile
    align_up(sizeof(float) * RELX_NZMAX * RELX_MAX_INCL) +                                   // angle histogram
    align_up(sizeof(double) * (size_t) ((kMaxLineBins + kSumBinsH - 1) / kSumBinsH) * RELX_NZMAX) +  // block sums
    align_up(sizeof(float) * (size_t) RELX_NZMAX * kMaxXillBins) +                           // xillver spectra
    align_up(sizeof(float) * (size_t) RELX_NZMAX * RELX_NCONV) +                             // convolved spectra
    align_up(sizeof(double) * (RELX_NZMAX + 1)) + align_up(sizeof(NthTable)) +               // nthcomp (Cp)
    align_up(sizeof(float4) * (size_t) (RELX_NZMAX + 1) * 900) +                             // nthcomp solve
    align_up(sizeof(float4) * (size_t) RELX_MAX_NRTAB * RELX_MAX_NG) +                      // interpolated table
    3 * kAlign;                                                                              // flags

// the scratch of this entry point (about 3.8 MB)
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct NoallocPtrs {
  RelxSetIn *sin;
  RelxSetState *sst;
  RelxRadial *rad;
  RelxCorners *cor;
  RelxZoneCorners *zcor;
  double *line_e, *tsum, *nthq;
  float *prof, *dist, *xill, *cout;
  NthTable *nth;
  float4 *nthscr, *htab;
  int *sflag, *err, *status;
};

// carve the arrays of one call from the scratch; returns the bytes used
static size_t carve(unsigned char *base, int model, int nza, int nbins, int ntile_max, int x_pad, int nrg,
                    NoallocPtrs *p) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char *q = base + off;
    off += align_up(bytes);
    return q;
  };
  p->sin = (RelxSetIn *) take(sizeof(RelxSetIn));
  p->sst = (RelxSetState *) take(sizeof(RelxSetState));
  p->rad = (RelxRadial *) take(sizeof(RelxRadial));
  p->cor = (RelxCorners *) take(sizeof(RelxCorners));
  p->zcor = (RelxZoneCorners *) take(sizeof(RelxZoneCorners));
  const bool line = (relx_kind(model) == RELX_RELLINE);
  p->line_e = (double *) take(line ? sizeof(double) * (nbins + 1) : 0);
  p->prof = (float *) take(sizeof(float) * (line ? (size_t) nbins : (size_t) nza * RELX_NCONV));
  p->dist = (float *) take(sizeof(float) * nza * RELX_MAX_INCL);
  p->tsum = (double *) take(sizeof(double) * ntile_max * nza);
  p->xill = (float *) take(sizeof(float) * (size_t) nza * x_pad);
  p->cout = (float *) take(sizeof(float) * (size_t) nza * RELX_NCONV);
  const bool cp = relx_is_cp(model);
  p->nthq = (double *) take(cp ? sizeof(double) * (RELX_NZMAX + 1) : 0);
  p->nth = (NthTable *) take(cp ? sizeof(NthTable) : 0);
  p->nthscr = (float4 *) take(cp ? nthcomp_scratch_bytes(1, nza, relx_kind(model) == RELX_XILLVER) : 0);
  p->htab = (float4 *) take(relx_kind(model) != RELX_XILLVER ? sizeof(float4) * (size_t) nrg : 0);
  p->sflag = (int *) take(sizeof(int));
  p->err = (int *) take(sizeof(int));
  p->status = (int *) take(sizeof(int));
  return off;
}

// RelxSetIn of the one set (energy offset 0) and the flags that must start at zero
__global__ void noalloc_pack_kernel(int npar, const double *__restrict__ params, int n_ener, int igt, double igi,
                                    int nzones_env, int flags, int nza, RelxSetIn *__restrict__ out,
                                    int *__restrict__ sflag, int *__restrict__ err) {
  if (threadIdx.x != 0) return;
  RelxSetIn s;
  for (int q = 0; q < RELX_NPARAM_MAX; q++) s.p[q] = q < npar ? params[q] : 0.0;
  s.e_off = 0;
  s.n_ener = n_ener;
  s.ion_grad_type = igt;
  s.iongrad_index = igi;
  s.nzones_env = nzones_env;
  s.flags = flags;
  s.nza = nza;
  *out = s;
  *sflag = RELX_OK;
  *err = RELX_OK;
}

__global__ void noalloc_status_kernel(const RelxSetState *__restrict__ st, const int *__restrict__ sflag,
                                      const int *__restrict__ err, int *__restrict__ status, int *__restrict__ out) {
  if (threadIdx.x != 0) return;
  int s = st->status;
  if (s == RELX_OK && *sflag != RELX_OK) s = *sflag;
  if (s == RELX_OK && *err != RELX_OK) s = *err;
  *status = s;
  if (out) *out = s;
}

// device address of the scratch, looked up once per device with that device current
static std::mutex g_setup_mu;
static void *g_scratch_ptr[64] = {nullptr};

void noalloc_forget_devices() {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  for (auto &p : g_scratch_ptr) p = nullptr;
}

static int scratch_for_device(int dev, unsigned char **out) {
  if (dev < 0 || dev >= 64) {
    runtime_set_error(RELX_ERR_ARG, "relx_eval_one_noalloc: device ordinal out of range");
    return RELX_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      char msg[256];
      std::snprintf(msg, sizeof(msg), "relx_eval_one_noalloc: cudaGetSymbolAddress of the scratch failed: %s",
                    cudaGetErrorString(e));
      runtime_set_error(RELX_ERR_CUDA, msg);
      return RELX_ERR_CUDA;
    }
    g_scratch_ptr[dev] = ptr;
  }
  *out = (unsigned char *) g_scratch_ptr[dev];
  return 0;
}

static int fail(int st, const char *msg) {
  runtime_set_error(st, msg);
  return st;
}

#define NOALLOC_CUDA(call)                                                         \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      char m_[256];                                                                \
      std::snprintf(m_, sizeof(m_), "%s: %s", #call, cudaGetErrorString(e_));      \
      return fail(RELX_ERR_CUDA, m_);                                              \
    }                                                                              \
  } while (0)

static int eval_one_noalloc(int model, const double *d_params, const double *d_energy, int n_bins,
                            const double *d_flux_in, double *d_flux, int *d_status, int ion_grad_type,
                            double iongrad_index, cudaStream_t s) {
  if (model < 0 || model >= RELX_NMODELS || !d_params || !d_energy || !d_flux || n_bins < 1)
    return fail(RELX_ERR_ARG, "relx_eval_one_noalloc: bad arguments");
  const int kind = relx_kind(model);
  const bool cp = relx_is_cp(model);
  if (kind == RELX_RELCONV && !d_flux_in)
    return fail(RELX_ERR_ARG, "relx_eval_one_noalloc: relconv needs the input spectrum");
  if (ion_grad_type < 0 || ion_grad_type > 2)
    return fail(RELX_ERR_ARG, "relx_eval_one_noalloc: ion_grad_type must be 0, 1 or 2");
  if (kind == RELX_RELLINE && n_bins > kMaxLineBins) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "relx_eval_one_noalloc: relline grid of %d bins exceeds the limit of %d bins",
                  n_bins, kMaxLineBins);
    return fail(RELX_ERR_ARG, msg);
  }
  int tab_dev = -1, dev = -1;
  RelxTables tab;
  if (!runtime_tables(&tab, &tab_dev, cp))
    return fail(RELX_ERR_NOTABLE, cp ? "relx_eval_one_noalloc: tables not loaded or xillverCp_v3.4.fits not found"
                                     : "relx_eval_one_noalloc: tables not loaded (call relx_init first)");
  NOALLOC_CUDA(cudaGetDevice(&dev));
  if (dev != tab_dev) return fail(RELX_ERR_ARG, "relx_eval_one_noalloc: the tables live on another device");
  if ((relx_is_relxill(kind) && tab.x_cpad > kMaxXillBins) || (kind == RELX_XILLVER && tab.x_nener_pad > kMaxXillBins))
    return fail(RELX_ERR_ARG, "relx_eval_one_noalloc: xillver table has more energy bins than the scratch holds");
  int nzones_env = 0, flags = 0;
  int nza = runtime_zones(model, ion_grad_type, &nzones_env, &flags);
  // relxilllpCp carries its ionisation-gradient type as a parameter (on the device here): room for
  // the zones of either choice
  if (model == RELX_RELXILLLPCP) nza = std::max(nza, runtime_zones(model, 1, nullptr, nullptr));
  if (nza < 1 || nza > RELX_NZMAX) return fail(RELX_ERR_ARG, "relx_eval_one_noalloc: zone count out of range");
  const int gbins = (kind == RELX_RELLINE) ? n_bins : RELX_NCONV;
  const int ntile_max = (gbins + kSumBinsH - 1) / kSumBinsH;  // 256-bin profile-sum blocks
  unsigned char *base = nullptr;
  int st = scratch_for_device(dev, &base);
  if (st) return st;
  NoallocPtrs p;
  if (carve(base, model, nza, n_bins, ntile_max, tab.x_cpad, tab.rel_nr * tab.rel_ng, &p) > kScratchBytes)
    return fail(RELX_ERR_ARG, "relx_eval_one_noalloc: request exceeds the static scratch");

  noalloc_pack_kernel<<<1, 32, 0, s>>>(runtime_nparams(model), d_params, n_bins, ion_grad_type, iongrad_index,
                                       nzones_env, flags, nza, p.sin, p.sflag, p.err);
  if (kind == RELX_XILLVER) {
    if (cp) NOALLOC_CUDA(launch_nthcomp(s, tab, p.sin, p.sst, 1, 1, true, p.nthq, p.nth, nullptr, nullptr, p.nthscr, 1, 0));
    NOALLOC_CUDA(launch_xillver_model(s, tab, 1, p.sin, d_energy, p.sst, d_flux, cp ? p.nthq : nullptr,
                                      cp ? p.nth : nullptr));
    noalloc_status_kernel<<<1, 32, 0, s>>>(p.sst, p.sflag, p.err, p.status, d_status);
    NOALLOC_CUDA(cudaGetLastError());
    runtime_set_error(RELX_OK, "");
    return RELX_OK;
  }
  setup_kernel<<<1, kSetupThreadsH, setup_smem_bytes(), s>>>(tab, model, p.sin, d_energy, p.line_e, p.sst, p.rad,
                                                            p.cor, p.zcor);
  if (cp) NOALLOC_CUDA(launch_nthcomp(s, tab, p.sin, p.sst, 1, nza, false, p.nthq, p.nth, p.cor, p.zcor, p.nthscr, nza + 1, 0));
  NOALLOC_CUDA(launch_line_table(1, s, tab, p.sst, p.htab));
  NOALLOC_CUDA(launch_relline(relx_is_relxill(kind), 1, ntile_max, s, tab, p.sin, p.sst, p.rad, p.line_e, nza, p.prof,
                              p.dist, p.tsum, kind == RELX_RELLINE || kind == RELX_RELCONV, nza > 1, p.htab));
  if (relx_is_relxill(kind)) {
    NOALLOC_CUDA(launch_xillver(s, tab, 1, nza, nza > RELX_ZDENSE || cp, true, p.sst, p.cor, p.zcor, p.dist, p.xill,
                                p.err, nullptr));
    conv_zone_kernel<<<dim3(nza, 1), kConvThreadsH, conv_smem_bytes(), s>>>(tab, p.sst, p.prof, p.tsum, ntile_max,
                                                                            kSumBinsH, p.xill, nza, p.cout,
                                                                            p.err);
    NOALLOC_CUDA(launch_finalize_relxill(s, true, 1, tab, p.sin, p.sst, p.cout, nza, d_energy, d_flux,
                                         cp ? p.nth : nullptr));
  } else if (kind == RELX_RELCONV) {
    relconv_conv_kernel<<<1, kConvThreadsH, conv_smem_bytes(), s>>>(tab, p.sin, p.sst, p.prof, p.tsum, ntile_max,
                                                                    kSumBinsH, nza, d_energy, d_flux_in, p.cout,
                                                                    p.sflag);
    finalize_relconv_kernel<<<1, kFinThreadsH, 0, s>>>(tab, p.sin, p.sst, p.cout, nza, d_energy, p.sflag, d_flux);
  } else {
    finalize_relline_kernel<<<1, kFinThreadsH, 0, s>>>(p.sin, p.sst, p.prof, p.tsum, ntile_max, kSumBinsH, nza,
                                                        d_flux);
  }
  noalloc_status_kernel<<<1, 32, 0, s>>>(p.sst, p.sflag, p.err, p.status, d_status);
  NOALLOC_CUDA(cudaGetLastError());
  runtime_set_error(RELX_OK, "");
  return RELX_OK;
}

}  // namespace relx

extern "C" int relx_eval_one_noalloc(int model, const double *d_params, const double *d_energy, int n_bins,
                                     const double *d_flux_in, double *d_flux, int *d_status, int ion_grad_type,
                                     double iongrad_index, void *stream) {
  return relx::eval_one_noalloc(model, d_params, d_energy, n_bins, d_flux_in, d_flux, d_status, ion_grad_type,
                                iongrad_index, (cudaStream_t) stream);
}
