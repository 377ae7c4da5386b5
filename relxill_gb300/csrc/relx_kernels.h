// relx_kernels.h -- declarations of the sm_103a kernels and their launch
// geometry, used by the host runtime (runtime.cu).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "relx_common.h"

namespace relx {

constexpr int kSetupThreadsH = 256;
constexpr int kLineThreadsH = 256;
constexpr int kSumBinsH = 256;   // bins per profile-sum block (tsum)
constexpr int kLineTileH = 512;  // energy bins per line-profile CTA
constexpr int kConvThreadsH = 256;
constexpr int kFinThreadsH = 128;
constexpr int kXmodThreadsH = 256;  // xillver model kernel

size_t setup_smem_bytes();
size_t line_smem_bytes(int nr, int ng, bool limb, int tile);
size_t hist_smem_bytes(int nr, int ng);
size_t conv_smem_bytes();
size_t fin_smem_bytes();

__global__ void setup_kernel(RelxTables tab, int model, const RelxSetIn *sin, const double *user_e, double *line_e,
                             RelxSetState *sout, RelxRadial *rout, RelxCorners *cout, RelxZoneCorners *zcout);

cudaError_t relline_set_smem(int nr, int ng);
// the sets' (a, mu0)-interpolated transfer-function tables (rel_nr x rel_ng float4 per set), read
// by the line profile and the emission-angle histogram
cudaError_t launch_line_table(int n_sets, cudaStream_t s, const RelxTables &tab, const RelxSetState *sst,
                              float4 *htab);
// nblk: 256-bin profile-sum blocks per set; htab: written by launch_line_table
cudaError_t launch_relline(bool hist, int n_sets, int nblk, cudaStream_t s, const RelxTables &tab,
                           const RelxSetIn *sin, const RelxSetState *sst, const RelxRadial *srad, const double *line_e,
                           int nza, float *prof, float *dist, double *tsum, bool any_limb, bool zsplit,
                           const float4 *htab);
// the emission-angle histograms alone (relxill models), for a launch on its own stream
cudaError_t launch_hist(int n_sets, cudaStream_t s, const RelxTables &tab, const RelxSetState *sst,
                        const RelxRadial *srad, int nza, float *dist, bool zsplit, const float4 *htab);

cudaError_t xillver_set_smem(int n_incl);
// bounded-wait self-test: writes the status of a wait that cannot complete (RELX_ERR_TIMEOUT)
cudaError_t launch_wait_selftest(cudaStream_t s, unsigned long long limit_ns, int *out);
// order: the sets in visiting order (launch_xill_order), or null for batch order
cudaError_t launch_xillver(cudaStream_t s, const RelxTables &tab, int n_sets, int nza, bool zone, bool dense,
                           const RelxSetState *sst, const RelxCorners *cor, const RelxZoneCorners *zcor,
                           const float *dist, float *xout, int *err, const int *order);
void launch_xill_order(cudaStream_t s, const RelxSetState *sst, const RelxCorners *cor, const RelxZoneCorners *zcor,
                       int n_sets, int *order);

// decoding of the xillver table's raw FITS rows on the device (table_ingest.cu)
struct XillIngest {
  int64_t width, col_off;   // bytes per FITS row, byte offset of the spectrum column
  int ne, pad;              // energies per spectrum, padded row length
  const double *lxi_div;    // 10^logXi per logXi grid value
  int64_t stride_lxi;       // row-index stride of the logXi parameter
  int n_lxi;                // logXi grid values (0: no logXi parameter)
  const double *dns_div;    // 10^(logN - 15) per density grid value (1 where logN = 15)
  int64_t stride_dns;       // row-index stride of the density parameter
  int n_dns;                // density grid values (0: no density parameter)
  const double *xe;         // xillver energy edges [ne + 1]
  const double *pfz_coef;   // photon flux of the spectrum shifted by g = 2/3, per energy
  float *spec;              // [rows][pad] output
  double *rowflux;          // [rows][3] energy flux, photon flux, shifted photon flux
  unsigned long long *bad;  // count of values that are not finite
};
cudaError_t launch_xill_ingest(cudaStream_t s, const XillIngest &g, const unsigned char *raw, int64_t row0, int nrows);
// every table row rebinned onto the conv bins [clo, clo + cn) and weighted by cf, rows of cpad floats
cudaError_t launch_xill_conv_rows(cudaStream_t s, const float *spec, int pitch, int64_t rows, const int4 *rb_pack,
                                  const float *cf, int clo, int cn, int cpad, float *out);
cudaError_t launch_xill_corner_flux(cudaStream_t s, const double *rowflux, const double *incl_w, int n_incl,
                                    int64_t n_corners, double *fcorr);

// the nthcomp photon grid and its per-point constants (host, FP64); co: the coarse normalisation
// grid's edges, bins starting inside [band_lo, band_hi] count
int nth_grid_build(const std::vector<double> &co, double band_lo, double band_hi, NthGrid &G);
cudaError_t nthcomp_set_smem();
// scratch of launch_nthcomp for n_sets sets (float4 per grid point and continuum)
size_t nthcomp_scratch_bytes(int n_sets, int nza, bool params);
// per set: the normalisation (calcNormWrtXillverTableSpec) of the source continuum (q[set][0]) and of
// every zone's (q[set][z + 1]), q holding RELX_NZMAX + 1 values per set, and the source's table;
// then the zones' normalisation changes on their corner weights (cor for sets with the de-duplicated
// list, zcor for the others) and the source normalisation.
// params: the xillver model, Gamma and kTe from the parameters, the source continuum only.
// scr: scratch of nthcomp_scratch_bytes for the whole batch, ncont_all continua per grid point,
// this launch's continua starting at c_off.
cudaError_t launch_nthcomp(cudaStream_t s, const RelxTables &tab, const RelxSetIn *sin, RelxSetState *sst, int n_sets,
                           int nza, bool params, double *q, NthTable *tabs, RelxCorners *cor, RelxZoneCorners *zcor,
                           float4 *scr, int64_t ncont_all, int64_t c_off);

// the xillver model: one CTA per set, writes the flux and the status fields of the set state
size_t xillver_model_smem_bytes(int n_ener, int n_ener_pad);
cudaError_t xillver_model_set_smem(int n_ener, int n_ener_pad);
// xillverCp: nthq / nth from launch_nthcomp (params mode); null for xillver
cudaError_t launch_xillver_model(cudaStream_t s, const RelxTables &tab, int n_sets, const RelxSetIn *sin,
                                 const double *user_e, RelxSetState *sst, double *flux, const double *nthq,
                                 const NthTable *nth);

__global__ void conv_zone_kernel(RelxTables tab, const RelxSetState *sst, const float *prof, const double *tsum,
                                 int ntile_max, int tile_bins, const float *xill, int nza, float *cout, int *err);
__global__ void relconv_conv_kernel(RelxTables tab, const RelxSetIn *sin, const RelxSetState *sst, const float *prof,
                                    const double *tsum, int ntile_max, int tile_bins, int nza, const double *user_e,
                                    const double *user_f, float *cout, int *sflag);
// nth: the nthcomp tables of the sets (Cp models), or null
// zone sum, primary continuum and rebin to the caller's grid; wide: 512 threads per set (for few sets)
cudaError_t launch_finalize_relxill(cudaStream_t s, bool wide, int n_sets, const RelxTables &tab,
                                    const RelxSetIn *sin, const RelxSetState *sst, const float *cout, int nza,
                                    const double *user_e, double *flux, const NthTable *nth);
__global__ void finalize_relconv_kernel(RelxTables tab, const RelxSetIn *sin, const RelxSetState *sst,
                                        const float *cout, int nza, const double *user_e, const int *sflag,
                                        double *flux);
__global__ void finalize_relline_kernel(const RelxSetIn *sin, const RelxSetState *sst, const float *prof,
                                        const double *tsum, int ntile_max, int tile_bins, int nza, double *flux);

}  // namespace relx
