/*
 * relxill_gb300.h -- C ABI of the GB300 (sm_103a) implementation of relxill's
 * relativistic convolution path.
 *
 * The ten local-model entry points keep the signature that the reference's
 * wrapper generator emits for XSPEC (src/create_wrapper_xspec.py:153-162) and
 * the parameter order of src/modelfiles/lmodel_relxill_public.dat, so a host
 * package that loads the reference's librelxill can load this library
 * instead.  Tables are found through RELXILL_TABLE_PATH as in the reference
 * (src/relutility.c:320-328).  The same environment switches are honoured:
 * RELXILL_NUM_RZONES, RELLINE_PHYSICAL_NORM, RELXILL_RENORMALIZE,
 * RELXILL_CONSTANT_DENSITY.  Returning radiation ($switch_returnrad of the
 * lamp-post models) reads table_returnRad_v20220301.fits from the same path;
 * a set that switches it on without that table fails with status 2.
 *
 * Errors: the void entry points fill `flux` with zeros on failure and record
 * the status (relx_last_status); the batched calls return it.
 */
#ifndef RELXILL_GB300_H
#define RELXILL_GB300_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* model ids of the batched calls */
enum {
  RELX_MODEL_RELLINE = 0, RELX_MODEL_RELCONV = 1, RELX_MODEL_RELXILL = 2, RELX_MODEL_RELXILLLP = 3,
  RELX_MODEL_RELLINELP = 4, RELX_MODEL_RELCONVLP = 5, RELX_MODEL_XILLVER = 6,
  RELX_MODEL_XILLVERCP = 7, RELX_MODEL_RELXILLCP = 8, RELX_MODEL_RELXILLLPCP = 9
};

/* Local models.  Replace c_lmodrelline / c_lmodrelconv / c_lmodrelxill /
 * c_lmodrelxilllp, generated by src/create_wrapper_xspec.py:153-162 from
 * lmodel_relxill_public.dat:1,13,46,61 and dispatched through
 * xspec_C_wrapper_eval_model (src/LocalModel.cpp:143-160).
 * energy: Nflux+1 ascending bin edges [keV]; parameter: the model's lmodel.dat
 * parameters in order; flux: Nflux photon fluxes per bin (input spectrum as
 * well for relconv); spectrum, fluxError and init are unused, as in the
 * reference. */
void c_lmodrelline(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                   double *fluxError, const char *init);
void c_lmodrelconv(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                   double *fluxError, const char *init);
void c_lmodrelxill(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                   double *fluxError, const char *init);
void c_lmodrelxilllp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init);
/* The lamp-post line and convolution models and the non-relativistic xillver
 * model (lmodel_relxill_public.dat:23,35,77; the same generated wrappers):
 * relline_lp takes lineE, h, a, Incl, Rin, Rout, z, limb, gamma,
 * switch_returnrad; relconv_lp h, beta, a, Incl, Rin, Rout, limb, gamma,
 * switch_returnrad (flux carries the input spectrum); xillver gamma, Afe,
 * Ecut, logxi, z, Incl, refl_frac. */
void c_lmodrellinelp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init);
void c_lmodrelconvlp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init);
void c_lmodxillver(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                   double *fluxError, const char *init);
/* The Cp flavour (lmodel_relxill_public.dat:86,96,112): the nthcomp primary
 * continuum (seed temperature 0.05 keV) and the 6-parameter table
 * xillverCp_v3.4.fits.  xillverCp takes gamma, Afe, kTe, logxi, logN, z,
 * Incl, refl_frac; relxillCp Incl, a, Rin, Rout, Rbr, Index1, Index2, z,
 * gamma, logxi, logN, Afe, kTe, refl_frac; relxilllpCp Incl, a, Rin, Rout, h,
 * beta, gamma, logxi, logN, Afe, kTe, refl_frac, z, iongrad_index,
 * $iongrad_type, $switch_returnrad, $switch_reflfrac_boost. */
void c_lmodxillverdensnthcomp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                              double *fluxError, const char *init);
void c_lmodrelxilldensnthcomp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                              double *fluxError, const char *init);
void c_lmodrelxilllpdensnthcomp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                                double *fluxError, const char *init);
/* The NS flavour of the public model list (lmodel_relxill_public.dat:131-153) is not part of
 * this library: the symbols exist so that a package built from the whole list links; a call
 * fills flux with zeros and sets relx_last_status() to 3 (unsupported). */
void c_lmodxillverns(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init);
void c_lmodrelxillns(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init);

/* Status of the last call on this process (0 = success).  The reference has
 * no status channel (src/LocalModel.cpp:153-159); this replaces its printed
 * errors and escaping exceptions. */
int relx_last_status(void);
const char *relx_last_error(void);

/* Load the tables from table_path (NULL: RELXILL_TABLE_PATH or "./") onto
 * the current CUDA device.  Called implicitly by the first evaluation; the
 * reference loads lazily in the same way (src/reltable.c:235,384,
 * src/xilltable.c:719). */
int relx_init(const char *table_path);
/* bytes of device memory held by the tables */
int relx_table_bytes(int64_t *bytes);
/* free all device memory of the library */
void relx_release(void);

/* Batched evaluation with host buffers; no counterpart in the reference,
 * which evaluates one parameter set per call.
 * params: n_sets x npar (npar = 10, 8, 13, 14, 10, 9, 7, 8, 14, 17 for relline,
 *   relconv, relxill, relxilllp, relline_lp, relconv_lp, xillver, xillverCp,
 *   relxillCp, relxilllpCp; lmodel.dat order);
 * energy: concatenated bin edges; set i uses energy[energy_offsets[i] ..
 *   energy_offsets[i+1]-1] (n_i + 1 edges);
 * flux: concatenated outputs, set i at flux[energy_offsets[i] - i .. + n_i - 1];
 * flux_in: relconv / relconv_lp input spectra in the same layout as flux
 *   (NULL otherwise);
 * status: n_sets per-set statuses (may be NULL);
 * ion_grad_type / iongrad_index: per-set hidden ionisation-gradient switch
 *   (0 const, 1 power law, 2 alpha disk) of relxilllp (NULL: 0).
 * Returns 0 or the first non-zero set status / API error. */
int relx_eval_batch(int model, int n_sets, const double *params, const double *energy,
                    const int64_t *energy_offsets, const double *flux_in, double *flux, int *status,
                    const int *ion_grad_type, const double *iongrad_index);

/* Same with device buffers, asynchronous on `stream` (a cudaStream_t; NULL:
 * the library's stream).  flux_in (relconv) uses the energy-edge layout
 * (set i at energy_offsets[i]).  h_energy_offsets and h_ion_grad_type are host
 * copies used to size the launch; for relxilllpCp, whose ionisation-gradient
 * type is parameter 15, h_ion_grad_type carries those values (NULL: all 0; a
 * set that needs more zones than the launch was sized for fails with
 * status 9). */
int relx_eval_batch_device(int model, int n_sets, const double *d_params, const double *d_energy,
                           const int64_t *d_energy_offsets, const int64_t *h_energy_offsets, const double *d_flux_in,
                           double *d_flux, int *d_status, const int *d_ion_grad_type, const int *h_ion_grad_type,
                           const double *d_iongrad_index, void *stream);

/* One parameter set, device buffers, no device allocation; no counterpart in
 * the reference.  For callers that must not allocate device memory while they
 * evaluate (memory owned by another framework's caching allocator, a fixed
 * memory budget, or a loop where cudaMalloc/cudaFree would stall other
 * streams).  Intermediate arrays live in one static device array of about
 * 3.8 MB shared by all calls: calls whose device work overlaps race on it, so
 * issue them on one stream or synchronise between them.  The first call on a
 * device looks up that array's address; make it before any stream capture.
 * relx_release (or relx_init with another table path) frees the tables these
 * calls read: do not run it while such calls are in flight on the device.
 * Limits: one set, relline grids of at most 16384 bins, tables loaded by
 * relx_init on the current device beforehand (RELX_ERR_NOTABLE otherwise; the
 * Cp models also need xillverCp_v3.4.fits).
 * d_params: npar doubles; d_energy: n_bins + 1 edges; d_flux_in: relconv input
 * (n_bins, else NULL); d_flux: n_bins outputs; d_status: one int (may be NULL).
 * Asynchronous on `stream` (a cudaStream_t; NULL: the default stream). */
int relx_eval_one_noalloc(int model, const double *d_params, const double *d_energy, int n_bins,
                          const double *d_flux_in, double *d_flux, int *d_status, int ion_grad_type,
                          double iongrad_index, void *stream);

/* Device line-profile cache, the counterpart of the reference's relbase
 * cache (src/Relcache.cpp:311-331, src/Relbase.cpp:461-538): sets whose
 * relativistic parameters match a cached entry reuse its line profile and skip
 * the line-profile kernels.  slots entries of about 260 KB each (rounded up to
 * a power of two); 0 turns it off (the default).  Used by every batched,
 * device and serving call; relline (whose profile lives on the caller's grid)
 * and sets with more than 16 zones are not cached. */
int relx_cache_config(int slots);
/* out[0] lookups, out[1] hits, out[2] slots */
int relx_cache_stats(int64_t *out);

/* Output cache of the local-model entry points (c_lmod*), the counterpart of
 * the reference's RelxillCache (src/Relcache.h:182-251, src/Relxill.cpp:295-400):
 * a relxill, relxilllp, relxillCp or relxilllpCp call whose parameters all lie
 * within 1e-8 of a recent call's (the reference's CACHE_LIMIT), on the same
 * energy grid and with the same environment options (RELXILL_NUM_RZONES,
 * RELLINE_PHYSICAL_NORM, RELXILL_RENORMALIZE, RELXILL_CONSTANT_DENSITY), returns
 * that call's flux without evaluating.  The last max_entries successful calls
 * are kept (50 by default, the reference's RELXILL_CACHE_SIZE); 0 turns it
 * off.  relx_init with other tables empties it.  Batched, device and serving
 * calls do not use it. */
int relx_output_cache_config(int max_entries);
/* out[0] lookups, out[1] hits, out[2] entries held */
int relx_output_cache_stats(int64_t *out);

/* Serving engine (no counterpart in the reference): continuous batching of
 * single-spectrum requests from many clients onto the batched path.  A
 * scheduler thread forms a batch of waiting requests (one model, arrival
 * order) whenever one of two batch slots is free, so a new batch is staged
 * while the previous one runs; a completion thread copies results to the
 * clients' buffers.  hbm_budget_bytes is the device workspace of the two
 * slots: each slot allocates half of it here and carves every batch from it
 * (admission control keeps a batch within it; a single request that needs
 * more completes with RELX_ERR_NOMEM), so serving allocates no device memory.
 * Returns NULL when the budget cannot be allocated.  max_batch bounds a
 * batch; cache_slots > 0 turns on the line-profile cache with that many
 * entries.  Results do not depend on which requests share a batch. */
typedef struct relx_server relx_server;
relx_server *relx_serve_create(int64_t hbm_budget_bytes, int max_batch, int cache_slots);
/* Queue one evaluation.  energy (n_bins + 1 edges), flux_in (relconv) and
 * flux_out (n_bins) are the caller's host buffers and must stay valid until
 * the request completes.  Returns the request id (>= 0) or -status. */
int64_t relx_serve_submit(relx_server *s, int model, const double *params, const double *energy, int n_bins,
                          const double *flux_in, double *flux_out, int ion_grad_type, double iongrad_index);
/* Completed requests since the last poll (at most max): ids, statuses and
 * latencies (submit to result in the caller's buffer, ms).  Completions are
 * kept until a poll returns them.  Returns the count. */
int relx_serve_poll(relx_server *s, int64_t *ids, int *status, double *latency_ms, int max);
/* Block until request id has completed (and has not yet been polled). */
int relx_serve_wait(relx_server *s, int64_t id, int *status);
/* out[0] completed, [1] batches, [2] mean batch size, [3] p50 ms, [4] p99 ms,
 * [5] max ms, [6] waiting requests, [7] last error; reset != 0 restarts the
 * latency and batch statistics. */
int relx_serve_stats(relx_server *s, double *out, int n, int reset);
/* Finish the queued requests and stop the engine. */
void relx_serve_destroy(relx_server *s);

/* Self-test of the bounded waits of the TMA pipeline (no counterpart in the
 * reference): one kernel waits, with a limit of limit_ms (at most 1000), on an
 * mbarrier that nothing completes and reports the status it saw in *status
 * (RELX_ERR_TIMEOUT).  No copy is issued; the context stays usable. */
int relx_selftest_wait_timeout(double limit_ms, int *status);

/* Launch tuning (no counterpart in the reference).  autotune != 0: the first
 * batch of 2048 sets or more of a (model, batch-size class, zone count) is run
 * once per candidate (one range, or pipelined chunks of 1024 sets) and the
 * fastest is kept for the class; that batch synchronises its stream (smaller
 * batches have one candidate, recorded without trials; the line-kernel tile is
 * fixed at 512 bins).
 * graphs != 0: a batch shape that recurs on the same workspace is captured
 * into a CUDA graph on its second launch and replayed afterwards.  Both are on
 * by default; every choice gives the same numbers. */
int relx_tuning_config(int autotune, int graphs);
/* tuned classes, 6 doubles each: model, size class (log2 of the set count),
 * zones, line tile, chunk, best ms; returns the count (at most max) */
int relx_tuning_report(double *out, int max);

/* Measurement hooks (no counterpart in the reference).  When enabled, every
 * kernel of every batch is bracketed by CUDA events on its launching stream;
 * relx_profile_read synchronises and returns the accumulated milliseconds
 * and launch counts per kernel kind (relx_profile_name(k), k < 9). */
int relx_profile_enable(int on);
int relx_profile_read(double *ms, int64_t *launches, int n);
const char *relx_profile_name(int k);
/* number of kernel launches issued by the library since load */
int64_t relx_launch_count(void);
/* statistics of the last batch of n_sets sets: out[0] de-duplicated xillver
 * corners, out[1] radial zones, out[2] line-profile window bins (sums);
 * out[3] floats per xillver table row on the convolution grid (the rows the
 * relxill models read), out[4] floats per row on the table's own grid; out
 * holds 5 values */
int relx_batch_stats(int n_sets, int64_t *out);
/* the FP32 FMA rate of the current device in GFLOP/s (2 FLOPs per FMA), timed
 * with CUDA events over a kernel of independent FMA chains on every SM: the
 * denominator of the line-profile kernel's roofline */
int relx_fp32_rate(double *gflops);

#ifdef __cplusplus
}
#endif
#endif
