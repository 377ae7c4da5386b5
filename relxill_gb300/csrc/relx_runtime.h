// relx_runtime.h -- hooks of the host runtime (runtime.cu) used by other host
// translation units.  Not part of the C ABI.
#pragma once
#include <cstddef>
#include <cstdint>

#include "relx_common.h"

namespace relx {

// copies the descriptor of the device tables loaded by relx_init into *out (false until then, or
// for cp when the xillverCp table was not found); *device = the device they live on.
// cp: the descriptor of the Cp models
bool runtime_tables(RelxTables *out, int *device, bool cp = false);
// forgets the per-device scratch addresses of the no-allocation entry point (relx_release)
void noalloc_forget_devices();
// radial zones a parameter set uses, and the environment options read for the call
int runtime_zones(int model, int ion_grad_type, int *nzones_env, int *flags);
// parameters of a model (-1 for an unknown model)
int runtime_nparams(int model);
// sets what relx_last_error() and relx_last_status() report
void runtime_set_error(int status, const char *msg);

// one batch of parameter sets in host memory (layout of relx_eval_batch)
struct HostBatch {
  int model = 0, n_sets = 0;
  const double *params = nullptr;   // n_sets x npar
  const double *energy = nullptr;   // concatenated edges
  const int64_t *eoff = nullptr;    // n_sets + 1 edge offsets
  const double *flux_in = nullptr;  // relconv inputs (flux layout) or null
  const int *igt = nullptr;         // ionisation-gradient type per set or null
  const double *igi = nullptr;      // ionisation-gradient index per set or null
};

// A batch slot owns a workspace, pinned staging, a stream and a completion event, so that
// batches on different slots are in flight together (serving engine).
struct BatchSlot;
// arena_bytes: the device region every batch of the slot is carved from (allocated here, so that
// serving allocates no device memory); pinned_bytes: the initial host staging
int slot_create(BatchSlot **out, size_t arena_bytes, size_t pinned_bytes);
void slot_destroy(BatchSlot *b);
// queue a batch on the slot (asynchronous); the slot's previous batch must have been waited for
int slot_enqueue(BatchSlot *b, const HostBatch &hb, bool use_cache);
// wait for the slot's batch; flux (flux layout of relx_eval_batch) and statuses in pinned memory,
// valid until the next slot_enqueue
int slot_wait(BatchSlot *b, const double **flux, const int **status);
// device workspace bytes of a batch (admission control; an upper bound of what the slot carves):
// n_edges energy edges in all, max_bins the largest set's bins, nza zones
size_t batch_device_bytes(int model, int n_sets, int64_t n_edges, int max_bins, int nza);
// (re)create the line-profile cache with `slots` entries (0: off)
int cache_configure(int slots);

}  // namespace relx
