// relx_runtime.h -- hooks of the host runtime (runtime.cu) used by other host
// translation units.  Not part of the C ABI.
#pragma once
#include "relx_common.h"

namespace relx {

// device tables loaded by relx_init (null until then); *device = the device they live on
const RelxTables *runtime_tables(int *device);
// radial zones a parameter set uses, and the environment options read for the call
int runtime_zones(int model, int ion_grad_type, int *nzones_env, int *flags);
// parameters of a model (-1 for an unknown model)
int runtime_nparams(int model);
// sets what relx_last_error() and relx_last_status() report
void runtime_set_error(int status, const char *msg);

}  // namespace relx
