/*
 * ref_driver.cpp -- C entry point into the compiled relxill reference
 * (oracle/_ref/librelxill_ref.so).  TEST INFRASTRUCTURE ONLY.
 *
 * ref_eval() evaluates one model through the reference's own local-model
 * path: xspec_C_wrapper_eval_model (LocalModel.cpp:143-160) for the public
 * parameter arrays, and LocalModel(ParamList, ModelName) (LocalModel.h:76-78)
 * when extra hidden parameters (the ionisation-gradient switch) are given.
 */
#include "LocalModel.h"
#include "ModelDatabase.h"

#include <cstdio>
#include <vector>

static ModelName model_from_id(int id) {
  switch (id) {
    case 0: return ModelName::relline;
    case 1: return ModelName::relconv;
    case 2: return ModelName::relxill;
    case 3: return ModelName::relxilllp;
    case 4: return ModelName::relline_lp;
    case 5: return ModelName::relconv_lp;
    case 6: return ModelName::xillver;
    case 7: return ModelName::xillverCp;
    case 8: return ModelName::relxillCp;
    case 9: return ModelName::relxilllpCp;
    default: return ModelName::relline;
  }
}

extern "C" int ref_eval(int model_id, const double *params, const double *energy, int n_flux, double *flux) {
  try {
    xspec_C_wrapper_eval_model(model_from_id(model_id), params, flux, n_flux, energy);
  } catch (std::exception &e) {
    std::printf("ref_eval: %s\n", e.what());
    return 1;
  }
  return 0;
}

/* relxilllp with the hidden ionisation-gradient switch (iongrad_type, iongrad_index) */
extern "C" int ref_eval_relxilllp_iongrad(const double *params, int iongrad_type, double iongrad_index,
                                          const double *energy, int n_flux, double *flux) {
  try {
    auto base = ModelDatabase::instance().param_list(ModelName::relxilllp);
    auto names = base.get_parnames();
    std::vector<double> vals;
    for (size_t i = 0; i < names.size(); i++) vals.push_back(params[i]);
    names.push_back(XPar::switch_iongrad_type);
    vals.push_back(iongrad_type);
    names.push_back(XPar::iongrad_index);
    vals.push_back(iongrad_index);
    LocalModel model{ParamList(names, vals), ModelName::relxilllp};
    XspecSpectrum spectrum{energy, flux, static_cast<size_t>(n_flux)};
    model.eval_model(spectrum);
  } catch (std::exception &e) {
    std::printf("ref_eval_relxilllp_iongrad: %s\n", e.what());
    return 1;
  }
  return 0;
}

/* Empty the reference's xillver spectrum cache (xilltable.c:30, data_storage)
 * so that the next evaluation behaves as the first one in a fresh process.
 * The rows are leaked on purpose: freeing them is the reference's job. */
extern "C" xillTable *cached_xill_tab;
extern "C" xillTable *cached_xill_tab_dens_nthcomp;
extern "C" void ref_reset_xillver_cache(void) {
  /* the full-output cache is keyed on the public parameters only
   * (Relcache.h:134-147), so hidden switches would hit it: empty it as well */
  RelxillCache::instance().empty();
  for (xillTable *t : {cached_xill_tab, cached_xill_tab_dens_nthcomp}) {
    if (t == nullptr) continue;
    for (int ii = 0; ii < t->num_elements; ii++) t->data_storage[ii] = nullptr;
  }
}
