// relcache.h -- device-resident line-profile cache (relcache.cu).
#pragma once
#include <cuda_runtime.h>

#include "relx_common.h"

namespace relx {

constexpr int kCacheKeyLen = 12;
constexpr int kCacheZones = RELX_ZDENSE;       // zones per entry (sets with more zones are not cached)
constexpr int kCacheTiles = RELX_NCONV / 256;  // 256-bin profile-sum blocks over the conv grid

struct RelCacheDev {
  int n_slots = 0;        // power of two
  double *keys = nullptr; // [n_slots][kCacheKeyLen]
  int *valid = nullptr;   // [n_slots]
  int *claim = nullptr;   // [n_slots] lowest missing set of the current batch mapping to the slot
  float *prof = nullptr;  // [n_slots][kCacheZones][RELX_NCONV] (the set's profile window is used)
  double *tsum = nullptr; // [n_slots][kCacheTiles][kCacheZones] profile sums per 256-bin block
  float *dist = nullptr;  // [n_slots][kCacheZones][RELX_MAX_INCL]
  unsigned long long *counters = nullptr;  // [0] lookups, [1] hits
};

struct RelCache {
  RelCacheDev d;
  void *base = nullptr;
  size_t bytes = 0;
  int create(int slots);  // rounds up to a power of two; 0 or RELX_ERR_NOMEM
  void release();
  cudaError_t clear(cudaStream_t s);
  bool enabled() const { return base != nullptr; }
};

// stream-ordered steps of a batch: lookup after setup (marks hits in the set state), fill before
// the line kernels, store after them
cudaError_t cache_lookup(const RelCache &c, cudaStream_t s, const RelxSetIn *sin, RelxSetState *sst, int n_sets,
                         int *slot_of);
cudaError_t cache_fill(const RelCache &c, cudaStream_t s, const RelxSetState *sst, const int *slot_of, int n_sets,
                       int nza, int ntile_max, int tile_bins, float *prof, double *tsum, float *dist);
cudaError_t cache_store(const RelCache &c, cudaStream_t s, const RelxSetIn *sin, const RelxSetState *sst,
                        const int *slot_of, int n_sets, int nza, int ntile_max, int tile_bins, const float *prof,
                        const double *tsum, const float *dist);

}  // namespace relx
