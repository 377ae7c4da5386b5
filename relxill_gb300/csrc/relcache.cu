// relcache.cu -- device-resident cache of relativistic line profiles, the
// counterpart of the reference's relbase cache (Relcache.cpp:311-331,
// Relbase.cpp:461-538), which keeps the line profile of recent relativistic
// parameters so that a change of the xillver parameters alone skips the
// ray-tracing stage.
//
// Key: the model, the zone count and the model's relativistic parameters
// (the parameters did_rel_param_change compares, Relcache.cpp:40-130; for the
// lamp post this includes Gamma, which enters the source-to-disk flux boost,
// Rellp.cpp:249-253).  Value: the per-zone line profile over the set's
// profile window, the per-(tile, zone) profile sums and the per-zone
// emission-angle histograms.  The value is computed by the same kernels as an
// uncached set, so a reused profile is the same number as a recomputed one.
//
// Direct mapped: a key hashes to one slot.  Within a batch a slot is claimed
// by the lowest-numbered missing set that maps to it, and only that set
// stores its result; everything else is stream ordered (lookup after setup,
// fill before the line kernels, store after them).
#include "relcache.h"
#include "relx_device.cuh"

namespace relx {

__device__ __forceinline__ bool cache_key(const RelxSetIn &in, const RelxSetState &s, double *key) {
  // sets whose emissivity holds returning radiation corrected by their xillver spectra depend on
  // the xillver parameters too and are not cached (the reference does not cache them either,
  // Relcache.cpp:93-97)
  if (s.status != RELX_OK || s.model == RELX_RELLINE || s.nz > kCacheZones || s.rr_corr) return false;
#pragma unroll
  for (int q = 0; q < kCacheKeyLen; q++) key[q] = 0.0;
  key[0] = (double) s.pmodel;
  key[1] = (double) s.nz;
  // relconv: Index1..limb (8); relconv_lp: h..gamma (8) and the returning-radiation switch;
  // relxill: Index1..z (8); relxilllp: h..gamma (8) and the returning-radiation switch
  // (lmodel_relxill_public.dat:13-21, 35-44, 46-59, 61-75)
#pragma unroll
  for (int q = 0; q < 8; q++) key[2 + q] = in.p[q];
  if (s.pmodel == RELX_RELXILLLP) key[10] = in.p[12];
  if (s.pmodel == RELX_RELCONVLP) key[10] = in.p[8];
  if (s.pmodel == RELX_RELXILLLPCP) key[10] = in.p[15];  // Incl..logxi (8) and the switch (:112-129)
  return true;
}

// FNV-1a over the key's 64-bit words, then the MurmurHash3 64-bit finaliser.  Parameters with
// short binary fractions (integers, halves) differ only in the high bits of their doubles, and a
// multiply carries bits upwards only: without the finaliser such keys share their low (slot) bits.
__device__ __forceinline__ unsigned long long key_hash(const double *key) {
  unsigned long long h = 1469598103934665603ull;
  for (int q = 0; q < kCacheKeyLen; q++) {
    h ^= (unsigned long long) __double_as_longlong(key[q]);
    h *= 1099511628211ull;
  }
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h;
}

__global__ void cache_lookup_kernel(RelCacheDev c, const RelxSetIn *__restrict__ sin, RelxSetState *__restrict__ sst,
                                    int n_sets, int *__restrict__ slot_of) {
  const int set = blockIdx.x * blockDim.x + threadIdx.x;
  if (set >= n_sets) return;
  double key[kCacheKeyLen];
  RelxSetState &s = sst[set];
  if (!cache_key(sin[set], s, key)) {
    slot_of[set] = -1;
    return;
  }
  const int slot = (int) (key_hash(key) & (unsigned long long) (c.n_slots - 1));
  slot_of[set] = slot;
  bool same = c.valid[slot] != 0;
  for (int q = 0; q < kCacheKeyLen && same; q++) same = c.keys[(size_t) slot * kCacheKeyLen + q] == key[q];
  atomicAdd(&c.counters[0], 1ull);
  if (same) {
    s.cached = 1;
    atomicAdd(&c.counters[1], 1ull);
  } else {
    atomicMin(&c.claim[slot], set);
  }
}

// copy a cached entry into the batch's profile, tile-sum and histogram arrays
__global__ void cache_fill_kernel(RelCacheDev c, const RelxSetState *__restrict__ sst, const int *__restrict__ slot_of,
                                  int nza, int ntile_max, int tile_bins, float *__restrict__ prof,
                                  double *__restrict__ tsum, float *__restrict__ dist) {
  const int set = blockIdx.x;
  const RelxSetState &s = sst[set];
  if (!s.cached) return;
  const int slot = slot_of[set];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int wlo = s.win_lo, whi = s.win_hi;
  for (int z = 0; z < s.nz; z++) {
    const float *src = c.prof + ((size_t) slot * kCacheZones + z) * RELX_NCONV;
    float *dst = prof + ((size_t) set * nza + z) * RELX_NCONV;
    for (int j = wlo + tid; j < whi; j += nt) dst[j] = src[j];
  }
  const int ntiles = (whi - wlo + tile_bins - 1) / tile_bins;
  for (int i = tid; i < ntiles * s.nz; i += nt) {
    const int t = i / s.nz, z = i - t * s.nz;
    tsum[((size_t) set * ntile_max + t) * nza + z] = c.tsum[((size_t) slot * kCacheTiles + t) * kCacheZones + z];
  }
  for (int i = tid; i < s.nz * RELX_MAX_INCL; i += nt)
    dist[(size_t) set * nza * RELX_MAX_INCL + i] = c.dist[(size_t) slot * kCacheZones * RELX_MAX_INCL + i];
}

// store the results of the sets that claimed their slot
__global__ void cache_store_kernel(RelCacheDev c, const RelxSetIn *__restrict__ sin,
                                   const RelxSetState *__restrict__ sst, const int *__restrict__ slot_of, int nza,
                                   int ntile_max, int tile_bins, const float *__restrict__ prof,
                                   const double *__restrict__ tsum, const float *__restrict__ dist) {
  const int set = blockIdx.x;
  const RelxSetState &s = sst[set];
  const int slot = slot_of[set];
  if (slot < 0 || s.cached || s.status != RELX_OK || c.claim[slot] != set) return;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int wlo = s.win_lo, whi = s.win_hi;
  for (int z = 0; z < s.nz; z++) {
    const float *src = prof + ((size_t) set * nza + z) * RELX_NCONV;
    float *dst = c.prof + ((size_t) slot * kCacheZones + z) * RELX_NCONV;
    for (int j = wlo + tid; j < whi; j += nt) dst[j] = src[j];
  }
  const int ntiles = (whi - wlo + tile_bins - 1) / tile_bins;
  for (int i = tid; i < ntiles * s.nz; i += nt) {
    const int t = i / s.nz, z = i - t * s.nz;
    c.tsum[((size_t) slot * kCacheTiles + t) * kCacheZones + z] = tsum[((size_t) set * ntile_max + t) * nza + z];
  }
  const bool has_dist = relx_is_relxill(s.model);
  for (int i = tid; i < s.nz * RELX_MAX_INCL; i += nt)
    c.dist[(size_t) slot * kCacheZones * RELX_MAX_INCL + i] = has_dist ? dist[(size_t) set * nza * RELX_MAX_INCL + i] : 0.0f;
  if (tid == 0) {
    double key[kCacheKeyLen];
    cache_key(sin[set], s, key);
    for (int q = 0; q < kCacheKeyLen; q++) c.keys[(size_t) slot * kCacheKeyLen + q] = key[q];
    c.valid[slot] = 1;
  }
}

// ---- host side ----------------------------------------------------------------
static size_t cache_bytes_per_slot() {
  return sizeof(double) * kCacheKeyLen + 2 * sizeof(int) + sizeof(float) * (size_t) kCacheZones * RELX_NCONV +
         sizeof(double) * kCacheTiles * kCacheZones + sizeof(float) * kCacheZones * RELX_MAX_INCL;
}

int RelCache::create(int slots) {
  release();
  int n = 1;
  while (n < slots) n <<= 1;
  const size_t per = cache_bytes_per_slot();
  if (cudaMalloc(&base, per * (size_t) n + 8 * 256) != cudaSuccess) {
    cudaGetLastError();
    base = nullptr;
    return RELX_ERR_NOMEM;
  }
  bytes = per * (size_t) n + 8 * 256;
  unsigned char *p = (unsigned char *) base;
  auto take = [&](size_t b) {
    unsigned char *q = p;
    p += (b + 255) / 256 * 256;
    return q;
  };
  d.n_slots = n;
  d.keys = (double *) take(sizeof(double) * kCacheKeyLen * (size_t) n);
  d.valid = (int *) take(sizeof(int) * (size_t) n);
  d.claim = (int *) take(sizeof(int) * (size_t) n);
  d.prof = (float *) take(sizeof(float) * (size_t) kCacheZones * RELX_NCONV * n);
  d.tsum = (double *) take(sizeof(double) * kCacheTiles * kCacheZones * (size_t) n);
  d.dist = (float *) take(sizeof(float) * kCacheZones * RELX_MAX_INCL * (size_t) n);
  d.counters = (unsigned long long *) take(2 * sizeof(unsigned long long));
  if (cudaMemset(d.valid, 0, sizeof(int) * (size_t) n) != cudaSuccess ||
      cudaMemset(d.counters, 0, 2 * sizeof(unsigned long long)) != cudaSuccess)
    return RELX_ERR_CUDA;
  return 0;
}

void RelCache::release() {
  if (base) cudaFree(base);
  base = nullptr;
  bytes = 0;
  d = RelCacheDev{};
}

cudaError_t RelCache::clear(cudaStream_t s) {
  if (!base) return cudaSuccess;
  return cudaMemsetAsync(d.valid, 0, sizeof(int) * (size_t) d.n_slots, s);
}

cudaError_t cache_lookup(const RelCache &c, cudaStream_t s, const RelxSetIn *sin, RelxSetState *sst, int n_sets,
                         int *slot_of) {
  cudaError_t e = cudaMemsetAsync(c.d.claim, 0x7f, sizeof(int) * (size_t) c.d.n_slots, s);
  if (e != cudaSuccess) return e;
  cache_lookup_kernel<<<(n_sets + 127) / 128, 128, 0, s>>>(c.d, sin, sst, n_sets, slot_of);
  return cudaGetLastError();
}

cudaError_t cache_fill(const RelCache &c, cudaStream_t s, const RelxSetState *sst, const int *slot_of, int n_sets,
                       int nza, int ntile_max, int tile_bins, float *prof, double *tsum, float *dist) {
  cache_fill_kernel<<<n_sets, 256, 0, s>>>(c.d, sst, slot_of, nza, ntile_max, tile_bins, prof, tsum, dist);
  return cudaGetLastError();
}

cudaError_t cache_store(const RelCache &c, cudaStream_t s, const RelxSetIn *sin, const RelxSetState *sst,
                        const int *slot_of, int n_sets, int nza, int ntile_max, int tile_bins, const float *prof,
                        const double *tsum, const float *dist) {
  cache_store_kernel<<<n_sets, 256, 0, s>>>(c.d, sin, sst, slot_of, nza, ntile_max, tile_bins, prof, tsum, dist);
  return cudaGetLastError();
}

}  // namespace relx
