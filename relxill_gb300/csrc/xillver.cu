// xillver.cu -- angle-resolved xillver interpolation per radial zone
// (check_xilltab_cache + interp_5d_tab_incl + calc_xillver_angdep and the
// normalisation change of the zone; xilltable.c:575-635, 812-876,
// Xillspec.cpp:557-573, Relxill.cpp:357-386).
//
// xill[z][E] = sum_corner sum_incl  w[corner][z] * dist[z][incl] * spec[corner][incl][E]
// where w holds the 4-D interpolation weight of the corner in zone z, the
// density division of the row and 1/normalisation-change of the zone, and
// dist is the zone's normalised emission-angle histogram.
//
// Launch: one CTA of 128 threads per (energy tile of 512 bins, parameter set),
// four CTAs per SM.  The corner list of a set is de-duplicated across zones by
// the setup kernel and holds only rows with a non-zero weight, so every table
// row a set needs is read once; sets are visited in table-row order
// (xill_order_kernel) so that sets sharing rows find them in L2.  The n_incl
// row segments of a corner (contiguous rows, incl is the fastest table index)
// are streamed into shared memory with cp.async.bulk (TMA bulk copies)
// completing on an mbarrier, two corners in flight per CTA (a third stage cost
// the fourth CTA per SM: 0.91 ms per 4096-set step against 0.78 with two); all
// waits are bounded and report a timeout through the error flag instead of
// hanging.
#include "relx_device.cuh"
#include "relx_tma.cuh"

namespace relx {

constexpr int kXillThreads = 128;
constexpr int kXillTile = 512;    // floats per row segment (2 KB), one float4 per thread
constexpr int kXillStages = 2;
static_assert(kXillTile == 4 * kXillThreads, "one float4 per thread");

// Self-test of the timeout path: one thread waits, with a short limit, on an mbarrier that
// expects 16 bytes no copy will deliver, and reports what the wait returned.  No copy is issued,
// so nothing is in flight when the CTA exits.
__global__ void wait_selftest_kernel(unsigned long long limit_ns, int *out) {
  __shared__ uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  mbar_expect_tx(&bar, 16);  // the arrival completes, the 16 transaction bytes never do
  *out = mbar_wait_bounded(&bar, 0, limit_ns) ? RELX_OK : RELX_ERR_TIMEOUT;
}

cudaError_t launch_wait_selftest(cudaStream_t s, unsigned long long limit_ns, int *out) {
  wait_selftest_kernel<<<1, 32, 0, s>>>(limit_ns, out);
  return cudaGetLastError();
}

template <int NZ>
struct XillSmem {
  uint64_t full[kXillStages];
  float w[RELX_MAX_UCORNER][NZ];        // corner weight per zone
  float dist[NZ][RELX_MAX_INCL];        // normalised emission-angle distribution per zone
  int row[RELX_MAX_UCORNER];
  int abort_flag;
  int pad_[3];
  float4 stage[1];  // [kXillStages][n_incl][kXillTile/4], dynamic tail
};

// Order in which the xillver kernel visits the sets: sets whose zones use the same table rows run
// next to each other, so that a row read from HBM by one set is found in L2 by the next.  Key: the
// first corner row of the set (table order).  Sorted in chunks of kOrderN sets (bitonic sort in
// shared memory); the results do not depend on the order.
constexpr int kOrderN = 4096;
constexpr int kOrderThreads = 1024;
__global__ void __launch_bounds__(kOrderThreads) xill_order_kernel(const RelxSetState *__restrict__ sst,
                                                                   const RelxCorners *__restrict__ scor,
                                                                   const RelxZoneCorners *__restrict__ zcor,
                                                                   int n_sets, int *__restrict__ order) {
  __shared__ unsigned long long key[kOrderN];
  const int base = blockIdx.x * kOrderN;
  const int n = min(kOrderN, n_sets - base);
  for (int i = threadIdx.x; i < kOrderN; i += kOrderThreads) {
    unsigned long long k = ~0ull;
    if (i < n) {
      const int set = base + i;
      const RelxSetState &s = sst[set];
      unsigned int r = 0xffffffffu;
      if (s.status == RELX_OK && s.model >= RELX_RELXILL) {
        if (s.xdense) {
          if (s.ucount > 0) r = (unsigned int) scor[set].row[0];
        } else if (zcor) {
          r = (unsigned int) zcor[set].row[0][0];
        }
      }
      k = ((unsigned long long) r << 32) | (unsigned int) set;
    }
    key[i] = k;
  }
  __syncthreads();
  for (int size = 2; size <= kOrderN; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < kOrderN / 2; i += kOrderThreads) {
        const int lo = 2 * i - (i & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const unsigned long long a = key[lo], b = key[hi];
        if ((a > b) == up) { key[lo] = b; key[hi] = a; }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < n; i += kOrderThreads) order[base + i] = (int) (key[i] & 0xffffffffull);
}

void launch_xill_order(cudaStream_t s, const RelxSetState *sst, const RelxCorners *cor, const RelxZoneCorners *zcor,
                       int n_sets, int *order) {
  xill_order_kernel<<<(n_sets + kOrderN - 1) / kOrderN, kOrderThreads, 0, s>>>(sst, cor, zcor, n_sets, order);
}

// NZ: zones held in registers (a set with more zones runs in a wider instance);
// NI: inclinations unrolled at compile time (0: any count up to RELX_MAX_INCL).
template <int NZ, int NI>
__global__ void __launch_bounds__(kXillThreads, 4) xillver_dense_kernel(RelxTables tab, const RelxSetState *__restrict__ sst,
                                                                        const RelxCorners *__restrict__ scor,
                                                                        const float *__restrict__ dist_raw, int nza,
                                                                        float *__restrict__ xout, int *__restrict__ err,
                                                                        const int *__restrict__ order) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  XillSmem<NZ> &m = *reinterpret_cast<XillSmem<NZ> *>(smem_raw);
  const int set = order ? order[blockIdx.y] : blockIdx.y, tile = blockIdx.x;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.model < RELX_RELXILL || !s.xdense || s.nz > NZ) return;
  constexpr int NIU = NI > 0 ? NI : RELX_MAX_INCL;
  const int tid = threadIdx.x;
  const int nz = s.nz, U = s.ucount, ni = NI > 0 ? NI : tab.x_nincl;
  const int pitch = tab.x_cpad;  // table rows on the conv grid
  const int e0 = tile * kXillTile;
  if (e0 >= pitch) return;
  const int len = min(kXillTile, pitch - e0);  // multiple of 4 floats (16 bytes)
  const uint32_t bytes_row = (uint32_t) len * 4u;

  // weights and normalised emission-angle distributions (renorm_relline_profile, Relprofile.cpp:783-795)
  const RelxCorners &C = scor[set];
  for (int i = tid; i < U * NZ; i += kXillThreads) {
    const int u = i / NZ, z = i - u * NZ;
    m.w[u][z] = (z < nz) ? C.w[u][z] : 0.0f;
  }
  for (int i = tid; i < U; i += kXillThreads) m.row[i] = C.row[i];
  if (tid < nz) {
    const float *d = dist_raw + ((size_t) set * nza + tid) * RELX_MAX_INCL;
    float sum = 0.0f;
    for (int i = 0; i < ni; i++) sum += d[i];
    for (int i = 0; i < ni; i++) m.dist[tid][i] = (sum > 1e-8f) ? d[i] / sum : 0.0f;
  }
  if (tid == 0) {
    m.abort_flag = 0;
    for (int st = 0; st < kXillStages; st++) mbar_init(&m.full[st], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int u) {
    const int st = u % kXillStages;
    mbar_expect_tx(&m.full[st], bytes_row * (uint32_t) ni);
    const float *src = tab.x_cspec + (size_t) m.row[u] * pitch + e0;
    for (int i = 0; i < ni; i++)
      bulk_g2s(&m.stage[(st * ni + i) * (kXillTile / 4)], src + (size_t) i * pitch, bytes_row, &m.full[st]);
  };
  int issued = 0;  // meaningful in thread 0 only
  if (tid == 0)
    for (int u = 0; u < min(U, kXillStages); u++) { issue(u); issued = u + 1; }

  float4 acc[NZ];
#pragma unroll
  for (int z = 0; z < NZ; z++) acc[z] = make_float4(0.f, 0.f, 0.f, 0.f);
  const int q = tid;  // float4 index inside the tile
  const bool active = q * 4 < len;
  int u_stop = U;
  for (int u = 0; u < U; u++) {
    const int st = u % kXillStages;
    const uint32_t parity = (uint32_t) ((u / kXillStages) & 1);
    if (!mbar_wait_bounded(&m.full[st], parity)) atomicExch(&m.abort_flag, 1);
    __syncthreads();
    if (m.abort_flag) { u_stop = u; break; }
    if (active) {
      float4 v[NIU];
#pragma unroll
      for (int i = 0; i < NIU; i++)
        if (i < ni) v[i] = m.stage[(st * ni + i) * (kXillTile / 4) + q];
#pragma unroll
      for (int z = 0; z < NZ; z++) {
        const float wz = m.w[u][z];
        if (wz != 0.0f) {
          float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int i = 0; i < NIU; i++) {
            if (i < ni) {
              const float d = m.dist[z][i];
              t.x += d * v[i].x; t.y += d * v[i].y; t.z += d * v[i].z; t.w += d * v[i].w;
            }
          }
          acc[z].x += wz * t.x; acc[z].y += wz * t.y; acc[z].z += wz * t.z; acc[z].w += wz * t.w;
        }
      }
    }
    __syncthreads();  // stage st is free again
    if (tid == 0 && u + kXillStages < U) { issue(u + kXillStages); issued = u + kXillStages + 1; }
  }
  if (m.abort_flag) {
    // wait (bounded) for the copies this CTA still has in flight, then report
    if (tid == 0) {
      for (int u = u_stop; u < issued; u++)
        (void) mbar_wait_bounded(&m.full[u % kXillStages], (uint32_t) ((u / kXillStages) & 1));
      atomicExch(err, RELX_ERR_TIMEOUT);
    }
    return;
  }
  if (active) {
#pragma unroll
    for (int z = 0; z < NZ; z++) {
      if (z < nz) {
        float4 *o = reinterpret_cast<float4 *>(xout + ((size_t) set * nza + z) * pitch + e0) + q;
        *o = acc[z];
      }
    }
  }
}

template <int NZ>
static size_t xill_smem_nz(int n_incl) {
  return sizeof(XillSmem<NZ>) + sizeof(float4) * ((size_t) kXillStages * n_incl * (kXillTile / 4) - 1);
}

// generic path for the sets without the de-duplicated corner list (more than RELX_ZDENSE zones, or
// more distinct rows than RELX_MAX_UCORNER): 16 or 32 corners per zone, plain loads
__global__ void __launch_bounds__(kXillThreads) xillver_zone_kernel(RelxTables tab, const RelxSetState *__restrict__ sst,
                                                                    const RelxZoneCorners *__restrict__ zcor,
                                                                    const float *__restrict__ dist_raw, int nza,
                                                                    float *__restrict__ xout) {
  const int set = blockIdx.y, tile = blockIdx.x;
  const RelxSetState &s = sst[set];
  if (s.status != RELX_OK || s.model < RELX_RELXILL || s.xdense) return;
  const int ncz = tab.x_npar == 6 ? 32 : 16;  // corners per zone (16, or 32 for the 6-parameter table)
  __shared__ float dist[RELX_MAX_INCL];
  const int tid = threadIdx.x, ni = tab.x_nincl, pitch = tab.x_cpad;  // table rows on the conv grid
  const int e0 = tile * kXillTile;
  if (e0 >= pitch) return;
  const int len = min(kXillTile, pitch - e0);
  const int q = tid;
  const bool active = q * 4 < len;
  for (int z = 0; z < s.nz; z++) {
    __syncthreads();
    if (tid == 0) {
      const float *d = dist_raw + ((size_t) set * nza + z) * RELX_MAX_INCL;
      float sum = 0.0f;
      for (int i = 0; i < ni; i++) sum += d[i];
      for (int i = 0; i < ni; i++) dist[i] = (sum > 1e-8f) ? d[i] / sum : 0.0f;
    }
    __syncthreads();
    if (!active) continue;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int c = 0; c < ncz; c++) {
      const float wz = zcor[set].w[z][c];
      if (wz == 0.0f) continue;  // zero weight: the row adds exactly nothing
      const float4 *src = reinterpret_cast<const float4 *>(tab.x_cspec + (size_t) zcor[set].row[z][c] * pitch + e0) + q;
      float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int i = 0; i < ni; i++) {
        float4 v = __ldg(src + (size_t) i * (pitch / 4));
        t.x += dist[i] * v.x; t.y += dist[i] * v.y; t.z += dist[i] * v.z; t.w += dist[i] * v.w;
      }
      acc.x += wz * t.x; acc.y += wz * t.y; acc.z += wz * t.z; acc.w += wz * t.w;
    }
    reinterpret_cast<float4 *>(xout + ((size_t) set * nza + z) * pitch + e0)[q] = acc;
  }
}

#define RELX_XILL_INSTANCES(X) X(1, 10) X(10, 10) X(16, 10) X(1, 0) X(10, 0) X(16, 0)

cudaError_t xillver_set_smem(int n_incl) {
#define X(nz, ni)                                                                                   \
  {                                                                                                 \
    cudaError_t e = cudaFuncSetAttribute(xillver_dense_kernel<nz, ni>,                              \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,               \
                                         (int) xill_smem_nz<nz>(n_incl));                           \
    if (e != cudaSuccess) return e;                                                                 \
  }
  RELX_XILL_INSTANCES(X)
#undef X
  return cudaSuccess;
}

// xillver stage of a batch: the dense kernel (instance by the batch's zone count and the table's
// inclination count) for the sets with the de-duplicated corner list, the zone kernel for the others.
// zone: some set may need the zone kernel; dense: some set may use the dense kernel.
cudaError_t launch_xillver(cudaStream_t s, const RelxTables &tab, int n_sets, int nza, bool zone, bool dense,
                           const RelxSetState *sst, const RelxCorners *cor, const RelxZoneCorners *zcor,
                           const float *dist, float *xout, int *err, const int *order) {
  const dim3 grid((tab.x_cpad + kXillTile - 1) / kXillTile, n_sets);
  if (zone) xillver_zone_kernel<<<grid, kXillThreads, 0, s>>>(tab, sst, zcor, dist, nza, xout);
  if (!dense) return cudaGetLastError();
  const int nzk = nza <= 1 ? 1 : (nza <= 10 ? 10 : 16);
  const int nik = tab.x_nincl == 10 ? 10 : 0;
#define X(nz, ni)                                                                                           \
  if (nzk == nz && nik == ni)                                                                               \
    xillver_dense_kernel<nz, ni><<<grid, kXillThreads, xill_smem_nz<nz>(tab.x_nincl), s>>>(tab, sst, cor, dist, \
                                                                                         nza, xout, err, order);
  RELX_XILL_INSTANCES(X)
#undef X
  return cudaGetLastError();
}

}  // namespace relx
