// runtime.cu -- host runtime of the relxill GB300 path: table loading and
// upload, device workspace, the kernel sequence of one batch, and the C ABI
// (include/relxill_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

#include "../../include/relxill_gb300.h"
#include "fits_reader.h"
#include "relx_common.h"
#include "relx_kernels.h"
#include "relx_runtime.h"
#include "relcache.h"

namespace relx {

static thread_local std::string g_errmsg;
static std::atomic<int> g_last_status{0};

#define RELX_CUDA(call)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      g_errmsg = std::string(#call) + ": " + cudaGetErrorString(e_);                       \
      return RELX_ERR_CUDA;                                                               \
    }                                                                                     \
  } while (0)

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
// a device region the buffers of one batch are carved from (the workspaces of the serving slots):
// carving is a bump of an offset, and the offset returns to 0 before each batch
struct Arena {
  unsigned char *base = nullptr;
  size_t bytes = 0, off = 0;
};

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  Arena *ar = nullptr;  // carve from this region instead of allocating
  int reserve(size_t n) {
    if (n <= bytes) return 0;
    if (ar) {
      const size_t want = (std::max(n, (size_t) 256) + 255) / 256 * 256;
      if (ar->off + want > ar->bytes) {
        g_errmsg = "batch needs more than the slot's " + std::to_string(ar->bytes) + " device bytes";
        return RELX_ERR_NOMEM;
      }
      p = ar->base + ar->off;
      bytes = want;
      ar->off += want;
      return 0;
    }
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    size_t want = std::max(n, (size_t) 256);
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      g_errmsg = "cudaMalloc of " + std::to_string(want) + " bytes failed";
      return RELX_ERR_NOMEM;
    }
    bytes = want;
    return 0;
  }
  template <typename T>
  T *as() const { return reinterpret_cast<T *>(p); }
  void release() {
    if (p && !ar) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

// page-locked host staging buffer (grown on demand, by at least half its size)
struct Pinned {
  void *h = nullptr;
  size_t bytes = 0;
  int reserve(size_t n) {
    if (n <= bytes) return 0;
    const size_t want = std::max(n, bytes + bytes / 2);
    if (h) cudaFreeHost(h);
    h = nullptr;
    bytes = 0;
    if (cudaMallocHost(&h, want) != cudaSuccess) {
      cudaGetLastError();
      g_errmsg = "cudaMallocHost of " + std::to_string(want) + " bytes failed";
      return RELX_ERR_NOMEM;
    }
    bytes = want;
    return 0;
  }
  void release() {
    if (h) cudaFreeHost(h);
    h = nullptr;
    bytes = 0;
  }
};

// Host copies to and from pinned staging, split over a few worker threads: one thread copies at
// a fraction of the host's memory bandwidth, and a batch of 4096 spectra moves about 90 MB of
// energy edges in and as much flux out.  Jobs of concurrent callers run one after the other.
struct CopyPiece {
  void *dst;
  const void *src;
  size_t n;
};
class CopyPool {
 public:
  static CopyPool &get() {
    static CopyPool *p = new CopyPool();  // workers live for the process
    return *p;
  }
  // performs every copy of `jobs`, pieces of at most kPiece bytes spread over the workers and the caller
  void run(const std::vector<CopyPiece> &jobs) {
    size_t total = 0;
    for (const auto &j : jobs) total += j.n;
    // serial in a process forked after the workers started (it has no worker threads)
    if (nthreads_ == 0 || total < kMinParallel || getpid() != pid_) {
      for (const auto &j : jobs)
        if (j.n) std::memcpy(j.dst, j.src, j.n);
      return;
    }
    std::lock_guard<std::mutex> one(call_mu_);  // one job at a time
    std::unique_lock<std::mutex> lk(mu_);      // no worker is inside a job here (active_ == 0)
    pieces_.clear();
    for (const auto &j : jobs)
      for (size_t o = 0; o < j.n; o += kPiece)
        pieces_.push_back({(unsigned char *) j.dst + o, (const unsigned char *) j.src + o, std::min(kPiece, j.n - o)});
    next_.store(0);
    remaining_ = pieces_.size();
    open_ = true;
    ++gen_;
    lk.unlock();
    cv_.notify_all();
    work();
    lk.lock();
    done_cv_.wait(lk, [&] { return remaining_ == 0; });
    open_ = false;  // late workers skip this job; wait for those still inside it
    done_cv_.wait(lk, [&] { return active_ == 0; });
  }

 private:
  static constexpr size_t kPiece = 1 << 20, kMinParallel = 4 << 20;
  CopyPool() {
    const char *e = std::getenv("RELX_COPY_THREADS");
    unsigned hc = std::thread::hardware_concurrency();
    int n = e ? std::atoi(e) : (int) std::min(12u, hc > 1 ? hc - hc / 4 : 0u);
    nthreads_ = std::max(0, std::min(n, 32));
    pid_ = getpid();
    for (int i = 0; i < nthreads_; i++) std::thread([this] { loop(); }).detach();
  }
  void work() {
    size_t done = 0;
    for (;;) {
      const size_t i = next_.fetch_add(1);
      if (i >= pieces_.size()) break;
      std::memcpy(pieces_[i].dst, pieces_[i].src, pieces_[i].n);
      done++;
    }
    if (done) {
      std::lock_guard<std::mutex> g(mu_);
      remaining_ -= done;
      if (remaining_ == 0) done_cv_.notify_all();
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (!open_) continue;
        active_++;
      }
      work();
      std::lock_guard<std::mutex> g(mu_);
      if (--active_ == 0) done_cv_.notify_all();
    }
  }
  int nthreads_ = 0;
  pid_t pid_ = 0;
  std::mutex call_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  std::vector<CopyPiece> pieces_;
  std::atomic<size_t> next_{0};
  size_t remaining_ = 0;
  int active_ = 0;
  bool open_ = false;
  uint64_t gen_ = 0;
};

template <typename T>
static int upload(DevBuf &b, const std::vector<T> &v) {
  int st = b.reserve(sizeof(T) * std::max<size_t>(v.size(), 1));
  if (st) return st;
  if (!v.empty()) RELX_CUDA(cudaMemcpy(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return 0;
}

// ---------------------------------------------------------------------------
// tables
// ---------------------------------------------------------------------------
struct Tables {
  RelxTables d{};
  DevBuf rel_a, rel_mu0, rel_r, rel_gmin, rel_gmax, rel_tc;
  DevBuf lp_a, lp_h, lp_rad, lp_intens, lp_del, lp_delinc;
  // one xillver table: the standard one (x) and the nthcomp one of the Cp models (xcp)
  struct XillBufs {
    DevBuf vals, spec, e, ew, fcorr, rb_imin, rb_imax, rb_fmin, rb_fmax, rb_pack, cspec;
    void release() {
      for (DevBuf *b : {&vals, &spec, &e, &ew, &fcorr, &rb_imin, &rb_imax, &rb_fmin, &rb_fmax, &rb_pack, &cspec})
        b->release();
    }
  } x, xcp;
  RelxTables dcp{};     // d with the xillver fields of the nthcomp table (valid if has_cp)
  bool has_cp = false;
  DevBuf rr_spin, rr_rlo, rr_rhi, rr_tfr, rr_g;
  DevBuf conv_e, conv_eff, conv_inv_emid, conv_cf, conv_cw, coarse_e, coarse_t, nth_grid;
  size_t bytes_total = 0;
  bool loaded = false;
  void release() {
    for (DevBuf *b : {&rel_a, &rel_mu0, &rel_r, &rel_gmin, &rel_gmax, &rel_tc, &lp_a, &lp_h, &lp_rad, &lp_intens,
                      &lp_del, &lp_delinc, &rr_spin, &rr_rlo, &rr_rhi, &rr_tfr, &rr_g, &conv_e, &conv_eff, &conv_inv_emid, &conv_cf,
                      &conv_cw, &coarse_e, &coarse_t, &nth_grid})
      b->release();
    x.release();
    xcp.release();
    has_cp = false;
    loaded = false;
  }
};

static void log_grid(std::vector<double> &e, int n, double emin, double emax) {
  // get_log_grid, relutility.c:399-405
  e.resize(n);
  for (int ii = 0; ii < n; ii++) e[ii] = std::exp(1.0 * ii / (n - 1) * (std::log(emax) - std::log(emin)) + std::log(emin));
}

static int load_relline(const std::string &dir, Tables &T) {
  FitsFile f;
  std::string err;
  if (!f.open(dir + "/rel_table_v0.5a.fits", &err)) { g_errmsg = err; return RELX_ERR_NOTABLE; }
  const FitsHdu *ha = f.find("a"), *hm = f.find("mu0");
  if (!ha || !hm) { g_errmsg = "relline table: missing a/mu0 extensions"; return RELX_ERR_TABLE; }
  int na = (int) ha->nrows, nm = (int) hm->nrows;
  std::vector<float> a(na), mu0(nm);
  f.read_f32(*ha, ha->col("a"), 0, na, a.data());
  f.read_f32(*hm, hm->col("mu0"), 0, nm, mu0.data());
  const auto &H = f.hdus();
  if ((int) H.size() < na * nm + 3) { g_errmsg = "relline table: too few extensions"; return RELX_ERR_TABLE; }
  const FitsHdu &h0 = H[3];
  int nr = (int) h0.nrows, ng = (int) h0.cols[h0.col("trff1")].repeat;
  if (nr > RELX_MAX_NRTAB || ng > RELX_MAX_NG || nr < 2 || ng < 3) {
    g_errmsg = "relline table dimensions exceed the kernel limits";
    return RELX_ERR_TABLE;
  }
  std::vector<float> r((size_t) na * nm * nr), gmin(r.size()), gmax(r.size());
  std::vector<float4> tc((size_t) na * nm * nr * ng);
  std::vector<float> t1((size_t) nr * ng), t2(t1.size()), c1(t1.size()), c2(t1.size());
  for (int ii = 0; ii < na; ii++) {
    for (int jj = 0; jj < nm; jj++) {
      const FitsHdu &h = H[ii * nm + jj + 3];  // HDU number ii*n_mu0+jj+4 (reltable.c:290)
      if (h.nrows != nr) { g_errmsg = "relline table: inconsistent rows"; return RELX_ERR_TABLE; }
      size_t b = (size_t) ii * nm + jj;
      std::vector<unsigned char> raw((size_t) (nr * h.width));
      bool ok = f.read_rows(h, 0, nr, raw.data()) && decode_f32(h, h.col("r"), raw.data(), nr, &r[b * nr]) &&
                decode_f32(h, h.col("gmin"), raw.data(), nr, &gmin[b * nr]) &&
                decode_f32(h, h.col("gmax"), raw.data(), nr, &gmax[b * nr]) &&
                decode_f32(h, h.col("trff1"), raw.data(), nr, t1.data()) &&
                decode_f32(h, h.col("trff2"), raw.data(), nr, t2.data()) &&
                decode_f32(h, h.col("cosne1"), raw.data(), nr, c1.data()) &&
                decode_f32(h, h.col("cosne2"), raw.data(), nr, c2.data());
      if (!ok) { g_errmsg = "relline table: read failed"; return RELX_ERR_TABLE; }
      for (int q = 0; q < nr * ng; q++) tc[b * nr * ng + q] = make_float4(t1[q], t2[q], c1[q], c2[q]);
    }
  }
  int st;
  if ((st = upload(T.rel_a, a)) || (st = upload(T.rel_mu0, mu0)) || (st = upload(T.rel_r, r)) ||
      (st = upload(T.rel_gmin, gmin)) || (st = upload(T.rel_gmax, gmax)) || (st = upload(T.rel_tc, tc)))
    return st;
  T.d.rel_na = na; T.d.rel_nmu0 = nm; T.d.rel_nr = nr; T.d.rel_ng = ng;
  T.d.rel_a = T.rel_a.as<float>(); T.d.rel_mu0 = T.rel_mu0.as<float>();
  T.d.rel_r = T.rel_r.as<float>(); T.d.rel_gmin = T.rel_gmin.as<float>(); T.d.rel_gmax = T.rel_gmax.as<float>();
  T.d.rel_tc = T.rel_tc.as<float4>();
  T.bytes_total += r.size() * 12 + tc.size() * 16;
  return 0;
}

static int load_lp(const std::string &dir, Tables &T) {
  FitsFile f;
  std::string err;
  if (!f.open(dir + "/rel_lp_table_v0.5b.fits", &err)) { g_errmsg = err; return RELX_ERR_NOTABLE; }
  const FitsHdu *h = f.find("I_h");
  if (!h) { g_errmsg = "lamp-post table: missing I_h"; return RELX_ERR_TABLE; }
  int na = (int) h->nrows;
  int nh = (int) h->cols[h->col("hgrid")].repeat, nrad = (int) h->cols[h->col("r")].repeat;
  if (nrad > RELX_MAX_NRADLP) { g_errmsg = "lamp-post table radii exceed the kernel limit"; return RELX_ERR_TABLE; }
  std::vector<float> a(na), hg((size_t) na * nh), rad((size_t) na * nrad);
  std::vector<float> in((size_t) na * nh * nrad), dl(in.size()), di(in.size()), tmp((size_t) na * nrad);
  std::vector<unsigned char> raw((size_t) (na * h->width));
  if (!f.read_rows(*h, 0, na, raw.data())) { g_errmsg = "lamp-post table: read failed"; return RELX_ERR_TABLE; }
  decode_f32(*h, h->col("a"), raw.data(), na, a.data());
  decode_f32(*h, h->col("hgrid"), raw.data(), na, hg.data());
  decode_f32(*h, h->col("r"), raw.data(), na, rad.data());
  for (int k = 0; k < nh; k++) {
    const std::string ks = std::to_string(k + 1);
    const char *names[3] = {"h", "del", "del_inc"};
    std::vector<float> *dst[3] = {&in, &dl, &di};
    for (int q = 0; q < 3; q++) {
      int c = h->col(names[q] + ks);
      if (c < 0 || !decode_f32(*h, c, raw.data(), na, tmp.data())) { g_errmsg = "lamp-post table: column missing"; return RELX_ERR_TABLE; }
      for (int ia = 0; ia < na; ia++)
        for (int ir = 0; ir < nrad; ir++) {
          float v = tmp[(size_t) ia * nrad + ir];
          if (q > 0) v = std::fabs(v);  // reltable.c:370-377
          (*dst[q])[((size_t) ia * nh + k) * nrad + ir] = v;
        }
    }
  }
  int st;
  if ((st = upload(T.lp_a, a)) || (st = upload(T.lp_h, hg)) || (st = upload(T.lp_rad, rad)) ||
      (st = upload(T.lp_intens, in)) || (st = upload(T.lp_del, dl)) || (st = upload(T.lp_delinc, di)))
    return st;
  T.d.lp_na = na; T.d.lp_nh = nh; T.d.lp_nrad = nrad;
  T.d.lp_a = T.lp_a.as<float>(); T.d.lp_h = T.lp_h.as<float>(); T.d.lp_rad = T.lp_rad.as<float>();
  T.d.lp_intens = T.lp_intens.as<float>(); T.d.lp_del = T.lp_del.as<float>(); T.d.lp_delinc = T.lp_delinc.as<float>();
  T.bytes_total += in.size() * 12;
  return 0;
}

constexpr double kPiHost = 3.14159265358979323846;

static const char *kXillNames[] = {"Gamma", "A_Fe", "logXi", "Ecut", "kTe", "Dens", "kTbb", "A_CO", "Frac", "Incl"};
static const int kXillIndex[] = {0, 1, 2, 3, 3, 4, 5, 1, 6, 7};  // common.h:141-150, xilltable.c:24-27

// A xillver table (init_xillver_table, xilltable.c:169-276, 410-447): 5 parameters, or 6 for the
// nthcomp table of the Cp models (xillverCp_v3.4.fits, common.h:166), Incl last.  X receives the
// device buffers, d its x_* fields.  missing_ok: an absent file is not an error (*present = false).
static int load_xillver(const std::string &dir, const char *fname, Tables &T, Tables::XillBufs &X, RelxTables &d,
                        std::vector<double> &xe_host, bool missing_ok, bool *present) {
  FitsFile f;
  std::string err;
  if (present) *present = false;
  if (!f.open(dir + "/" + fname, &err)) {
    if (missing_ok) return 0;
    g_errmsg = err;
    return RELX_ERR_NOTABLE;
  }
  if (present) *present = true;
  const FitsHdu *hp = f.find("PARAMETERS"), *he = f.find("ENERGIES"), *hs = f.find("SPECTRA");
  if (!hp || !he || !hs) { g_errmsg = "xillver table: missing extensions"; return RELX_ERR_TABLE; }
  int npar = (int) hp->nrows;
  if (npar != 5 && npar != 6) { g_errmsg = "xillver table: 5 or 6 parameters expected"; return RELX_ERR_TABLE; }
  std::vector<std::string> names;
  std::vector<double> nv(npar);
  f.read_str(*hp, 0, 0, npar, &names);
  f.read_f64(*hp, 8, 0, npar, nv.data());
  int maxv = (int) hp->cols[9].repeat;
  std::vector<float> vals((size_t) npar * maxv);
  f.read_f32(*hp, 9, 0, npar, vals.data());
  int pidx[RELX_MAX_XPAR];
  int nvals[RELX_MAX_XPAR];
  int has_dens = 0, q_lxi = -1, q_dns = -1;
  for (int q = 0; q < npar; q++) {
    nvals[q] = (int) nv[q];
    pidx[q] = -1;
    for (int j = 0; j < 10; j++)
      if (names[q] == kXillNames[j]) pidx[q] = kXillIndex[j];
    if (pidx[q] < 0) { g_errmsg = "xillver table: unknown parameter " + names[q]; return RELX_ERR_TABLE; }
    if (pidx[q] == 4) { has_dens = 1; q_dns = q; }
    if (pidx[q] == 2) q_lxi = q;
  }
  if (pidx[npar - 1] != 7) { g_errmsg = "xillver table: Incl must be the last parameter"; return RELX_ERR_TABLE; }
  if (nvals[npar - 1] > RELX_MAX_INCL) { g_errmsg = "xillver table: too many inclinations"; return RELX_ERR_TABLE; }
  int ne = (int) he->nrows;
  std::vector<float> elo(ne), ehi(ne);
  f.read_f32(*he, 0, 0, ne, elo.data());
  f.read_f32(*he, 1, 0, ne, ehi.data());
  xe_host.resize(ne + 1);
  for (int i = 0; i < ne; i++) xe_host[i] = elo[i];  // xilltable.c:1104-1109
  xe_host[ne] = ehi[ne - 1];
  int64_t rows = 1;
  for (int q = 0; q < npar; q++) rows *= nvals[q];
  if (hs->nrows != rows) { g_errmsg = "xillver table: SPECTRA row count"; return RELX_ERR_TABLE; }
  const FitsColumn &sc = hs->cols[1];
  if (sc.code != 'E' || sc.repeat != ne) { g_errmsg = "xillver table: SPECTRA column"; return RELX_ERR_TABLE; }
  const int pad = (ne + 3) / 4 * 4;
  // Flux integrals of every row for the returning-radiation correction factors
  // (get_xillver_fluxcorrection_factors, Xillspec.cpp:109-160, 344-361, 457-526): the energy flux
  // in 0.1-1000 keV, the photon flux in 0.15-500 keV, and that photon flux after the rebin of the
  // spectrum shifted by g = 2/3 (a fixed linear map of the row: coefficients pfz_coef).
  std::vector<double> pfz_coef(ne, 0.0);  // uploaded for the decoding kernel below
  {
    const double g0 = 2. / 3.;
    std::vector<double> ez(ne + 1);
    for (int i = 0; i <= ne; i++) ez[i] = xe_host[i] / g0;
    int imin = 0, imax = 0;  // the walk of _rebin_spectrum (relutility.c:549-601), new grid ez, old grid xe
    for (int ii = 0; ii < ne; ii++) {
      if (!((xe_host[0] <= ez[ii + 1]) && (xe_host[ne] >= ez[ii]))) continue;
      while (imin <= ne && xe_host[imin] <= ez[ii]) imin++;
      if (imin > 0) imin--;
      while (imax < ne && xe_host[imax] <= ez[ii + 1]) imax++;
      if (imax > 0) imax--;
      if (!(xe_host[ii] >= 0.15 && xe_host[ii + 1] <= 500.0)) continue;  // band of the photon flux
      double elo = ez[ii], ehi = ez[ii + 1];
      if (elo < xe_host[imin]) elo = xe_host[imin];
      if (ehi > xe_host[imax + 1]) ehi = xe_host[imax + 1];
      if (imax == imin) {
        pfz_coef[imin] += g0 * (ehi - elo) / (xe_host[imin + 1] - xe_host[imin]);
      } else {
        pfz_coef[imin] += g0 * (xe_host[imin + 1] - elo) / (xe_host[imin + 1] - xe_host[imin]);
        pfz_coef[imax] += g0 * (ehi - xe_host[imax]) / (xe_host[imax + 1] - xe_host[imax]);
        for (int q = imin + 1; q <= imax - 1; q++) pfz_coef[q] += g0;
      }
    }
  }
  // strides of the row index (incl fastest, xilltable.c:325-337)
  int64_t stride_lxi = 1, stride_dns = 1;
  for (int q = npar - 1; q > q_lxi; q--) stride_lxi *= nvals[q];
  for (int q = npar - 1; q > q_dns; q--) stride_dns *= nvals[q];
  int st = X.spec.reserve(sizeof(float) * (size_t) rows * pad);
  if (st) return st;
  const int ni = nvals[npar - 1];
  std::vector<double> xe = xe_host;
  std::vector<float2> xew((size_t) ne + 1);
  for (int i = 0; i <= ne; i++) xew[i] = make_float2((float) xe[i], i < ne ? (float) (xe[i + 1] - xe[i]) : 0.0f);
  // 10^logXi per logXi grid value (renorm_xill_spec, xilltable.c:478-485) and the inclination
  // weights of the corner average (calc_angle_averaged_xill_spec, Xillspec.cpp:109-127: the
  // reference weights inclination i by norm_factor_semi_infinite_slab(incl_i * 180 / pi) / n_incl
  // with incl_i the table value in degrees; restated as it is)
  // a table with a density parameter also divides by 10^(logN - 15) of the row (renorm_xill_spec)
  std::vector<double> lxi_div(q_lxi >= 0 ? nvals[q_lxi] : 1, 1.0), dns_div(q_dns >= 0 ? nvals[q_dns] : 1, 1.0),
      incl_w(ni);
  if (q_lxi >= 0)
    for (int k = 0; k < nvals[q_lxi]; k++) lxi_div[k] = std::pow(10, (double) vals[(size_t) q_lxi * maxv + k]);
  if (q_dns >= 0)
    for (int k = 0; k < nvals[q_dns]; k++) {
      const double dn = (double) vals[(size_t) q_dns * maxv + k];
      if (std::fabs(dn - 15) > 1e-6) dns_div[k] = std::pow(10, dn - 15);
    }
  for (int i = 0; i < ni; i++) {
    const double incl_deg = (double) vals[(size_t) (npar - 1) * maxv + i] * 180 / kPiHost;
    incl_w[i] = 0.5 * std::cos(incl_deg * kPiHost / 180) / ni;
  }
  if ((st = upload(X.vals, vals)) || (st = upload(X.e, xe)) || (st = upload(X.ew, xew)) ||
      (st = X.fcorr.reserve(sizeof(double) * 3 * (size_t) (rows / ni))))
    return st;
  // decode on the GPU (table_ingest.cu): raw rows read in chunks into two pinned buffers, so that
  // the file read of one chunk overlaps the copy and decoding of the previous one
  const int64_t chunk = 4096;
  const size_t chunk_bytes = (size_t) chunk * hs->width;
  DevBuf d_raw[2], d_rowflux, d_div, d_dns, d_pfz, d_inclw, d_bad;
  Pinned h_raw[2];
  cudaStream_t stream = nullptr;
  cudaEvent_t done[2] = {nullptr, nullptr};
  auto cleanup = [&]() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto &e : done)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
    for (auto &b : d_raw) b.release();
    for (auto &b : h_raw) b.release();
    d_rowflux.release();
    d_div.release();
    d_dns.release();
    d_pfz.release();
    d_inclw.release();
    d_bad.release();
  };
  int rc = 0;
  if ((rc = d_raw[0].reserve(chunk_bytes)) || (rc = d_raw[1].reserve(chunk_bytes)) ||
      (rc = h_raw[0].reserve(chunk_bytes)) || (rc = h_raw[1].reserve(chunk_bytes)) ||
      (rc = d_rowflux.reserve(sizeof(double) * 3 * (size_t) rows)) || (rc = upload(d_div, lxi_div)) ||
      (rc = upload(d_dns, dns_div)) ||
      (rc = upload(d_pfz, pfz_coef)) || (rc = upload(d_inclw, incl_w)) || (rc = d_bad.reserve(8))) {
    cleanup();
    return rc;
  }
  XillIngest g;
  g.width = hs->width;
  g.col_off = sc.offset;
  g.ne = ne;
  g.pad = pad;
  g.lxi_div = d_div.as<double>();
  g.stride_lxi = stride_lxi;
  g.n_lxi = q_lxi >= 0 ? nvals[q_lxi] : 0;
  g.dns_div = d_dns.as<double>();
  g.stride_dns = stride_dns;
  g.n_dns = q_dns >= 0 ? nvals[q_dns] : 0;
  g.xe = X.e.as<double>();
  g.pfz_coef = d_pfz.as<double>();
  g.spec = X.spec.as<float>();
  g.rowflux = d_rowflux.as<double>();
  g.bad = d_bad.as<unsigned long long>();
  cudaError_t ce = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  for (int b = 0; b < 2 && ce == cudaSuccess; b++) ce = cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(g.bad, 0, 8, stream);
  for (int64_t r0 = 0, k = 0; r0 < rows && ce == cudaSuccess; r0 += chunk, k++) {
    const int b = (int) (k & 1);
    const int64_t nr = std::min(chunk, rows - r0);
    if (k >= 2 && (ce = cudaEventSynchronize(done[b])) != cudaSuccess) break;  // buffer b is free again
    if (!f.read_rows(*hs, r0, nr, (unsigned char *) h_raw[b].h)) {
      g_errmsg = "xillver table: read failed";
      cleanup();
      return RELX_ERR_TABLE;
    }
    if ((ce = cudaMemcpyAsync(d_raw[b].p, h_raw[b].h, (size_t) nr * hs->width, cudaMemcpyHostToDevice, stream)) !=
            cudaSuccess ||
        (ce = launch_xill_ingest(stream, g, d_raw[b].as<unsigned char>(), r0, (int) nr)) != cudaSuccess)
      break;
    ce = cudaEventRecord(done[b], stream);
  }
  if (ce == cudaSuccess)
    ce = launch_xill_corner_flux(stream, g.rowflux, d_inclw.as<double>(), ni, rows / ni, X.fcorr.as<double>());
  unsigned long long nbad = 0;
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&nbad, g.bad, 8, cudaMemcpyDeviceToHost, stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream);
  cleanup();
  if (ce != cudaSuccess) {
    g_errmsg = std::string("xillver table ingest: ") + cudaGetErrorString(ce);
    return RELX_ERR_CUDA;
  }
  if (nbad) {  // table validation
    g_errmsg = "xillver table: " + std::to_string(nbad) + " spectrum values are not finite";
    return RELX_ERR_TABLE;
  }
  d.x_npar = npar; d.x_nener = ne; d.x_nener_pad = pad; d.x_nincl = nvals[npar - 1];
  for (int q = 0; q < RELX_MAX_XPAR; q++) { d.x_nvals[q] = q < npar ? nvals[q] : 0; d.x_pindex[q] = q < npar ? pidx[q] : -1; }
  d.x_has_dens = has_dens;
  d.x_vals = X.vals.as<float>();
  d.x_maxvals = maxv;
  d.x_spec = X.spec.as<float>();
  d.x_rows = rows;
  d.x_e = X.e.as<double>();
  d.x_ew = X.ew.as<float2>();
  d.x_fcorr = X.fcorr.as<double>();
  T.bytes_total += (size_t) rows * pad * 4;
  return 0;
}

// Returning-radiation table (fits_read_returnRadTable, Relreturn_Table.cpp:180-330): extension SPIN
// (column a), then FRAC01, FRAC02, ... with RELX_RR_NR rows.  Optional: without the file the
// models run unless a set switches returning radiation on, which then fails with RELX_ERR_TABLE.
// Per (spin, incident bin, emitting bin, g sample) the device keeps frac_g, the energy shift g of
// the sample (get_gfac_grid, Relreturn_Datastruct.cpp:51-59), log2 g, and 1 where the reference
// boosts the sample by g^(gamma-1) (|g - 1| > 1e-3, Relreturn_Corona.cpp:114-116), else 0.
static int load_rrad(const std::string &dir, Tables &T) {
  T.d.rr_nspin = 0;
  FitsFile f;
  std::string err;
  if (!f.open(dir + "/table_returnRad_v20220301.fits", &err)) return 0;
  const FitsHdu *hs = f.find("SPIN");
  const int ca = hs ? hs->col("a") : -1;
  if (!hs || ca < 0 || hs->nrows < 1 || hs->nrows > RELX_RR_MAXSPIN) {
    g_errmsg = "return radiation table: SPIN extension";
    return RELX_ERR_TABLE;
  }
  const int nspin = (int) hs->nrows, NR = RELX_RR_NR, NG = RELX_RR_NG;
  std::vector<double> spin(nspin), rlo((size_t) nspin * NR), rhi((size_t) nspin * NR),
      tfr((size_t) nspin * NR * NR);
  std::vector<float4> g4((size_t) nspin * NR * NR * NG);
  if (!f.read_f64(*hs, ca, 0, nspin, spin.data())) { g_errmsg = "return radiation table: spins"; return RELX_ERR_TABLE; }
  std::vector<double> gmin((size_t) NR * NR), gmax((size_t) NR * NR), fg((size_t) NR * NR * NG);
  for (int k = 0; k < nspin; k++) {
    char ext[16];
    std::snprintf(ext, sizeof ext, "FRAC%02d", k + 1);
    const FitsHdu *h = f.find(ext);
    if (!h || h->nrows != NR) { g_errmsg = std::string("return radiation table: extension ") + ext; return RELX_ERR_TABLE; }
    const int c_rlo = h->col("rlo"), c_rhi = h->col("rhi"), c_tfr = h->col("tf_r"), c_gmin = h->col("gmin"),
              c_gmax = h->col("gmax"), c_fg = h->col("frac_g");
    if (c_rlo < 0 || c_rhi < 0 || c_tfr < 0 || c_gmin < 0 || c_gmax < 0 || c_fg < 0 || h->cols[c_tfr].repeat != NR ||
        h->cols[c_gmin].repeat != NR || h->cols[c_gmax].repeat != NR || h->cols[c_fg].repeat != (int64_t) NR * NG ||
        !f.read_f64(*h, c_rlo, 0, NR, &rlo[(size_t) k * NR]) || !f.read_f64(*h, c_rhi, 0, NR, &rhi[(size_t) k * NR]) ||
        !f.read_f64(*h, c_tfr, 0, NR, &tfr[(size_t) k * NR * NR]) || !f.read_f64(*h, c_gmin, 0, NR, gmin.data()) ||
        !f.read_f64(*h, c_gmax, 0, NR, gmax.data()) || !f.read_f64(*h, c_fg, 0, NR, fg.data())) {
      g_errmsg = std::string("return radiation table: columns of ") + ext;
      return RELX_ERR_TABLE;
    }
    for (int i = 0; i < NR * NR; i++) {
      for (int jj = 0; jj < NG; jj++) {
        const double g = (jj + 0.5) / NG * (gmax[i] - gmin[i]) + gmin[i];
        if (!(g > 0.0)) { g_errmsg = "return radiation table: energy shift <= 0"; return RELX_ERR_TABLE; }
        const float boosted = std::fabs(g - 1) > 1e-3 ? 1.0f : 0.0f;
        // [spin][incident bin][sample][emitting bin]: a warp's lanes (emitting bins) read contiguous rows
        const int ro = i / NR, re = i - ro * NR;
        g4[(((size_t) k * NR + ro) * NG + jj) * NR + re] =
            make_float4((float) fg[(size_t) i * NG + jj], (float) g, (float) std::log2(g), boosted);
      }
    }
  }
  int st;
  if ((st = upload(T.rr_spin, spin)) || (st = upload(T.rr_rlo, rlo)) || (st = upload(T.rr_rhi, rhi)) ||
      (st = upload(T.rr_tfr, tfr)) || (st = upload(T.rr_g, g4)))
    return st;
  T.d.rr_spin = T.rr_spin.as<double>();
  T.d.rr_rlo = T.rr_rlo.as<double>();
  T.d.rr_rhi = T.rr_rhi.as<double>();
  T.d.rr_tfr = T.rr_tfr.as<double>();
  T.d.rr_g = T.rr_g.as<float4>();
  T.d.rr_nspin = nspin;
  T.bytes_total += g4.size() * sizeof(float4) + tfr.size() * sizeof(double);
  return 0;
}

// the reference's _rebin_spectrum walk (relutility.c:549-601) as a per-output-bin map
static void rebin_map(const std::vector<double> &ener, const std::vector<double> &ener0, std::vector<int> &imn,
                      std::vector<int> &imx, std::vector<float> &fmn, std::vector<float> &fmx) {
  const int nbins = (int) ener.size() - 1, nbins0 = (int) ener0.size() - 1;
  imn.assign(nbins, -1);
  imx.assign(nbins, -1);
  fmn.assign(nbins, 0.0f);
  fmx.assign(nbins, 0.0f);
  int imin = 0, imax = 0;
  for (int ii = 0; ii < nbins; ii++) {
    if ((ener0[0] <= ener[ii + 1]) && (ener0[nbins0] >= ener[ii])) {
      while (imin <= nbins0 && ener0[imin] <= ener[ii]) imin++;
      if (imin > 0) imin--;
      while (imax < nbins0 && ener0[imax] <= ener[ii + 1]) imax++;
      if (imax > 0) imax--;
      double elo = ener[ii], ehi = ener[ii + 1];
      if (elo < ener0[imin]) elo = ener0[imin];
      if (ehi > ener0[imax + 1]) ehi = ener0[imax + 1];
      imn[ii] = imin;
      imx[ii] = imax;
      if (imax == imin) {
        fmn[ii] = (float) ((ehi - elo) / (ener0[imin + 1] - ener0[imin]));
      } else {
        fmn[ii] = (float) ((ener0[imin + 1] - elo) / (ener0[imin + 1] - ener0[imin]));
        fmx[ii] = (float) ((ehi - ener0[imax]) / (ener0[imax + 1] - ener0[imax]));
      }
    }
  }
}

static int load_tables(const std::string &dir, Tables &T) {
  T.release();
  T.d = RelxTables{};
  T.bytes_total = 0;
  std::vector<double> xe, xe_cp;
  int st;
  bool has_cp = false;
  if ((st = load_relline(dir, T)) || (st = load_lp(dir, T)) ||
      (st = load_xillver(dir, "xillver-a-Ec5.fits", T, T.x, T.d, xe, false, nullptr)) ||
      (st = load_xillver(dir, "xillverCp_v3.4.fits", T, T.xcp, T.dcp, xe_cp, true, &has_cp)) ||
      (st = load_rrad(dir, T)))
    return st;
  // conv grid (get_relxill_conv_energy_grid, Xillspec.cpp:44-54) and derived arrays
  std::vector<double> ce;
  log_grid(ce, RELX_NCONV + 1, RELX_EMIN_CONV, RELX_EMAX_CONV);
  std::vector<float2> ceff(ce.size());
  std::vector<float> inv_emid(RELX_NCONV), cf(RELX_NCONV);
  std::vector<float2> cw(RELX_NCONV);
  for (size_t i = 0; i < ce.size(); i++) {
    float hi = (float) ce[i];
    ceff[i] = make_float2(hi, (float) (ce[i] - (double) hi));
  }
  int band_lo = RELX_NCONV, band_hi = -1;
  for (int j = 0; j < RELX_NCONV; j++) {
    inv_emid[j] = (float) (1.0 / (0.5 * (ce[j] + ce[j + 1])));
    cf[j] = (float) (0.5 * (ce[j] + ce[j + 1]) / (ce[j + 1] - ce[j]));  // Relbase.cpp:93-103
    cw[j] = make_float2((float) (0.5 * (ce[j] + ce[j + 1])), (float) (ce[j + 1] - ce[j]));
    if (ce[j] >= RELX_EMIN_XILL && ce[j + 1] < RELX_EMAX_XILL) {   // Relbase.cpp:205
      band_lo = std::min(band_lo, j);
      band_hi = std::max(band_hi, j);
    }
  }
  int pos1 = 0;
  {  // binary_search(ener, n+1, 1.0), Relbase.cpp:133-137
    int klo = 0, khi = RELX_NCONV;
    while (khi - klo > 1) { int k = (khi + klo) / 2; if (ce[k] > 1.0) khi = k; else klo = k; }
    pos1 = klo;
  }
  std::vector<double> co;
  log_grid(co, RELX_NCOARSE + 1, RELX_EMIN_NORM, RELX_EMAX_NORM);
  std::vector<float4> ct(RELX_NCOARSE);
  // bins of the normalisation band (Xillspec.cpp:185-190) outside the band of get_energy_flux_band
  // (e_lo >= 0.1 and e_hi <= 1000, Xillspec.cpp:132-144); only the end bins can differ
  T.d.coarse_b2_skip[0] = T.d.coarse_b2_skip[1] = -1;
  for (int b : {0, RELX_NCOARSE - 1}) {
    const bool band1 = co[b] >= RELX_EMIN_NORM && co[b] <= RELX_EMAX_NORM;
    const bool band2 = co[b] >= 0.1 && co[b + 1] <= 1000;
    if (band1 && !band2) T.d.coarse_b2_skip[b == 0 ? 0 : 1] = b;
  }
  for (int b = 0; b < RELX_NCOARSE; b++) {
    const double em = 0.5 * (co[b] + co[b + 1]);
    const bool in_band = co[b] >= RELX_EMIN_NORM && co[b] <= RELX_EMAX_NORM;
    const float hi = (float) em;
    ct[b] = make_float4(hi, (float) (co[b + 1] - co[b]), in_band ? hi : 0.0f, in_band ? (float) (em - (double) hi) : 0.0f);
  }
  // rebin map xillver grid -> conv grid, per xillver table
  auto rebin_tables = [&](const std::vector<double> &xg, Tables::XillBufs &X, RelxTables &d) -> int {
    std::vector<int> imn, imx;
    std::vector<float> fmn, fmx;
    rebin_map(ce, xg, imn, imx, fmn, fmx);
    std::vector<int4> rbp(imn.size());
    for (size_t j = 0; j < imn.size(); j++) {
      int fa, fb;
      std::memcpy(&fa, &fmn[j], 4);
      std::memcpy(&fb, &fmx[j], 4);
      rbp[j] = make_int4(imn[j], imx[j], fa, fb);
    }
    int r;
    if ((r = upload(X.rb_imin, imn)) || (r = upload(X.rb_imax, imx)) || (r = upload(X.rb_fmin, fmn)) ||
        (r = upload(X.rb_fmax, fmx)) || (r = upload(X.rb_pack, rbp)))
      return r;
    d.rb_imin = X.rb_imin.as<int>();
    d.rb_imax = X.rb_imax.as<int>();
    d.rb_fmin = X.rb_fmin.as<float>();
    d.rb_fmax = X.rb_fmax.as<float>();
    d.rb_pack = X.rb_pack.as<int4>();
    // the conv bins the table reaches: its rows on the conv grid are kept for these only
    int clo = -1, chi = -1;
    for (size_t j = 0; j < imn.size(); j++)
      if (imn[j] >= 0) { if (clo < 0) clo = (int) j; chi = (int) j; }
    if (clo < 0) {
      g_errmsg = "xillver table: its energy grid does not overlap the convolution grid";
      return RELX_ERR_TABLE;
    }
    d.x_clo = clo;
    d.x_cn = chi + 1 - clo;
    d.x_cpad = (d.x_cn + 3) & ~3;
    return 0;
  };
  if ((st = rebin_tables(xe, T.x, T.d)) || (has_cp && (st = rebin_tables(xe_cp, T.xcp, T.dcp)))) return st;
  if ((st = upload(T.conv_e, ce)) || (st = upload(T.conv_eff, ceff)) || (st = upload(T.conv_inv_emid, inv_emid)) ||
      (st = upload(T.conv_cf, cf)) || (st = upload(T.conv_cw, cw)) || (st = upload(T.coarse_e, co)) ||
      (st = upload(T.coarse_t, ct)))
    return st;
  T.d.conv_e = T.conv_e.as<double>();
  T.d.conv_eff = T.conv_eff.as<float2>();
  T.d.conv_inv_emid = T.conv_inv_emid.as<float>();
  T.d.conv_cf = T.conv_cf.as<float>();
  T.d.conv_cw = T.conv_cw.as<float2>();
  T.d.conv_pos1 = pos1;
  T.d.conv_lg0 = (float) std::log(RELX_EMIN_CONV);
  T.d.conv_ilg = (float) (RELX_NCONV / std::log(RELX_EMAX_CONV / RELX_EMIN_CONV));
  T.d.conv_band_lo = band_lo;
  T.d.conv_band_hi = band_hi;
  T.d.coarse_e = T.coarse_e.as<double>();
  T.d.coarse_t = T.coarse_t.as<float4>();
  // the table rows on the conv grid, weighted by E/dE (the convolution's input)
  auto conv_rows = [&](Tables::XillBufs &X, RelxTables &d) -> int {
    int r;
    if ((r = X.cspec.reserve(sizeof(float) * (size_t) d.x_rows * d.x_cpad))) return r;
    RELX_CUDA(launch_xill_conv_rows(nullptr, d.x_spec, d.x_nener_pad, d.x_rows, d.rb_pack, T.d.conv_cf, d.x_clo,
                                    d.x_cn, d.x_cpad, X.cspec.as<float>()));
    RELX_CUDA(cudaDeviceSynchronize());
    d.x_cspec = X.cspec.as<float>();
    T.bytes_total += (size_t) d.x_rows * d.x_cpad * 4;
    return 0;
  };
  if ((st = conv_rows(T.x, T.d)) || (has_cp && (st = conv_rows(T.xcp, T.dcp)))) return st;
  {  // the nthcomp photon grid of the Cp models
    std::vector<NthGrid> g(1);
    if ((st = nth_grid_build(co, RELX_EMIN_NORM, RELX_EMAX_NORM, g[0])) || (st = upload(T.nth_grid, g))) return st;
    T.d.nth_grid = T.nth_grid.as<NthGrid>();
  }
  // the nthcomp descriptor: everything of d but the xillver fields
  if (has_cp) {
    RelxTables c = T.d;
    const RelxTables &x = T.dcp;
    c.x_npar = x.x_npar; c.x_nener = x.x_nener; c.x_nener_pad = x.x_nener_pad; c.x_nincl = x.x_nincl;
    for (int q = 0; q < RELX_MAX_XPAR; q++) { c.x_nvals[q] = x.x_nvals[q]; c.x_pindex[q] = x.x_pindex[q]; }
    c.x_has_dens = x.x_has_dens;
    c.x_vals = x.x_vals;
    c.x_maxvals = x.x_maxvals;
    c.x_spec = x.x_spec;
    c.x_rows = x.x_rows;
    c.x_e = x.x_e;
    c.x_ew = x.x_ew;
    c.x_fcorr = x.x_fcorr;
    c.rb_imin = x.rb_imin; c.rb_imax = x.rb_imax; c.rb_fmin = x.rb_fmin; c.rb_fmax = x.rb_fmax; c.rb_pack = x.rb_pack;
    c.x_cspec = x.x_cspec; c.x_clo = x.x_clo; c.x_cn = x.x_cn; c.x_cpad = x.x_cpad;
    T.dcp = c;
  }
  T.has_cp = has_cp;
  T.loaded = true;
  return 0;
}

// ---------------------------------------------------------------------------
// workspace and batch evaluation
// ---------------------------------------------------------------------------
static int model_nparams(int model) {
  switch (model) {
    case RELX_RELLINE: return 10;   // lmodel_relxill_public.dat:1-11
    case RELX_RELCONV: return 8;    // :13-21
    case RELX_RELXILL: return 13;   // :46-59
    case RELX_RELXILLLP: return 14; // :61-75
    case RELX_RELLINELP: return 10; // :23-33
    case RELX_RELCONVLP: return 9;  // :35-44
    case RELX_XILLVER: return 7;    // :77-84
    case RELX_XILLVERCP: return 8;  // :86-94
    case RELX_RELXILLCP: return 14; // :96-110
    case RELX_RELXILLLPCP: return 17;  // :112-129
    default: return -1;
  }
}

struct EnvOpts {
  int nzones_env = 0, flags = 0;
};
static EnvOpts read_env() {
  EnvOpts o;
  const char *v = std::getenv("RELXILL_NUM_RZONES");
  if (v) o.nzones_env = (int) std::atof(v);
  v = std::getenv("RELLINE_PHYSICAL_NORM");
  if (v && (int) std::strtod(v, nullptr) == 1) o.flags |= 1;
  v = std::getenv("RELXILL_RENORMALIZE");
  if (v && (int) std::atof(v) == 1) o.flags |= 2;
  v = std::getenv("RELXILL_CONSTANT_DENSITY");
  if (v && (int) std::strtod(v, nullptr) == 1) o.flags |= 4;
  return o;
}

// ---- output cache of the local-model entry points: the counterpart of the reference's RelxillCache
// (Relcache.h:182-251, used by relxill_kernel, Relxill.cpp:295-400).  A relxill-family call whose
// parameters all lie within 1e-8 of a recent call's (CACHE_LIMIT, Relcache.h:32, Relcache.cpp:46-48)
// returns that call's flux without evaluating.  The reference keys on the parameters alone and
// rebins its cached spectrum onto each call's grid; here the flux is kept on the caller's grid,
// so the grid and the environment options that change a spectrum are part of the key.  Newest
// first; the oldest is dropped beyond max_entries (RELXILL_CACHE_SIZE 50, Relcache.h:37).
struct OutEntry {
  int model;
  EnvOpts env;
  std::vector<double> par, ener, flux;
};
struct OutCache {
  std::mutex mu;
  std::deque<OutEntry> q;
  size_t max_entries = 50;
  int64_t lookups = 0, hits = 0;
};
static OutCache &outcache() {
  static OutCache c;
  return c;
}
static void outcache_clear() {
  OutCache &oc = outcache();
  std::lock_guard<std::mutex> lock(oc.mu);
  oc.q.clear();
}
static bool outcache_find(int model, const EnvOpts &env, const double *par, int npar, const double *energy,
                          int nflux, double *flux) {
  OutCache &oc = outcache();
  std::lock_guard<std::mutex> lock(oc.mu);
  if (oc.max_entries == 0) return false;
  oc.lookups++;
  for (const OutEntry &e : oc.q) {
    if (e.model != model || e.env.nzones_env != env.nzones_env || e.env.flags != env.flags ||
        (int) e.flux.size() != nflux)
      continue;
    bool same = true;
    for (int q = 0; q < npar && same; q++) same = !(std::fabs(e.par[q] - par[q]) > 1e-8);
    if (!same || std::memcmp(e.ener.data(), energy, sizeof(double) * (size_t) (nflux + 1)) != 0) continue;
    std::memcpy(flux, e.flux.data(), sizeof(double) * (size_t) nflux);
    oc.hits++;
    return true;
  }
  return false;
}
static void outcache_add(int model, const EnvOpts &env, const double *par, int npar, const double *energy, int nflux,
                         const double *flux) {
  OutCache &oc = outcache();
  std::lock_guard<std::mutex> lock(oc.mu);
  if (oc.max_entries == 0) return;
  oc.q.push_front(OutEntry{model, env, std::vector<double>(par, par + npar),
                           std::vector<double>(energy, energy + nflux + 1), std::vector<double>(flux, flux + nflux)});
  while (oc.q.size() > oc.max_entries) oc.q.pop_back();
}

// number of zones a set will use (get_num_zones, relutility.c:506-544)
static int zones_for(int model, int ion_grad_type, int envn) {
  const int kind = relx_kind(model);
  if (kind == RELX_XILLVER) return 1;
  if (ion_grad_type != 0) return (envn > 9 && envn <= RELX_NZMAX) ? envn : RELX_NZONES_IONGRAD;
  if (kind == RELX_RELXILLLP) return (envn > 0 && envn <= RELX_NZMAX) ? envn : RELX_NZONES;
  return 1;
}

struct Workspace {
  DevBuf setin, st, rad, corners, zcorners, line_e, prof, dist, tsum, xill, cout, user_e, user_f, flux, sflag,
      status, err, params, eoff, igt, igi, order, cslot, nthq, nthtab, nthscr, htab;
  Arena arena;  // set by use_arena: every buffer is carved from it
  std::array<DevBuf *, 27> all() {
    return {&setin, &st, &rad, &corners, &zcorners, &line_e, &prof, &dist, &tsum, &xill, &cout, &user_e,
            &user_f, &flux, &sflag, &status, &err, &params, &eoff, &igt, &igi, &order, &cslot, &nthq,
            &nthtab, &nthscr, &htab};
  }
  // carve the buffers from [base, base + bytes) from now on (the workspace holds no allocation)
  void use_arena(void *base, size_t bytes) {
    release();
    arena.base = (unsigned char *) base;
    arena.bytes = bytes;
    arena.off = 0;
    for (DevBuf *b : all()) b->ar = &arena;
  }
  // before a batch: no buffer of the previous batch stays addressable
  void arena_reset() {
    for (DevBuf *b : all()) b->release();
    arena.off = 0;
  }
  void release() {
    for (DevBuf *b : all()) b->release();
  }
};

struct Context {
  std::mutex mu;
  Tables T;
  Workspace W;
  cudaStream_t stream = nullptr;
  int device = -1;
  std::string table_dir;
  bool attrs_set = false;
  Pinned pin;             // host staging of the host-buffer API (its first group)
  std::vector<Pinned> pin_groups;      // staging of the further groups of a large host batch
  std::vector<cudaEvent_t> group_ev;   // completion of each group's copies back
  Workspace W2;                        // workspace of the odd groups
  cudaStream_t gstream[2] = {nullptr, nullptr};  // streams of the even and odd groups
  RelCache cache;         // line-profile cache (off until relx_cache_config)
  cudaStream_t aux[2] = {nullptr, nullptr};      // streams of pipelined chunks
  // per launching stream, a side stream for the emission-angle histograms and the xillver stage,
  // which depend on the set-up only and run beside the line profile (fork and join events)
  struct Side {
    cudaStream_t main, side;
    cudaEvent_t fork, join;
  };
  std::vector<Side> sides;
  cudaEvent_t aux_ev[2] = {nullptr, nullptr}, fork_ev = nullptr;
  // CUDA graphs of recent batch shapes (replayed when the shape and workspace recur)
  struct GraphEntry {
    std::vector<uintptr_t> key;
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;
    uint64_t used = 0;
  };
  std::vector<GraphEntry> graphs;
  std::vector<std::vector<uintptr_t>> graph_seen;  // shapes launched once (captured on the second launch)
  uint64_t graph_clock = 0;
  bool graphs_on = true;
  // autotuned chunking per (model, batch-size class, zones); the line tile is recorded (fixed)
  struct TuneEntry {
    int model, sclass, nza, line_tile, chunk;
    double ms[4];
  };
  std::vector<TuneEntry> tune;
  bool autotune_on = true;
  cudaEvent_t cache_ev = nullptr;  // recorded after the last batch's cache store
  bool cache_ev_valid = false;
};

static void graphs_clear(Context &C);

static Context &ctx() {
  static Context *c = new Context();
  return *c;
}

static int set_kernel_attrs(const Tables &T) {
  RELX_CUDA(cudaFuncSetAttribute(setup_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) setup_smem_bytes()));
  // four set-up CTAs per SM (52 KB each): the largest shared-memory carve-out
  RELX_CUDA(cudaFuncSetAttribute(setup_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  RELX_CUDA(relline_set_smem(T.d.rel_nr, T.d.rel_ng));
  RELX_CUDA(nthcomp_set_smem());
  RELX_CUDA(xillver_set_smem(T.d.x_nincl));
  {
    // one kernel serves both tables: its dynamic shared-memory limit is the larger of the two
    int ne = T.d.x_nener, nep = T.d.x_nener_pad;
    if (T.has_cp && xillver_model_smem_bytes(T.dcp.x_nener, T.dcp.x_nener_pad) > xillver_model_smem_bytes(ne, nep)) {
      ne = T.dcp.x_nener;
      nep = T.dcp.x_nener_pad;
    }
    RELX_CUDA(xillver_model_set_smem(ne, nep));
  }
  RELX_CUDA(cudaFuncSetAttribute(conv_zone_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) conv_smem_bytes()));
  RELX_CUDA(cudaFuncSetAttribute(relconv_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) conv_smem_bytes()));
  return 0;
}

static int ensure_init(Context &C, const char *path) {
  if (C.T.loaded && (!path || C.table_dir == path)) return 0;
  std::string dir;
  if (path) dir = path;
  else {
    const char *e = std::getenv("RELXILL_TABLE_PATH");  // relutility.c:320-328
    dir = e ? e : "./";
  }
  RELX_CUDA(cudaGetDevice(&C.device));
  if (!C.stream) RELX_CUDA(cudaStreamCreateWithFlags(&C.stream, cudaStreamNonBlocking));
  int st = load_tables(dir, C.T);
  if (st) return st;
  C.table_dir = dir;
  RELX_CUDA(C.cache.clear(C.stream));  // cached profiles belong to the previous tables
  outcache_clear();
  graphs_clear(C);
  if ((st = set_kernel_attrs(C.T))) return st;
  return 0;
}

// pack (params, energy offsets) into RelxSetIn on the device
__global__ void pack_kernel(int n_sets, int npar, const double *__restrict__ params, const int64_t *__restrict__ eoff,
                            const int *__restrict__ igt, const double *__restrict__ igi, int nzones_env, int flags,
                            int nza, RelxSetIn *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_sets) return;
  RelxSetIn s;
  for (int q = 0; q < RELX_NPARAM_MAX; q++) s.p[q] = q < npar ? params[(size_t) i * npar + q] : 0.0;
  s.e_off = eoff[i];
  s.n_ener = (int) (eoff[i + 1] - eoff[i] - 1);
  s.ion_grad_type = igt ? igt[i] : 0;
  s.iongrad_index = igi ? igi[i] : 0.0;
  s.nzones_env = nzones_env;
  s.flags = flags;
  s.nza = nza;
  out[i] = s;
}

__global__ void status_kernel(int n_sets, const RelxSetState *__restrict__ st, const int *__restrict__ sflag,
                              const int *__restrict__ err, int *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_sets) return;
  int s = st[i].status;
  if (s == RELX_OK && sflag[i] != RELX_OK) s = sflag[i];
  if (s == RELX_OK && *err != RELX_OK) s = *err;
  out[i] = s;
}

// ---- optional per-kernel timing with CUDA events on the launching stream ----
enum ProfKernel { PK_PACK, PK_SETUP, PK_LINE, PK_XILL, PK_CONV, PK_FIN, PK_STATUS, PK_NTH, PK_HIST, PK_N };
static const char *kProfNames[PK_N] = {"pack",     "setup",  "relline", "xillver", "conv",
                                       "finalize", "status", "nthcomp", "hist"};
struct Profiler {
  bool on = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> rec;
  double ms[PK_N] = {0};
  int64_t n[PK_N] = {0};
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
};
static Profiler g_prof;
static std::atomic<int64_t> g_launches{0};

struct ProfScope {
  int k;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  // kid: kernel kind; nk: kernels launched inside the scope
  ProfScope(int kid, cudaStream_t st, int nk = 1) : k(kid), s(st) {
    g_launches += nk;
    if (g_prof.on) {
      a = g_prof.get();
      b = g_prof.get();
      cudaEventRecord(a, s);
    }
  }
  ~ProfScope() {
    if (g_prof.on) {
      cudaEventRecord(b, s);
      g_prof.rec.push_back({k, {a, b}});
    }
  }
};

static int prof_collect() {
  for (auto &r : g_prof.rec) {
    RELX_CUDA(cudaEventSynchronize(r.second.second));
    float ms = 0;
    RELX_CUDA(cudaEventElapsedTime(&ms, r.second.first, r.second.second));
    g_prof.ms[r.first] += ms;
    g_prof.n[r.first] += 1;
    g_prof.pool.push_back(r.second.first);
    g_prof.pool.push_back(r.second.second);
  }
  g_prof.rec.clear();
  return 0;
}

struct BatchShape {
  int model, n_sets, nza;
  int nz_min = 1;     // the smallest zone count of the batch's sets
  int nblk;           // 256-bin profile-sum blocks per set
  int line_tile = kLineTileH;  // energy bins per line-kernel CTA
  int chunk = 0;      // sets per pipelined chunk (0: one range)
  bool any_limb = false;  // some set uses a limb-darkening law (relline / relconv limb parameter)
  int64_t n_edges;  // total energy edges
};

static int reserve_workspace(const Tables &T, Workspace &W, const BatchShape &b, bool need_zone_corners) {
  const size_t S = b.n_sets;
  const size_t nza = b.nza;
  const int kind = relx_kind(b.model);
  int st;
  if ((st = W.setin.reserve(S * sizeof(RelxSetIn))) || (st = W.st.reserve(S * sizeof(RelxSetState))) ||
      (st = W.user_e.reserve(b.n_edges * sizeof(double))) || (st = W.flux.reserve(b.n_edges * sizeof(double))) ||
      (st = W.sflag.reserve(S * sizeof(int))) || (st = W.status.reserve(S * sizeof(int))) ||
      (st = W.err.reserve(sizeof(int))) || (st = W.cslot.reserve(S * sizeof(int))))
    return st;
  if (relx_is_cp(b.model) &&
      ((st = W.nthq.reserve(S * (RELX_NZMAX + 1) * sizeof(double))) || (st = W.nthtab.reserve(S * sizeof(NthTable))) ||
       (st = W.nthscr.reserve(nthcomp_scratch_bytes((int) S, (int) nza, kind == RELX_XILLVER)))))
    return st;
  if (kind == RELX_XILLVER) return 0;  // no line profile, no convolution
  if ((st = W.rad.reserve(S * sizeof(RelxRadial))) || (st = W.dist.reserve(S * nza * RELX_MAX_INCL * sizeof(float))) ||
      (st = W.tsum.reserve(S * b.nblk * nza * sizeof(double))) ||
      (st = W.htab.reserve(S * (size_t) T.d.rel_nr * T.d.rel_ng * sizeof(float4))))
    return st;
  if (kind == RELX_RELLINE) {
    if ((st = W.line_e.reserve(b.n_edges * sizeof(double))) || (st = W.prof.reserve(b.n_edges * sizeof(float))))
      return st;
  } else {
    if ((st = W.prof.reserve(S * nza * RELX_NCONV * sizeof(float))) ||
        (st = W.cout.reserve(S * nza * RELX_NCONV * sizeof(float))))
      return st;
    if (kind == RELX_RELCONV && (st = W.user_f.reserve(b.n_edges * sizeof(double)))) return st;
  }
  if (relx_is_relxill(kind)) {
    if ((st = W.corners.reserve(S * sizeof(RelxCorners))) || (st = W.order.reserve(S * sizeof(int))) ||
        (st = W.xill.reserve(S * nza * (size_t) std::max(T.d.x_cpad, T.dcp.x_cpad) * sizeof(float))))
      return st;
    if (need_zone_corners && (st = W.zcorners.reserve(S * sizeof(RelxZoneCorners)))) return st;
  }
  return 0;
}

// the side stream of launching stream s (null when none can be made: the work then stays on s)
static Context::Side *side_of(Context &C, cudaStream_t s) {
  for (auto &x : C.sides)
    if (x.main == s) return &x;
  if (C.sides.size() >= 16) return nullptr;
  Context::Side x{s, nullptr, nullptr, nullptr};
  if (cudaStreamCreateWithFlags(&x.side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&x.fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&x.join, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    if (x.side) cudaStreamDestroy(x.side);
    if (x.fork) cudaEventDestroy(x.fork);
    return nullptr;
  }
  C.sides.push_back(x);
  return &C.sides.back();
}

// the kernel sequence for one batch; all pointers are device pointers, asynchronous on `s`
// The kernel sequence for the sets [base, base + n) of a batch, asynchronous on s.  Per-set
// arrays are addressed from the range's first set; energy grids and fluxes keep the batch's
// absolute offsets.  cached: use the line-profile cache (whole batches only).
static int launch_range(Context &C, Workspace &W, const BatchShape &b, cudaStream_t s, int base, int n, bool cached) {
  const bool cp = relx_is_cp(b.model);
  const RelxTables &tab = cp ? C.T.dcp : C.T.d;  // the Cp models use the xillverCp table
  double *nthq = cp ? W.nthq.as<double>() + (size_t) base * (RELX_NZMAX + 1) : nullptr;
  NthTable *ntab = cp ? W.nthtab.as<NthTable>() + base : nullptr;
  const size_t nza = b.nza;
  const int kind = relx_kind(b.model);
  const bool conv_grid = kind != RELX_RELLINE;
  RelxSetIn *sin = W.setin.as<RelxSetIn>() + base;
  RelxSetState *sst = W.st.as<RelxSetState>() + base;
  RelxRadial *rad = W.rad.as<RelxRadial>() + base;
  RelxCorners *cor = W.corners.p ? W.corners.as<RelxCorners>() + base : nullptr;
  RelxZoneCorners *zcor = W.zcorners.p ? W.zcorners.as<RelxZoneCorners>() + base : nullptr;
  float *prof = conv_grid ? W.prof.as<float>() + (size_t) base * nza * RELX_NCONV : W.prof.as<float>();
  float *dist = W.dist.as<float>() + (size_t) base * nza * RELX_MAX_INCL;
  double *tsum = W.tsum.as<double>() + (size_t) base * b.nblk * nza;
  float *xill = W.xill.p ? W.xill.as<float>() + (size_t) base * nza * tab.x_cpad : nullptr;
  float *cout = W.cout.p ? W.cout.as<float>() + (size_t) base * nza * RELX_NCONV : nullptr;
  int *sflag = W.sflag.as<int>() + base;
  double *flux = W.flux.as<double>() - base;  // kernels address set i at e_off(i) - i
  const double *user_e = W.user_e.as<double>();
  if (kind == RELX_XILLVER) {
    if (cp) {
      ProfScope ps(PK_NTH, s);
      RELX_CUDA(launch_nthcomp(s, tab, sin, sst, n, 1, true, nthq, ntab, nullptr, nullptr, W.nthscr.as<float4>(),
                               (int64_t) b.n_sets, (int64_t) base));
    }
    {
      ProfScope ps(PK_XILL, s);
      RELX_CUDA(launch_xillver_model(s, tab, n, sin, user_e, sst, flux, nthq, ntab));
    }
    ProfScope ps(PK_STATUS, s);
    status_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, sst, sflag, W.err.as<int>(), W.status.as<int>() + base);
    RELX_CUDA(cudaGetLastError());
    return 0;
  }
  {
    ProfScope ps(PK_SETUP, s);
    setup_kernel<<<n, kSetupThreadsH, setup_smem_bytes(), s>>>(tab, b.model, sin, user_e, W.line_e.as<double>(), sst,
                                                               rad, cor, zcor);
  }
  if (cp) {  // the nthcomp continua of the source and the zones, their normalisations on the corner weights
    ProfScope ps(PK_NTH, s, 2);
    RELX_CUDA(launch_nthcomp(s, tab, sin, sst, n, b.nza, false, nthq, ntab, cor, zcor, W.nthscr.as<float4>(),
                             (int64_t) b.n_sets * (b.nza + 1), (int64_t) base * (b.nza + 1)));
  }
  if (cached) {
    ProfScope ps(PK_SETUP, s, 2);
    if (C.cache_ev_valid) RELX_CUDA(cudaStreamWaitEvent(s, C.cache_ev, 0));
    RELX_CUDA(cache_lookup(C.cache, s, sin, sst, n, W.cslot.as<int>() + base));
    RELX_CUDA(cache_fill(C.cache, s, sst, W.cslot.as<int>() + base, n, b.nza, b.nblk, kSumBinsH, prof, tsum,
                         dist));
  }
  // relxill models: the emission-angle histograms and the xillver zone spectra depend on the set-up
  // only; they run on a side stream while the line profile runs on s, and s waits for them (all on
  // s while per-kernel timing is on, so that the kernels' intervals do not overlap)
  // the sets' interpolated transfer-function tables (line_table_kernel), then the line profile on
  // s; the histograms and the xillver zone spectra on the side stream after the tables
  float4 *htab = W.htab.as<float4>() + (size_t) base * tab.rel_nr * tab.rel_ng;
  const bool relxill = relx_is_relxill(kind);
  Context::Side *sd = (relxill && !g_prof.on) ? side_of(C, s) : nullptr;
  cudaStream_t xs = sd ? sd->side : s;
  // few sets: a CTA per zone as well, so that the line profile and the histograms of a single
  // spectrum spread over more SMs (the same numbers: zones are summed separately either way)
  const int ntile = (b.nblk * kSumBinsH + kLineTileH - 1) / kLineTileH;
  const bool zsplit = b.nza > 1 && (int64_t) n * ntile < 2 * 152;
  {
    ProfScope ps(PK_LINE, s, 2 + (b.any_limb ? 1 : 0));
    RELX_CUDA(launch_line_table(n, s, tab, sst, htab));
    if (sd) {
      RELX_CUDA(cudaEventRecord(sd->fork, s));
      RELX_CUDA(cudaStreamWaitEvent(xs, sd->fork, 0));
    }
    RELX_CUDA(launch_relline(false, n, b.nblk, s, tab, sin, sst, rad, W.line_e.as<double>(), b.nza, prof, dist, tsum,
                             b.any_limb, zsplit, htab));
  }
  if (relxill) {
    {
      ProfScope ps(PK_HIST, xs);
      RELX_CUDA(launch_hist(n, xs, tab, sst, rad, b.nza, dist, b.nza > 1 && n < 2 * 152, htab));
    }
    {
      // the zone kernel for sets with more than RELX_ZDENSE zones and for 6-parameter sets whose
      // corners do not fit the de-duplicated list; the dense kernel, in table-row order, for the rest
      const bool zone = b.nza > RELX_ZDENSE || cp;
      const bool dense = b.nz_min <= RELX_ZDENSE;
      ProfScope ps(PK_XILL, xs, (zone ? 1 : 0) + (dense ? 2 : 0));
      int *order = dense ? W.order.as<int>() + base : nullptr;
      if (dense) launch_xill_order(xs, sst, cor, zcor, n, order);
      RELX_CUDA(launch_xillver(xs, tab, n, b.nza, zone, dense, sst, cor, zcor, dist, xill, W.err.as<int>(), order));
    }
    if (sd) {
      RELX_CUDA(cudaEventRecord(sd->join, xs));
      RELX_CUDA(cudaStreamWaitEvent(s, sd->join, 0));
    }
  }
  if (cached) {
    ProfScope ps(PK_LINE, s);
    RELX_CUDA(cache_store(C.cache, s, sin, sst, W.cslot.as<int>() + base, n, b.nza, b.nblk, kSumBinsH, prof,
                          tsum, dist));
    if (!C.cache_ev) RELX_CUDA(cudaEventCreateWithFlags(&C.cache_ev, cudaEventDisableTiming));
    RELX_CUDA(cudaEventRecord(C.cache_ev, s));
    C.cache_ev_valid = true;
  }
  if (relxill) {
    {
      ProfScope ps(PK_CONV, s);
      conv_zone_kernel<<<dim3(b.nza, n), kConvThreadsH, conv_smem_bytes(), s>>>(tab, sst, prof, tsum, b.nblk,
                                                                              kSumBinsH, xill, b.nza, cout,
                                                                              W.err.as<int>());
    }
    {
      ProfScope ps(PK_FIN, s);
      RELX_CUDA(launch_finalize_relxill(s, b.n_sets < 2 * 152, n, tab, sin, sst, cout, b.nza, user_e, flux, ntab));
    }
  } else if (kind == RELX_RELCONV) {
    ProfScope ps(PK_CONV, s, 2);  // convolution and finalize
    relconv_conv_kernel<<<n, kConvThreadsH, conv_smem_bytes(), s>>>(tab, sin, sst, prof, tsum, b.nblk,
                                                                    kSumBinsH, b.nza, user_e, W.user_f.as<double>(),
                                                                    cout, sflag);
    finalize_relconv_kernel<<<n, kFinThreadsH, 0, s>>>(tab, sin, sst, cout, b.nza, user_e, sflag, flux);
  } else {
    ProfScope ps(PK_FIN, s);
    finalize_relline_kernel<<<n, kFinThreadsH, 0, s>>>(sin, sst, prof, tsum, b.nblk, kSumBinsH, b.nza, flux);
  }
  {
    ProfScope ps(PK_STATUS, s);
    status_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, sst, sflag, W.err.as<int>(), W.status.as<int>() + base);
  }
  RELX_CUDA(cudaGetLastError());
  return 0;
}

// Sets per pipelined chunk (0: one range).  Chunks alternate between two streams so that the
// kernels of one chunk overlap those of the next (the FP64-bound set-up, the ALU-bound line
// profile and the HBM-bound xillver stage use different units).
static int chunk_sets() {
  const char *v = std::getenv("RELX_CHUNK_SETS");
  return v ? std::max(0, std::atoi(v)) : 0;
}

// the batch as launched, without graphs
static int launch_direct(Context &C, Workspace &W, const BatchShape &b, cudaStream_t s, bool cached) {
  const int S = b.n_sets;
  RELX_CUDA(cudaMemsetAsync(W.sflag.p, 0, S * sizeof(int), s));
  RELX_CUDA(cudaMemsetAsync(W.err.p, 0, sizeof(int), s));
  const int chunk = b.chunk;
  if (cached || chunk <= 0 || S < 2 * chunk) return launch_range(C, W, b, s, 0, S, cached);
  for (int k = 0; k < 2; k++) {
    if (!C.aux[k]) RELX_CUDA(cudaStreamCreateWithFlags(&C.aux[k], cudaStreamNonBlocking));
    if (!C.aux_ev[k]) RELX_CUDA(cudaEventCreateWithFlags(&C.aux_ev[k], cudaEventDisableTiming));
  }
  if (!C.fork_ev) RELX_CUDA(cudaEventCreateWithFlags(&C.fork_ev, cudaEventDisableTiming));
  RELX_CUDA(cudaEventRecord(C.fork_ev, s));
  for (int k = 0; k < 2; k++) RELX_CUDA(cudaStreamWaitEvent(C.aux[k], C.fork_ev, 0));
  int st = 0;
  for (int base = 0, i = 0; base < S; base += chunk, i++) {
    if ((st = launch_range(C, W, b, C.aux[i & 1], base, std::min(chunk, S - base), false))) return st;
  }
  for (int k = 0; k < 2; k++) {
    RELX_CUDA(cudaEventRecord(C.aux_ev[k], C.aux[k]));
    RELX_CUDA(cudaStreamWaitEvent(s, C.aux_ev[k], 0));
  }
  return 0;
}

static std::vector<uintptr_t> graph_key(const Workspace &W, const BatchShape &b) {
  std::vector<uintptr_t> k = {(uintptr_t) b.model, (uintptr_t) b.n_sets, (uintptr_t) b.nza, (uintptr_t) b.nz_min,
                              (uintptr_t) b.nblk, (uintptr_t) b.line_tile, (uintptr_t) b.chunk,
                              (uintptr_t) b.any_limb, (uintptr_t) b.n_edges};
  for (const DevBuf *d : {&W.setin, &W.st, &W.rad, &W.corners, &W.zcorners, &W.line_e, &W.prof, &W.dist, &W.tsum,
                          &W.xill, &W.cout, &W.user_e, &W.user_f, &W.flux, &W.sflag, &W.status, &W.err, &W.order})
    k.push_back((uintptr_t) d->p);
  return k;
}

static void graphs_clear(Context &C) {
  for (auto &g : C.graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  C.graphs.clear();
  C.graph_seen.clear();
}

// cache: the line-profile cache, whose steps are ordered after the previous batch's cache store
// (C.cache_ev), so batches on different streams never read a slot while it is written.
// Without the cache and without per-kernel profiling, the kernel sequence of a batch is captured
// into a CUDA graph on its first launch and replayed whenever the same shape meets the same
// workspace buffers (a sampler or fit that evaluates the same number of sets on the same grids
// every step).
static int launch_batch(Context &C, Workspace &W, const BatchShape &b, cudaStream_t s, bool use_cache) {
  const bool cached = use_cache && C.cache.enabled() && relx_kind(b.model) != RELX_RELLINE &&
                      b.model != RELX_XILLVER;
  if (cached || g_prof.on || !C.graphs_on || s == nullptr) return launch_direct(C, W, b, s, cached);
  const std::vector<uintptr_t> key = graph_key(W, b);
  for (auto &g : C.graphs) {
    if (g.key == key) {
      g.used = ++C.graph_clock;
      g_launches += g.kernels;
      RELX_CUDA(cudaGraphLaunch(g.exec, s));
      return 0;
    }
  }
  // capture only shapes that recur: the first launch of a shape runs directly
  if (std::find(C.graph_seen.begin(), C.graph_seen.end(), key) == C.graph_seen.end()) {
    if (C.graph_seen.size() >= 32) C.graph_seen.erase(C.graph_seen.begin());
    C.graph_seen.push_back(key);
    return launch_direct(C, W, b, s, false);
  }
  // streams and events the captured sequence uses exist before the capture starts
  if (relx_is_relxill(relx_kind(b.model))) {
    (void) side_of(C, s);
    if (b.chunk > 0 && b.n_sets >= 2 * b.chunk) {
      for (int k = 0; k < 2; k++) {
        if (!C.aux[k]) RELX_CUDA(cudaStreamCreateWithFlags(&C.aux[k], cudaStreamNonBlocking));
        if (!C.aux_ev[k]) RELX_CUDA(cudaEventCreateWithFlags(&C.aux_ev[k], cudaEventDisableTiming));
        (void) side_of(C, C.aux[k]);
      }
      if (!C.fork_ev) RELX_CUDA(cudaEventCreateWithFlags(&C.fork_ev, cudaEventDisableTiming));
    }
  }
  const int64_t l0 = g_launches.load();
  RELX_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  const int st = launch_direct(C, W, b, s, false);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (st || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    if (st) return st;
    g_errmsg = std::string("graph capture: ") + cudaGetErrorString(e);
    return RELX_ERR_CUDA;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) {
    g_errmsg = std::string("graph instantiate: ") + cudaGetErrorString(ei);
    return RELX_ERR_CUDA;
  }
  if (C.graphs.size() >= 16) {  // drop the least recently used
    auto lru = std::min_element(C.graphs.begin(), C.graphs.end(),
                                [](const Context::GraphEntry &a, const Context::GraphEntry &c) { return a.used < c.used; });
    cudaGraphExecDestroy(lru->exec);
    C.graphs.erase(lru);
  }
  Context::GraphEntry g;
  g.key = key;
  g.exec = exec;
  g.kernels = (int) (g_launches.load() - l0);
  g.used = ++C.graph_clock;
  C.graphs.push_back(g);
  RELX_CUDA(cudaGraphLaunch(exec, s));
  return 0;
}

// Autotuner: the first batch of 2048 sets or more of a (model, batch-size class, zone count) runs
// once with every candidate (one range, or pipelined chunks of 1024 sets) and keeps the fastest;
// later batches of the class use it.  Every candidate gives the same numbers (the chunks only
// reorder independent sets), so the last trial's results stand.  The trials synchronise the
// stream.  Smaller batches have one candidate, recorded without trials.
static int tuned_launch(Context &C, Workspace &W, BatchShape &b, cudaStream_t s, bool use_cache,
                        bool allow_tune = true) {
  const bool cached = use_cache && C.cache.enabled() && relx_kind(b.model) != RELX_RELLINE &&
                      b.model != RELX_XILLVER;
  int sclass = 0;
  while ((1 << (sclass + 1)) <= b.n_sets) sclass++;
  const Context::TuneEntry *known = nullptr;
  for (const auto &t : C.tune)
    if (t.model == b.model && t.sclass == sclass && t.nza == b.nza) known = &t;
  const bool explicit_choice = std::getenv("RELX_CHUNK_SETS") != nullptr;
  b.line_tile = kLineTileH;
  if (known && !cached && !explicit_choice) b.chunk = known->chunk;
  // the candidates: one range, or pipelined chunks of 1024 sets for large batches
  if (known || !allow_tune || !C.autotune_on || g_prof.on || cached || explicit_choice ||
      relx_kind(b.model) == RELX_RELLINE || b.model == RELX_XILLVER)
    return launch_batch(C, W, b, s, use_cache);
  if (b.n_sets < 2048) {  // one candidate: recorded without trials
    C.tune.push_back(Context::TuneEntry{b.model, sclass, b.nza, kLineTileH, 0, {0, 0, 0, 0}});
    return launch_batch(C, W, b, s, use_cache);
  }
  struct Cand { int tile, chunk; };
  std::vector<Cand> cands = {{kLineTileH, 0}, {kLineTileH, 1024}};
  cudaEvent_t e0, e1;
  RELX_CUDA(cudaEventCreate(&e0));
  RELX_CUDA(cudaEventCreate(&e1));
  Context::TuneEntry t{b.model, sclass, b.nza, 512, 0, {0, 0, 0, 0}};
  float best = 1e30f;
  int st = 0;
  for (size_t i = 0; i < cands.size() && !st; i++) {
    b.line_tile = cands[i].tile;
    b.chunk = cands[i].chunk;
    // an untimed launch first: the first launches of a process also load the kernels
    if ((st = launch_direct(C, W, b, s, false))) break;
    cudaEventRecord(e0, s);
    st = launch_direct(C, W, b, s, false);
    cudaEventRecord(e1, s);
    if (!st && cudaEventSynchronize(e1) == cudaSuccess) {
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      t.ms[i] = ms;
      if (ms < best) {
        best = ms;
        t.line_tile = cands[i].tile;
        t.chunk = cands[i].chunk;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  C.tune.push_back(t);
  b.line_tile = t.line_tile;
  b.chunk = t.chunk;
  return 0;  // the workspace holds the last trial's results
}

// params_host (may be null): the host parameters; relxilllpCp carries its ionisation-gradient type
// as parameter 15 ($iongrad_type, lmodel_relxill_public.dat:126)
static int batch_shape(int model, int n_sets, const int64_t *eoff_host, const int *igt_host, const EnvOpts &env,
                       BatchShape *b, bool *need_zc, const double *params_host = nullptr) {
  b->model = model;
  b->n_sets = n_sets;
  b->n_edges = eoff_host[n_sets];
  int nza = 1, nz_min = RELX_NZMAX, maxn = 0;
  const int npar = model_nparams(model);
  for (int i = 0; i < n_sets; i++) {
    int n = (int) (eoff_host[i + 1] - eoff_host[i] - 1);
    if (n < 1) return RELX_ERR_ARG;
    maxn = std::max(maxn, n);
    int igt = igt_host ? igt_host[i] : 0;
    if (model == RELX_RELXILLLPCP && params_host) igt = (int) std::lround(params_host[(size_t) i * npar + 14]);
    const int nz = zones_for(model, igt, env.nzones_env);
    nza = std::max(nza, nz);
    nz_min = std::min(nz_min, nz);
  }
  b->nza = nza;
  b->nz_min = std::min(nz_min, nza);
  b->chunk = chunk_sets();
  const int kind = relx_kind(model);
  b->any_limb = (kind == RELX_RELLINE || kind == RELX_RELCONV);
  const int gmax = (kind == RELX_RELLINE) ? maxn : RELX_NCONV;
  b->nblk = (gmax + kSumBinsH - 1) / kSumBinsH;
  *need_zc = nza > RELX_ZDENSE || relx_is_cp(model);  // the 6-parameter table uses per-zone corners
  return 0;
}

// Stages the inputs of a host batch through pinned memory, launches the batch and queues the
// copies of the results (flux, then per-set statuses) back into pinned memory, all asynchronous on
// s.  *o_flux / *o_status: their offsets in P.  Caller holds C.mu.
static int enqueue_host_batch(Context &C, Workspace &W, Pinned &P, cudaStream_t s, const HostBatch &hb,
                              bool use_cache, size_t *o_flux, size_t *o_status, bool allow_tune = true) {
  const int model = hb.model, n_sets = hb.n_sets;
  if (model < 0 || model >= RELX_NMODELS || n_sets <= 0 || !hb.params || !hb.energy || !hb.eoff) return RELX_ERR_ARG;
  const bool conv = relx_kind(model) == RELX_RELCONV;
  if (conv && !hb.flux_in) return RELX_ERR_ARG;
  if (relx_is_cp(model) && !C.T.has_cp) {
    g_errmsg = "xillverCp_v3.4.fits not found: the Cp models need the nthcomp xillver table";
    return RELX_ERR_NOTABLE;
  }
  const EnvOpts env = read_env();
  BatchShape b;
  bool need_zc = false;
  int st;
  if ((st = batch_shape(model, n_sets, hb.eoff, hb.igt, env, &b, &need_zc, hb.params))) return st;
  if ((st = reserve_workspace(C.T, W, b, need_zc))) return st;
  const int npar = model_nparams(model);
  const size_t pb = sizeof(double) * (size_t) n_sets * npar, eb = sizeof(double) * (size_t) b.n_edges;
  const size_t ob = sizeof(int64_t) * (size_t) (n_sets + 1), gb = hb.igt ? sizeof(int) * n_sets : 0,
               ib = hb.igi ? sizeof(double) * n_sets : 0;
  const size_t fb = conv ? eb : 0;
  const size_t nflux = (size_t) (b.n_edges - n_sets);
  if ((st = P.reserve(pb + eb + ob + gb + ib + fb + nflux * sizeof(double) + sizeof(int) * n_sets + 64 * 10)))
    return st;
  unsigned char *h = (unsigned char *) P.h;
  size_t off = 0;
  std::vector<CopyPiece> jobs;
  auto put = [&](const void *src, size_t n) {
    size_t o = off;
    if (n && src) jobs.push_back({h + o, src, n});
    off += (n + 63) / 64 * 64;
    return o;
  };
  size_t o_p = put(hb.params, pb), o_e = put(hb.energy, eb), o_o = put(hb.eoff, ob);
  size_t o_g = hb.igt ? put(hb.igt, gb) : 0, o_i = hb.igi ? put(hb.igi, ib) : 0;
  size_t o_f = 0;
  if (conv) {
    // input flux arrives with n per set; spread to the edge layout (offset e_off per set)
    o_f = put(nullptr, fb);
    double *fi = (double *) (h + o_f);
    for (int i = 0; i < n_sets; i++) {
      int n = (int) (hb.eoff[i + 1] - hb.eoff[i] - 1);
      jobs.push_back({fi + hb.eoff[i], hb.flux_in + (hb.eoff[i] - i), sizeof(double) * n});
    }
  }
  CopyPool::get().run(jobs);
  *o_flux = put(nullptr, nflux * sizeof(double));
  *o_status = put(nullptr, sizeof(int) * n_sets);
  if ((st = W.params.reserve(pb)) || (st = W.eoff.reserve(ob)) || (hb.igt && (st = W.igt.reserve(gb))) ||
      (hb.igi && (st = W.igi.reserve(ib))))
    return st;
  RELX_CUDA(cudaMemcpyAsync(W.params.p, h + o_p, pb, cudaMemcpyHostToDevice, s));
  RELX_CUDA(cudaMemcpyAsync(W.user_e.p, h + o_e, eb, cudaMemcpyHostToDevice, s));
  RELX_CUDA(cudaMemcpyAsync(W.eoff.p, h + o_o, ob, cudaMemcpyHostToDevice, s));
  if (hb.igt) RELX_CUDA(cudaMemcpyAsync(W.igt.p, h + o_g, gb, cudaMemcpyHostToDevice, s));
  if (hb.igi) RELX_CUDA(cudaMemcpyAsync(W.igi.p, h + o_i, ib, cudaMemcpyHostToDevice, s));
  if (conv) RELX_CUDA(cudaMemcpyAsync(W.user_f.p, h + o_f, fb, cudaMemcpyHostToDevice, s));
  {
    ProfScope ps(PK_PACK, s);
    pack_kernel<<<(n_sets + 127) / 128, 128, 0, s>>>(n_sets, npar, W.params.as<double>(), W.eoff.as<int64_t>(),
                                                     hb.igt ? W.igt.as<int>() : nullptr,
                                                     hb.igi ? W.igi.as<double>() : nullptr, env.nzones_env, env.flags,
                                                     b.nza, W.setin.as<RelxSetIn>());
  }
  if ((st = tuned_launch(C, W, b, s, use_cache, allow_tune))) return st;
  RELX_CUDA(cudaMemcpyAsync(h + *o_flux, W.flux.p, nflux * sizeof(double), cudaMemcpyDeviceToHost, s));
  RELX_CUDA(cudaMemcpyAsync(h + *o_status, W.status.p, sizeof(int) * n_sets, cudaMemcpyDeviceToHost, s));
  return 0;
}

// host-buffer evaluation: copies in, evaluates, copies out, synchronises.  A large batch runs as
// groups of consecutive sets, each with its own pinned staging, alternating between two streams
// and two workspaces: the host stages group g + 1 while the GPU computes group g, the copies of
// one group overlap the kernels of the other, and the host copies the results of group g out while
// the GPU computes the later groups.  Both workspaces are reserved for the largest group before the
// first one is queued (no buffer is reallocated while a group is in flight).
// group boundaries s0[0..ng]: groups of about `per` sets (RELX_HOST_GROUP_SETS, default 1024), the
// first and the last smaller (RELX_HOST_EDGE_SETS, default half of `per`), so that the GPU starts
// early and the last copy out is short.  Measured on the 4096-set relxilllp workload (ms per step,
// host buffers): ends of 512 and 1024-set groups 9.84, ends of 256 10.16, 128 10.43, one group
// 11.08 -- a small group leaves the GPU partly idle for longer than its copies take.
static std::vector<int> host_groups(int n_sets) {
  const char *e = std::getenv("RELX_HOST_GROUP_SETS");
  const int per = (e && std::atoi(e) >= 64) ? std::atoi(e) : 1024;
  const char *ee = std::getenv("RELX_HOST_EDGE_SETS");
  const int edge = (ee && std::atoi(ee) >= 16 && std::atoi(ee) <= per) ? std::atoi(ee) : per / 2;
  std::vector<int> b{0};
  if (n_sets < 2 * per) {
    b.push_back(n_sets);
    return b;
  }
  const int mid = n_sets - 2 * edge;
  const int nm = std::max(1, std::min(14, (mid + per / 2) / per));
  b.push_back(edge);
  for (int g = 1; g <= nm; g++) b.push_back(edge + (int) ((int64_t) g * mid / nm));
  b.push_back(n_sets);
  return b;
}

static int eval_host(const HostBatch &hb, double *flux, int *status) {
  if (!flux) return RELX_ERR_ARG;
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  int st = ensure_init(C, nullptr);
  if (st) return st;
  const int n = hb.n_sets;
  if (hb.model < 0 || hb.model >= RELX_NMODELS || n <= 0 || !hb.params || !hb.energy || !hb.eoff)
    return RELX_ERR_ARG;
  const std::vector<int> s0 = host_groups(n);
  const int ng = (int) s0.size() - 1;
  const int npar = model_nparams(hb.model);
  const bool conv = relx_kind(hb.model) == RELX_RELCONV;
  std::vector<std::vector<int64_t>> offs(ng);
  std::vector<HostBatch> sub(ng);
  for (int g = 0; g < ng; g++) {
    const int a = s0[g], m = s0[g + 1] - a;
    const int64_t e0 = hb.eoff[a];
    offs[g].resize(m + 1);
    for (int i = 0; i <= m; i++) offs[g][i] = hb.eoff[a + i] - e0;
    HostBatch &b = sub[g];
    b = hb;
    b.n_sets = m;
    b.params = hb.params + (size_t) a * npar;
    b.energy = hb.energy + e0;
    b.eoff = offs[g].data();
    b.flux_in = (conv && hb.flux_in) ? hb.flux_in + (e0 - a) : hb.flux_in;
    b.igt = hb.igt ? hb.igt + a : nullptr;
    b.igi = hb.igi ? hb.igi + a : nullptr;
  }
  if (ng > 1) {
    const EnvOpts env = read_env();
    for (int g = 0; g < ng; g++) {
      BatchShape b;
      bool need_zc = false;
      if ((st = batch_shape(sub[g].model, sub[g].n_sets, sub[g].eoff, sub[g].igt, env, &b, &need_zc, sub[g].params)) ||
          (st = reserve_workspace(C.T, C.W, b, need_zc)) || (st = reserve_workspace(C.T, C.W2, b, need_zc)))
        return st;
    }
    for (int k = 0; k < 2; k++)
      if (!C.gstream[k]) RELX_CUDA(cudaStreamCreateWithFlags(&C.gstream[k], cudaStreamNonBlocking));
  }
  if ((int) C.pin_groups.size() < ng) C.pin_groups.resize(ng);
  while ((int) C.group_ev.size() < ng) {
    cudaEvent_t e;
    RELX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    C.group_ev.push_back(e);
  }
  std::vector<size_t> o_flux(ng), o_status(ng);
  for (int g = 0; g < ng; g++) {
    Pinned &P = (g == 0) ? C.pin : C.pin_groups[g];
    Workspace &W = (g & 1) ? C.W2 : C.W;
    cudaStream_t gs = (ng > 1) ? C.gstream[g & 1] : C.stream;
    if ((st = enqueue_host_batch(C, W, P, gs, sub[g], true, &o_flux[g], &o_status[g])) ||
        cudaEventRecord(C.group_ev[g], gs) != cudaSuccess) {
      cudaDeviceSynchronize();  // earlier groups may still read their staging
      cudaGetLastError();
      return st ? st : RELX_ERR_CUDA;
    }
  }
  int worst = 0;
  std::vector<CopyPiece> out;
  for (int g = 0; g < ng; g++) {
    RELX_CUDA(cudaEventSynchronize(C.group_ev[g]));
    const unsigned char *h = (const unsigned char *) ((g == 0) ? C.pin.h : C.pin_groups[g].h);
    const int a = s0[g], m = s0[g + 1] - a;
    const int64_t nf = offs[g][m] - m;
    out.assign(1, CopyPiece{flux + (hb.eoff[a] - a), h + o_flux[g], sizeof(double) * (size_t) nf});
    CopyPool::get().run(out);
    const int *sts = (const int *) (h + o_status[g]);
    for (int i = 0; i < m; i++) {
      if (status) status[a + i] = sts[i];
      if (sts[i] != 0 && worst == 0) worst = sts[i];
    }
  }
  return worst;
}

// ---- batch slots of the serving engine ----
struct BatchSlot {
  Workspace W;
  Pinned P;
  void *arena = nullptr;  // the device region of W
  cudaStream_t s = nullptr;
  cudaEvent_t done = nullptr;
  size_t o_flux = 0, o_status = 0;
  bool pending = false;
};

void slot_destroy(BatchSlot *b) {
  if (!b) return;
  if (b->s) cudaStreamSynchronize(b->s);
  b->W.release();
  if (b->arena) cudaFree(b->arena);
  b->P.release();
  if (b->done) cudaEventDestroy(b->done);
  if (b->s) cudaStreamDestroy(b->s);
  delete b;
}

int slot_create(BatchSlot **out, size_t arena_bytes, size_t pinned_bytes) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  int st = ensure_init(C, nullptr);
  if (st) return st;
  BatchSlot *b = new BatchSlot();
  if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    slot_destroy(b);
    g_errmsg = "slot stream or event creation failed";
    return RELX_ERR_CUDA;
  }
  if (cudaMalloc(&b->arena, arena_bytes) != cudaSuccess) {
    cudaGetLastError();
    b->arena = nullptr;
    slot_destroy(b);
    g_errmsg = "cudaMalloc of the slot's " + std::to_string(arena_bytes) + " bytes failed";
    return RELX_ERR_NOMEM;
  }
  b->W.use_arena(b->arena, arena_bytes);
  if ((st = b->P.reserve(pinned_bytes))) {
    slot_destroy(b);
    return st;
  }
  *out = b;
  return 0;
}

int slot_enqueue(BatchSlot *b, const HostBatch &hb, bool use_cache) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  // the previous batch of the slot has been waited for: its buffers may be carved again; no
  // autotuning trials here (they would hold the batch for several launches)
  b->W.arena_reset();
  int st = enqueue_host_batch(C, b->W, b->P, b->s, hb, use_cache, &b->o_flux, &b->o_status, false);
  if (st) return st;
  RELX_CUDA(cudaEventRecord(b->done, b->s));
  b->pending = true;
  return 0;
}

int slot_wait(BatchSlot *b, const double **flux, const int **status) {
  if (!b->pending) return RELX_ERR_ARG;
  cudaError_t e = cudaEventSynchronize(b->done);
  b->pending = false;
  if (e != cudaSuccess) {
    g_errmsg = std::string("batch slot: ") + cudaGetErrorString(e);
    return RELX_ERR_CUDA;
  }
  *flux = (const double *) ((const unsigned char *) b->P.h + b->o_flux);
  *status = (const int *) ((const unsigned char *) b->P.h + b->o_status);
  return 0;
}

size_t batch_device_bytes(int model, int n_sets, int64_t n_edges, int max_bins, int nza) {
  const int kind = relx_kind(model);
  const size_t S = (size_t) n_sets, E = (size_t) n_edges;
  // parameters, grid offsets and the ionisation-gradient arrays (enqueue_host_batch), and the
  // 256-byte rounding of each of the workspace's 27 buffers
  const size_t staged = S * (sizeof(double) * RELX_NPARAM_MAX + sizeof(int64_t) + sizeof(int) + sizeof(double)) +
                        sizeof(int64_t) + 27 * 256 + 256;
  const size_t cp = relx_is_cp(model) ? S * (sizeof(NthTable) + sizeof(double) * (RELX_NZMAX + 1)) : 0;
  if (kind == RELX_XILLVER)
    return staged + cp + S * (sizeof(RelxSetIn) + sizeof(RelxSetState) + sizeof(int) * 4) + sizeof(int) +
           (relx_is_cp(model) ? nthcomp_scratch_bytes(n_sets, 1, true) : 0) + sizeof(double) * 2 * E;
  const int gmax = (kind == RELX_RELLINE) ? std::max(max_bins, 1) : RELX_NCONV;
  const size_t nblk = (size_t) (gmax + kSumBinsH - 1) / kSumBinsH;
  size_t per_set = sizeof(RelxSetIn) + sizeof(RelxSetState) + sizeof(RelxRadial) + sizeof(int) * 4 +
                   sizeof(float) * nza * RELX_MAX_INCL + sizeof(double) * nblk * nza +
                   sizeof(float4) * (size_t) RELX_MAX_NRTAB * RELX_MAX_NG;  // the interpolated transfer functions
  size_t per_edge = sizeof(double) * 2;                                      // user grid, flux
  if (kind == RELX_RELLINE) per_edge += sizeof(double) + sizeof(float);     // line grid, profile
  else per_edge += (kind == RELX_RELCONV) ? sizeof(double) : 0;              // relconv input
  if (kind != RELX_RELLINE) per_set += 2 * sizeof(float) * (size_t) nza * RELX_NCONV;
  if (relx_is_relxill(kind))
    per_set += sizeof(RelxCorners) + sizeof(float) * (size_t) nza * 4096;
  if (relx_is_cp(model) || nza > RELX_ZDENSE) per_set += sizeof(RelxZoneCorners);
  return staged + cp + per_set * S + per_edge * E + sizeof(int) +
         (relx_is_cp(model) ? nthcomp_scratch_bytes(n_sets, nza, false) : 0);
}

int cache_configure(int slots) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  if (C.stream) RELX_CUDA(cudaStreamSynchronize(C.stream));
  RELX_CUDA(cudaDeviceSynchronize());  // no batch may use the old cache
  C.cache.release();
  C.cache_ev_valid = false;
  if (slots <= 0) return 0;
  return C.cache.create(slots);
}

// ---- hooks for the other host translation units (not part of the C ABI) ----
bool runtime_tables(RelxTables *out, int *device, bool cp) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  if (!C.T.loaded || (cp && !C.T.has_cp)) return false;
  if (device) *device = C.device;
  *out = cp ? C.T.dcp : C.T.d;
  return true;
}
int runtime_zones(int model, int ion_grad_type, int *nzones_env, int *flags) {
  const EnvOpts env = read_env();
  if (nzones_env) *nzones_env = env.nzones_env;
  if (flags) *flags = env.flags;
  return zones_for(model, ion_grad_type, env.nzones_env);
}
int runtime_nparams(int model) { return model_nparams(model); }
void runtime_set_error(int status, const char *msg) {
  if (msg) g_errmsg = msg;
  g_last_status = status;
}

}  // namespace relx

// ===========================================================================
// C ABI
// ===========================================================================
using namespace relx;

extern "C" {

int relx_init(const char *table_path) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  int st = ensure_init(C, table_path);
  g_last_status = st;
  return st;
}

const char *relx_last_error(void) { return g_errmsg.c_str(); }

int relx_last_status(void) { return g_last_status.load(); }

int relx_eval_batch(int model, int n_sets, const double *params, const double *energy,
                    const int64_t *energy_offsets, const double *flux_in, double *flux, int *status,
                    const int *ion_grad_type, const double *iongrad_index) {
  HostBatch hb;
  hb.model = model;
  hb.n_sets = n_sets;
  hb.params = params;
  hb.energy = energy;
  hb.eoff = energy_offsets;
  hb.flux_in = flux_in;
  hb.igt = ion_grad_type;
  hb.igi = iongrad_index;
  int st = eval_host(hb, flux, status);
  g_last_status = st;
  return st;
}

int relx_eval_batch_device(int model, int n_sets, const double *d_params, const double *d_energy,
                           const int64_t *d_energy_offsets, const int64_t *h_energy_offsets, const double *d_flux_in,
                           double *d_flux, int *d_status, const int *d_ion_grad_type, const int *h_ion_grad_type,
                           const double *d_iongrad_index, void *stream) {
  if (model < 0 || model >= RELX_NMODELS || n_sets <= 0 || !d_params || !d_energy || !d_energy_offsets ||
      !h_energy_offsets || !d_flux)
    return RELX_ERR_ARG;
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  int st = ensure_init(C, nullptr);
  if (st) return st;
  if (relx_is_cp(model) && !C.T.has_cp) {
    g_errmsg = "xillverCp_v3.4.fits not found: the Cp models need the nthcomp xillver table";
    return RELX_ERR_NOTABLE;
  }
  const EnvOpts env = read_env();
  BatchShape b;
  bool need_zc = false;
  if ((st = batch_shape(model, n_sets, h_energy_offsets, h_ion_grad_type, env, &b, &need_zc))) return st;
  if ((st = reserve_workspace(C.T, C.W, b, need_zc))) return st;
  cudaStream_t s = stream ? (cudaStream_t) stream : C.stream;
  Workspace &W = C.W;
  RELX_CUDA(cudaMemcpyAsync(W.user_e.p, d_energy, sizeof(double) * b.n_edges, cudaMemcpyDeviceToDevice, s));
  if (relx_kind(model) == RELX_RELCONV) {
    if (!d_flux_in) return RELX_ERR_ARG;
    RELX_CUDA(cudaMemcpyAsync(W.user_f.p, d_flux_in, sizeof(double) * b.n_edges, cudaMemcpyDeviceToDevice, s));
  }
  {
    ProfScope ps(PK_PACK, s);
    pack_kernel<<<(n_sets + 127) / 128, 128, 0, s>>>(n_sets, model_nparams(model), d_params, d_energy_offsets,
                                                     d_ion_grad_type, d_iongrad_index, env.nzones_env, env.flags,
                                                     b.nza, W.setin.as<RelxSetIn>());
  }
  if ((st = tuned_launch(C, W, b, s, true))) return st;
  RELX_CUDA(cudaMemcpyAsync(d_flux, W.flux.p, sizeof(double) * (b.n_edges - n_sets), cudaMemcpyDeviceToDevice, s));
  if (d_status) RELX_CUDA(cudaMemcpyAsync(d_status, W.status.p, sizeof(int) * n_sets, cudaMemcpyDeviceToDevice, s));
  return 0;
}

int relx_profile_enable(int on) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  int st = prof_collect();
  for (int k = 0; k < PK_N; k++) { g_prof.ms[k] = 0; g_prof.n[k] = 0; }
  g_prof.on = on != 0;
  return st;
}

int relx_profile_read(double *ms, int64_t *launches, int n) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  int st = prof_collect();
  for (int k = 0; k < n && k < PK_N; k++) {
    if (ms) ms[k] = g_prof.ms[k];
    if (launches) launches[k] = g_prof.n[k];
  }
  return st;
}

const char *relx_profile_name(int k) { return (k >= 0 && k < PK_N) ? kProfNames[k] : ""; }

int64_t relx_launch_count(void) { return g_launches.load(); }

int relx_batch_stats(int n_sets, int64_t *out) {
  // out[0] = sum of de-duplicated xillver corners, out[1] = sum of zones, out[2] = sum of line-profile window bins
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  if ((size_t) n_sets * sizeof(RelxSetState) > C.W.st.bytes) return RELX_ERR_ARG;
  std::vector<RelxSetState> st((size_t) n_sets);
  RELX_CUDA(cudaStreamSynchronize(C.stream));
  RELX_CUDA(cudaMemcpy(st.data(), C.W.st.p, sizeof(RelxSetState) * n_sets, cudaMemcpyDeviceToHost));
  out[0] = out[1] = out[2] = 0;
  out[3] = C.T.d.x_cpad;
  out[4] = C.T.d.x_nener_pad;
  for (auto &x : st) {
    if (x.status) continue;
    out[0] += x.ucount;
    out[1] += x.nz;
    out[2] += x.win_hi - x.win_lo;
  }
  return 0;
}

int relx_selftest_wait_timeout(double limit_ms, int *status) {
  if (!status || !(limit_ms > 0.0) || limit_ms > 1000.0) return RELX_ERR_ARG;
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  int *d = nullptr;
  RELX_CUDA(cudaMalloc(&d, sizeof(int)));
  cudaError_t e = launch_wait_selftest(nullptr, (unsigned long long) (limit_ms * 1e6), d);
  if (e == cudaSuccess) e = cudaMemcpy(status, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    g_errmsg = std::string("wait self-test: ") + cudaGetErrorString(e);
    return RELX_ERR_CUDA;
  }
  return 0;
}

int relx_tuning_config(int autotune, int graphs) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  C.autotune_on = autotune != 0;
  C.graphs_on = graphs != 0;
  if (!C.graphs_on) {
    if (C.stream) cudaStreamSynchronize(C.stream);
    graphs_clear(C);
  }
  return 0;
}

int relx_tuning_report(double *out, int max) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  int n = 0;
  for (const auto &t : C.tune) {
    if (n >= max) break;
    double best = 1e30;
    for (double m : t.ms)
      if (m > 0 && m < best) best = m;
    const double v[6] = {(double) t.model, (double) t.sclass, (double) t.nza, (double) t.line_tile, (double) t.chunk,
                         best < 1e30 ? best : 0.0};
    for (int i = 0; i < 6; i++) out[n * 6 + i] = v[i];
    n++;
  }
  return n;
}

int relx_cache_config(int slots) {
  int st = cache_configure(slots);
  g_last_status = st;
  return st;
}

int relx_cache_stats(int64_t *out) {
  if (!out) return RELX_ERR_ARG;
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  out[0] = out[1] = out[2] = 0;
  if (!C.cache.enabled()) return 0;
  RELX_CUDA(cudaDeviceSynchronize());
  unsigned long long c[2];
  RELX_CUDA(cudaMemcpy(c, C.cache.d.counters, sizeof(c), cudaMemcpyDeviceToHost));
  out[0] = (int64_t) c[0];
  out[1] = (int64_t) c[1];
  out[2] = C.cache.d.n_slots;
  return 0;
}

int relx_output_cache_config(int max_entries) {
  if (max_entries < 0) return RELX_ERR_ARG;
  OutCache &oc = outcache();
  std::lock_guard<std::mutex> lock(oc.mu);
  oc.max_entries = (size_t) max_entries;
  while (oc.q.size() > oc.max_entries) oc.q.pop_back();
  return 0;
}

int relx_output_cache_stats(int64_t *out) {
  if (!out) return RELX_ERR_ARG;
  OutCache &oc = outcache();
  std::lock_guard<std::mutex> lock(oc.mu);
  out[0] = oc.lookups;
  out[1] = oc.hits;
  out[2] = (int64_t) oc.q.size();
  return 0;
}

int relx_table_bytes(int64_t *bytes) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  if (!C.T.loaded) return RELX_ERR_NOTABLE;
  *bytes = (int64_t) C.T.bytes_total;
  return 0;
}

void relx_release(void) {
  Context &C = ctx();
  std::lock_guard<std::mutex> lock(C.mu);
  if (C.stream) cudaStreamSynchronize(C.stream);
  graphs_clear(C);
  C.W.release();
  C.W2.release();
  C.T.release();
  C.pin.release();
  for (auto &p : C.pin_groups) p.release();
  C.cache.release();
  C.cache_ev_valid = false;
  noalloc_forget_devices();
}

// ---- local-model entry points with the XSPEC signature (create_wrapper_xspec.py:153-162) ----
static void lmod_eval(int model, const double *energy, int Nflux, const double *parameter, double *flux) {
  if (!energy || !parameter || !flux || Nflux <= 0) {
    g_last_status = RELX_ERR_ARG;
    return;
  }
  const int kind = relx_kind(model);
  const bool cacheable = kind == RELX_RELXILL || kind == RELX_RELXILLLP;  // relxill_kernel's models
  const EnvOpts env = read_env();
  const int npar = model_nparams(model);
  if (cacheable && outcache_find(model, env, parameter, npar, energy, Nflux, flux)) {
    g_last_status = RELX_OK;
    return;
  }
  int64_t eoff[2] = {0, (int64_t) Nflux + 1};
  int status = 0;
  std::vector<double> out((size_t) Nflux);
  std::vector<double> in;
  const bool conv = relx_kind(model) == RELX_RELCONV;
  if (conv) in.assign(flux, flux + Nflux);
  HostBatch hb;
  hb.model = model;
  hb.n_sets = 1;
  hb.params = parameter;
  hb.energy = energy;
  hb.eoff = eoff;
  hb.flux_in = conv ? in.data() : nullptr;
  int st = eval_host(hb, out.data(), &status);
  g_last_status = st ? st : status;
  if (st == 0 || st == status) {
    std::memcpy(flux, out.data(), sizeof(double) * Nflux);
    if (cacheable && st == 0 && status == 0) outcache_add(model, env, parameter, npar, energy, Nflux, flux);
  } else {
    std::fprintf(stderr, " *** relxill-gb300 error %d: %s\n", st, g_errmsg.c_str());
    for (int i = 0; i < Nflux; i++) flux[i] = 0.0;
  }
}

void c_lmodrelline(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                   double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_RELLINE, energy, Nflux, parameter, flux);
}
void c_lmodrelconv(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                   double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_RELCONV, energy, Nflux, parameter, flux);
}
void c_lmodrelxill(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                   double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_RELXILL, energy, Nflux, parameter, flux);
}
void c_lmodrelxilllp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_RELXILLLP, energy, Nflux, parameter, flux);
}
void c_lmodrellinelp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_RELLINELP, energy, Nflux, parameter, flux);
}
void c_lmodrelconvlp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_RELCONVLP, energy, Nflux, parameter, flux);
}
void c_lmodxillver(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                   double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_XILLVER, energy, Nflux, parameter, flux);
}
void c_lmodxillverdensnthcomp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                              double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_XILLVERCP, energy, Nflux, parameter, flux);
}
void c_lmodrelxilldensnthcomp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                              double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_RELXILLCP, energy, Nflux, parameter, flux);
}
void c_lmodrelxilllpdensnthcomp(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                                double *fluxError, const char *init) {
  (void) spectrum; (void) fluxError; (void) init;
  lmod_eval(RELX_RELXILLLPCP, energy, Nflux, parameter, flux);
}

// The NS flavour of the public model list (lmodel_relxill_public.dat:131-153: a neutron-star
// blackbody illuminating the disk, its own xillverNS table) is not part of this library; the
// symbols exist so that a package built from the whole public model list links, and a call fills
// flux with zeros and reports RELX_ERR_UNSUPPORTED.
static void lmod_unsupported(const char *name, double *flux, int Nflux) {
  if (flux)
    for (int i = 0; i < Nflux; i++) flux[i] = 0.0;
  g_errmsg = std::string(name) + ": the NS (blackbody illumination) flavour is not part of this library";
  g_last_status = RELX_ERR_UNSUPPORTED;
}
void c_lmodxillverns(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init) {
  (void) energy; (void) parameter; (void) spectrum; (void) fluxError; (void) init;
  lmod_unsupported("xillverNS", flux, Nflux);
}
void c_lmodrelxillns(const double *energy, int Nflux, const double *parameter, int spectrum, double *flux,
                     double *fluxError, const char *init) {
  (void) energy; (void) parameter; (void) spectrum; (void) fluxError; (void) init;
  lmod_unsupported("relxillNS", flux, Nflux);
}

}  // extern "C"
