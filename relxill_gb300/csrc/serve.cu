// serve.cu -- serving engine: continuous batching of single-spectrum requests
// from many clients (for example the walkers of a sampler) onto the batched
// GPU path.
//
// Clients submit requests at any time.  A scheduler thread forms a batch from
// the requests that are waiting whenever one of two batch slots is free (each
// slot owns a device workspace, pinned staging, a stream and a completion
// event), so a new batch is staged and queued while the previous one runs on
// the GPU.  A batch holds requests of one model, in arrival order, up to the
// engine's maximum batch size and up to the device memory the slot may use
// (admission by the HBM budget given at creation; each slot allocates its half of the budget at
// creation and carves every batch from it).  A completion thread waits
// for the slots in order, copies each result to the client's buffer and
// records the request's latency.  The line-profile cache (relcache.cu), when
// enabled, lets requests whose relativistic parameters repeat skip the
// line-profile stage.  Every set of a batch is computed with a fixed reduction
// order, so a request's result does not depend on the other requests it was
// batched with.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/relxill_gb300.h"
#include "relx_common.h"
#include "relx_runtime.h"

namespace relx {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  int model = 0, n_bins = 0, igt = 0;
  double igi = 0.0;
  double params[RELX_NPARAM_MAX] = {0};
  const double *energy = nullptr;   // client's buffers, valid until completion
  const double *flux_in = nullptr;
  double *flux_out = nullptr;
  Clock::time_point t_submit;
  int nza = 1;
};

struct Completed {
  int64_t id;
  int status;
  double latency_ms;
};

struct SlotState {
  BatchSlot *slot = nullptr;
  std::vector<Request> reqs;  // requests of the batch in flight
  std::vector<double> params, energy, flux_in, igi;
  std::vector<int64_t> eoff;
  std::vector<int> igt;
  bool busy = false;
  int status = 0;
};

struct Server {
  int64_t budget = 0;
  size_t slot_bytes = 0;
  int max_batch = 0;
  bool use_cache = false;
  std::mutex mu;
  std::condition_variable cv_sched, cv_done, cv_wait;
  std::deque<Request> pending;
  SlotState slots[2];
  std::deque<int> inflight;  // slot indices in launch order
  std::vector<Completed> completed;  // not yet polled
  std::unordered_map<int64_t, Completed> finished;  // for relx_serve_wait
  std::vector<double> lat;   // latencies since the last stats reset
  int64_t next_id = 0, n_done = 0, n_batches = 0, n_batched = 0;
  int last_error = 0;
  bool stop = false;
  bool sched_exited = false;  // set after the scheduler thread has been joined
  std::thread sched, done;

  void scheduler();
  void completer();
};

static int model_npar(int model) { return runtime_nparams(model); }

void Server::scheduler() {
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    cv_sched.wait(lk, [&] {
      return (stop && pending.empty()) || (!pending.empty() && (!slots[0].busy || !slots[1].busy));
    });
    if (pending.empty()) return;  // stopping
    const int si = !slots[0].busy ? 0 : 1;
    SlotState &S = slots[si];
    // form the batch: the oldest request's model, arrival order, within max_batch and the slot's memory
    const int model = pending.front().model;
    S.reqs.clear();
    int64_t edges = 0;
    int nza = 1, max_bins = 0;
    for (auto it = pending.begin(); it != pending.end() && (int) S.reqs.size() < max_batch;) {
      if (it->model != model) { ++it; continue; }
      const int z = std::max(nza, it->nza), mb = std::max(max_bins, it->n_bins);
      const size_t need = batch_device_bytes(model, (int) S.reqs.size() + 1, edges + it->n_bins + 1, mb, z);
      // a request that alone needs more than the slot's memory forms a batch of its own, which the
      // slot refuses (status RELX_ERR_NOMEM)
      if (!S.reqs.empty() && need > slot_bytes) break;
      edges += it->n_bins + 1;
      nza = z;
      max_bins = mb;
      S.reqs.push_back(*it);
      it = pending.erase(it);
    }
    S.busy = true;
    lk.unlock();
    // pack the host batch
    const int n = (int) S.reqs.size(), npar = model_npar(model);
    S.params.resize((size_t) n * npar);
    S.eoff.assign(n + 1, 0);
    S.igt.resize(n);
    S.igi.resize(n);
    for (int i = 0; i < n; i++) S.eoff[i + 1] = S.eoff[i] + S.reqs[i].n_bins + 1;
    S.energy.resize((size_t) S.eoff[n]);
    const bool conv = relx_kind(model) == RELX_RELCONV;
    if (conv) S.flux_in.resize((size_t) (S.eoff[n] - n));
    bool any_ig = false;
    for (int i = 0; i < n; i++) {
      const Request &r = S.reqs[i];
      std::memcpy(&S.params[(size_t) i * npar], r.params, sizeof(double) * npar);
      std::memcpy(&S.energy[(size_t) S.eoff[i]], r.energy, sizeof(double) * (r.n_bins + 1));
      if (conv) std::memcpy(&S.flux_in[(size_t) (S.eoff[i] - i)], r.flux_in, sizeof(double) * r.n_bins);
      S.igt[i] = r.igt;
      S.igi[i] = r.igi;
      any_ig = any_ig || r.igt != 0;
    }
    HostBatch hb;
    hb.model = model;
    hb.n_sets = n;
    hb.params = S.params.data();
    hb.energy = S.energy.data();
    hb.eoff = S.eoff.data();
    hb.flux_in = conv ? S.flux_in.data() : nullptr;
    hb.igt = any_ig ? S.igt.data() : nullptr;
    hb.igi = any_ig ? S.igi.data() : nullptr;
    S.status = slot_enqueue(S.slot, hb, use_cache);
    lk.lock();
    inflight.push_back(si);
    n_batches++;
    n_batched += n;
    cv_done.notify_one();
  }
}

void Server::completer() {
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    cv_done.wait(lk, [&] { return !inflight.empty() || sched_exited; });
    if (inflight.empty()) return;  // the scheduler has exited and nothing is in flight
    const int si = inflight.front();
    SlotState &S = slots[si];
    lk.unlock();
    int st = S.status;
    const double *flux = nullptr;
    const int *sts = nullptr;
    if (st == 0) st = slot_wait(S.slot, &flux, &sts);
    const auto now = Clock::now();
    std::vector<Completed> out;
    out.reserve(S.reqs.size());
    int64_t off = 0;
    for (size_t i = 0; i < S.reqs.size(); i++) {
      const Request &r = S.reqs[i];
      int rs = st;
      if (st == 0) {
        std::memcpy(r.flux_out, flux + off, sizeof(double) * r.n_bins);
        rs = sts[i];
      } else {
        std::memset(r.flux_out, 0, sizeof(double) * r.n_bins);
      }
      off += r.n_bins;
      out.push_back({r.id, rs, std::chrono::duration<double, std::milli>(now - r.t_submit).count()});
    }
    lk.lock();
    inflight.pop_front();
    S.busy = false;
    if (st) last_error = st;
    for (auto &c : out) {
      completed.push_back(c);
      finished[c.id] = c;
      lat.push_back(c.latency_ms);
      n_done++;
    }
    cv_sched.notify_one();
    cv_wait.notify_all();
  }
}

}  // namespace relx

using namespace relx;

struct relx_server {
  Server s;
};

extern "C" {

relx_server *relx_serve_create(int64_t hbm_budget_bytes, int max_batch, int cache_slots) {
  if (max_batch <= 0 || hbm_budget_bytes <= 0) return nullptr;
  if (cache_slots > 0 && cache_configure(cache_slots) != 0) return nullptr;
  relx_server *h = new relx_server();
  Server &S = h->s;
  S.budget = hbm_budget_bytes;
  S.max_batch = max_batch;
  S.use_cache = cache_slots > 0;
  S.slot_bytes = (size_t) (hbm_budget_bytes / 2);
  // each slot allocates its half of the budget here, and every batch is carved from it: serving
  // itself allocates no device memory.  Host staging starts at max_batch spectra of the 4096-bin
  // convolution grid (at most 256 MB) and grows by half when a batch needs more.
  const size_t per_req = sizeof(double) * (RELX_NPARAM_MAX + 3 * 4097) + 64;
  const size_t pinned = std::min((size_t) 256 << 20, per_req * (size_t) max_batch);
  for (auto &sl : S.slots) {
    if (slot_create(&sl.slot, S.slot_bytes, pinned) != 0) {
      for (auto &t : S.slots) slot_destroy(t.slot);
      delete h;
      return nullptr;
    }
  }
  S.sched = std::thread([&S] { S.scheduler(); });
  S.done = std::thread([&S] { S.completer(); });
  return h;
}

int64_t relx_serve_submit(relx_server *h, int model, const double *params, const double *energy, int n_bins,
                          const double *flux_in, double *flux_out, int ion_grad_type, double iongrad_index) {
  if (!h || model < 0 || model >= RELX_NMODELS || !params || !energy || !flux_out || n_bins < 1) return -RELX_ERR_ARG;
  if (relx_kind(model) == RELX_RELCONV && !flux_in) return -RELX_ERR_ARG;
  Request r;
  r.model = model;
  r.n_bins = n_bins;
  r.igt = ion_grad_type;
  r.igi = iongrad_index;
  std::memcpy(r.params, params, sizeof(double) * runtime_nparams(model));
  r.energy = energy;
  r.flux_in = flux_in;
  r.flux_out = flux_out;
  r.nza = runtime_zones(model, ion_grad_type, nullptr, nullptr);
  r.t_submit = Clock::now();
  Server &S = h->s;
  std::lock_guard<std::mutex> lk(S.mu);
  r.id = S.next_id++;
  S.pending.push_back(r);
  S.cv_sched.notify_one();
  return r.id;
}

int relx_serve_poll(relx_server *h, int64_t *ids, int *status, double *latency_ms, int max) {
  if (!h || max < 0) return -RELX_ERR_ARG;
  Server &S = h->s;
  std::lock_guard<std::mutex> lk(S.mu);
  const int n = std::min<int>(max, (int) S.completed.size());
  for (int i = 0; i < n; i++) {
    if (ids) ids[i] = S.completed[i].id;
    if (status) status[i] = S.completed[i].status;
    if (latency_ms) latency_ms[i] = S.completed[i].latency_ms;
    S.finished.erase(S.completed[i].id);
  }
  S.completed.erase(S.completed.begin(), S.completed.begin() + n);
  return n;
}

int relx_serve_wait(relx_server *h, int64_t id, int *status) {
  if (!h || id < 0) return RELX_ERR_ARG;
  Server &S = h->s;
  std::unique_lock<std::mutex> lk(S.mu);
  if (id >= S.next_id) return RELX_ERR_ARG;
  S.cv_wait.wait(lk, [&] { return S.finished.count(id) != 0 || S.stop; });
  auto it = S.finished.find(id);
  if (it == S.finished.end()) return RELX_ERR_ARG;
  if (status) *status = it->second.status;
  return 0;
}

int relx_serve_stats(relx_server *h, double *out, int n, int reset) {
  if (!h || !out || n < 1) return RELX_ERR_ARG;
  Server &S = h->s;
  std::lock_guard<std::mutex> lk(S.mu);
  std::vector<double> l = S.lat;
  std::sort(l.begin(), l.end());
  auto pct = [&](double p) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t) (p * (l.size() - 1) + 0.5))]; };
  const double v[8] = {(double) S.n_done, (double) S.n_batches,
                       S.n_batches ? (double) S.n_batched / S.n_batches : 0.0, pct(0.50), pct(0.99),
                       l.empty() ? 0.0 : l.back(), (double) S.pending.size(), (double) S.last_error};
  for (int i = 0; i < n && i < 8; i++) out[i] = v[i];
  if (reset) {
    S.lat.clear();
    S.n_batches = 0;
    S.n_batched = 0;
  }
  return 0;
}

void relx_serve_destroy(relx_server *h) {
  if (!h) return;
  Server &S = h->s;
  {
    std::lock_guard<std::mutex> lk(S.mu);
    S.stop = true;
  }
  S.cv_sched.notify_all();
  S.cv_done.notify_all();
  S.cv_wait.notify_all();
  S.sched.join();
  {
    std::lock_guard<std::mutex> lk(S.mu);
    S.sched_exited = true;
  }
  S.cv_done.notify_all();
  S.done.join();
  for (auto &sl : S.slots) slot_destroy(sl.slot);
  delete h;
}

}  // extern "C"
