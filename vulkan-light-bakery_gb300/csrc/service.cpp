// service.cpp -- the resident bake service of include/vlb.h (vlb_service_*).
//
// No reference counterpart: the reference bakes one scene per process
// (baker/main.cpp:22-24, LightBaker::bake light_baker.cpp:287-328).  This is
// the serving loop around the batched bake:
//
//   submit (any thread)  -> queue (FIFO, mutex)
//   worker thread        -> cuts the queue into a batch (probe cap,
//                           device-memory budget), launches it with the
//                           vlb_bake_batch machinery on a private stream
//                           without waiting, records an event, and retires
//                           batches whose event has fired (copies each
//                           request's rows out of pinned staging);
//                           up to max_inflight batches are queued on the GPU,
//                           so the next batch is assembled while one runs.
//
// Slicing: a batch takes at most slice_probes probes of any one request.  A
// larger request stays at its place in the queue and gives one slice (a range
// of its probes) to each batch until all its probes are launched, so the
// requests behind it ride in the same batches instead of waiting for all of
// it: a small request waits for at most max_inflight batches of bounded
// size.  Each probe's result does not depend on the batch or the slice (the
// bake is per probe), so a sliced request returns the bits of vlb_bake.
//   wait (any thread)    -> condition variable on the ticket.
//
// Kept hits: a bake submitted with keep_hits stores (triangle slot, distance)
// per ray in stream-ordered device memory; a relight of it skips the primary
// walk (the trace kernel reads the kept hit) and re-traces only the shadow
// ray.  Kept sets count against the budget and are evicted least recently
// used when a batch needs room; the host copy of the probes stays, so a
// relight of an evicted set bakes in full with the same result.
//
// Budget accounting: device bytes of the batches in flight (radiance tile or
// fused chunk partials, outputs, probe and sort scratch) plus the resident
// kept sets.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "vlb_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint64_t kDefaultBudget = 64ull << 30;
constexpr uint32_t kDefaultMaxProbes = 1u << 20;
constexpr uint32_t kDefaultInflight = 2;
constexpr uint32_t kDefaultSlice = 2048;

uint32_t svc_k(uint32_t lmax) { return (lmax + 1) * (lmax + 1); }

// Message of the calling thread's last failed service call.
thread_local std::string t_err;
vlb_status sfail(vlb_status st, const std::string& msg) {
  t_err = msg;
  return st;
}

// Device bytes a batch holds for one request while it runs: the radiance
// tile (FP32, BF16 hi/lo pairs or one BF16), or for the fused walk its chunk
// partials and tickets.
uint64_t transient_bytes(uint64_t n, uint64_t S, uint32_t K, uint32_t prec) {
  uint64_t work;
  if (prec == VLB_PREC_FUSED) {
    const uint64_t D = vlbk::fused_chunk_rays(uint32_t(S)), C = (S + D - 1) / D;
    work = n * ((C > 1 ? C * 3 * K * 4 : 0) + 4);
  } else {
    work = n * S * 3 * (prec == VLB_PREC_BF16 ? 2 : 4);
  }
  return work + n * (12 + 4 + 16 + uint64_t(K) * 12);
}
// Device bytes of a kept-hit set.
uint64_t hitset_bytes(uint64_t n, uint64_t S) { return n * S * 8 + n * 12; }

// The cut rule shared by the worker and vlb_service_plan: does a request of
// (probes, bytes) still join the batch being formed?
bool joins(bool empty, uint64_t cur_probes, uint64_t cur_bytes, uint64_t probes, uint64_t bytes, uint64_t max_probes,
           uint64_t room) {
  if (empty) return bytes <= room;
  return cur_probes + probes <= max_probes && cur_bytes + bytes <= room;
}

struct Request {
  uint64_t ticket = 0;
  const vlb_scene* scene = nullptr;
  std::vector<float> probes;  // host copy (bakes)
  uint32_t n = 0;             // probes (a relight: the kept bake's)
  uint32_t next_off = 0;      // probes launched so far (slices)
  uint32_t pending = 0;       // slices launched and not yet retired
  bool failed = false;
  vlb_bake_params params{};
  uint64_t relight_of = 0;
  bool keep = false;
  Clock::time_point t_submit;
  enum State { kQueued, kRunning, kDone, kFailed } state = kQueued;
  vlb_status status = VLB_OK;
  std::string err;
  std::vector<float> result;
  double latency_ms = 0.0;
};

struct HitSet {
  const vlb_scene* scene = nullptr;
  const vlb_dirset* dirs = nullptr;
  float tmin = 0.f, tmax = 0.f;
  uint32_t n = 0;
  std::vector<float> h_probes;
  float* d_probes = nullptr;
  int2* d_hits = nullptr;
  uint64_t bytes = 0;
  uint64_t last_use = 0;
  bool resident = false;   // device copies exist (allocated when the keeping bake launched)
  bool dropped = false;    // released by the user: freed by the worker
};

// One request's probes [off, off + cnt) in a batch, its rows at `out` floats
// into the staging buffer.
struct Slice {
  Request* r;
  uint32_t off, cnt;
  size_t out;
};

struct Batch {
  std::vector<Slice> slices;
  cudaEvent_t done = nullptr;
  float* h_out = nullptr;    // pinned staging
  size_t h_cap = 0;
  int* h_err = nullptr;      // pinned copy of the device error counters
  uint64_t bytes = 0;
  uint64_t rays = 0;
};

}  // namespace

struct vlb_service {
  vlb_ctx* user = nullptr;
  vlb_ctx* ctx = nullptr;  // private context: own stream, accepts the user's objects
  vlb_service_config cfg{};
  uint32_t K = 9;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  uint64_t next_ticket = 1;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  std::unordered_map<uint64_t, std::unique_ptr<HitSet>> sets;  // by the keeping bake's ticket
  uint64_t use_clock = 0;
  vlb_service_stats stats{};
  uint64_t set_bytes = 0, flight_bytes = 0;

  // worker-only state
  std::deque<Batch> inflight;
  std::vector<std::pair<float*, size_t>> pinned_pool;
  std::vector<int*> err_pool;
  std::vector<cudaEvent_t> event_pool;
  std::thread worker;

  void run();
  bool launch_next(std::unique_lock<std::mutex>& lk);
  void retire(Batch& b, std::unique_lock<std::mutex>& lk);
  void free_set(HitSet& s);
  void fail_slices(std::vector<Slice>& sl, vlb_status st, const std::string& msg);
  void fail_request(Request* r, vlb_status st, const std::string& msg);
  void finalize(Request* r);
  void note_bytes() {
    stats.bytes_in_use = set_bytes + flight_bytes;
    stats.bytes_peak = std::max(stats.bytes_peak, stats.bytes_in_use);
  }
};

void vlb_service::free_set(HitSet& s) {
  if (!s.resident) return;
  cudaFreeAsync(s.d_hits, ctx->stream);
  cudaFreeAsync(s.d_probes, ctx->stream);
  s.d_hits = nullptr;
  s.d_probes = nullptr;
  s.resident = false;
  set_bytes -= s.bytes;
}

// A request is complete when all its probes are launched (or it failed) and
// no slice of it is running.
void vlb_service::finalize(Request* r) {
  if (r->pending || (!r->failed && r->next_off < r->n)) return;
  if (r->failed) {
    auto q = std::find(queue.begin(), queue.end(), r->ticket);
    if (q != queue.end()) queue.erase(q);
    r->state = Request::kFailed;
    r->result.clear();
    ++stats.failed;
  } else {
    r->state = Request::kDone;
    r->latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - r->t_submit).count();
    ++stats.completed;
  }
  cv_done.notify_all();
}

void vlb_service::fail_request(Request* r, vlb_status st, const std::string& msg) {
  if (!r->failed) {
    r->failed = true;
    r->status = st;
    r->err = msg;
  }
  finalize(r);
}

// Slices that were not launched (or whose batch failed): their requests fail.
void vlb_service::fail_slices(std::vector<Slice>& sl, vlb_status st, const std::string& msg) {
  for (Slice& x : sl) fail_request(x.r, st, msg);
}

// Forms and launches the next batch from the queue, in order, one slice per
// request.  Called with the lock held; returns false when nothing could be
// launched now.
bool vlb_service::launch_next(std::unique_lock<std::mutex>& lk) {
  const uint64_t budget = cfg.hbm_budget_bytes;
  std::vector<Slice> take;
  uint64_t probes = 0, bytes = 0, keep_bytes = 0;
  auto room = [&]() { return budget > set_bytes + flight_bytes ? budget - set_bytes - flight_bytes : 0; };
  for (size_t qi = 0; qi < queue.size();) {
    Request* r = reqs[queue[qi]].get();
    if (r->failed) {  // a slice of it failed: its other probes are not launched
      queue.erase(queue.begin() + long(qi));
      finalize(r);
      continue;
    }
    HitSet* src = nullptr;
    if (r->relight_of) {
      auto it = sets.find(r->relight_of);
      src = it == sets.end() ? nullptr : it->second.get();
      // the kept bake's hits are written by its own launches: every probe of it
      // launched before, none in this batch
      auto kr = reqs.find(r->relight_of);
      const bool launched = kr == reqs.end() || kr->second->failed || kr->second->next_off >= kr->second->n;
      bool here = false;
      for (const Slice& x : take) here |= x.r->ticket == r->relight_of;
      if (!launched || here) { ++qi; continue; }
    }
    // one batch bakes one shading (vlb_bake_batch's rule)
    if (!take.empty() && r->params.shading != take.front().r->params.shading) break;
    const uint32_t cnt = std::min(r->n - r->next_off, cfg.slice_probes);
    const uint32_t S = src ? src->dirs->n : r->params.dirs->n;
    uint64_t b = transient_bytes(cnt, S, K, cfg.precision);
    // a kept set is allocated whole with a bake's first slice
    const uint64_t kb = r->keep && !r->relight_of && r->next_off == 0 ? hitset_bytes(r->n, S) : 0;
    b += kb;
    // room: budget minus what is held; evict unused kept sets (LRU) if the head does not fit
    if (!joins(take.empty(), probes, bytes, cnt, b, cfg.max_batch_probes, room())) {
      if (!take.empty()) break;
      while (b > room()) {
        HitSet* lru = nullptr;
        for (auto& kv : sets)
          if (kv.second->resident && kv.second.get() != src &&
              (!lru || kv.second->last_use < lru->last_use))
            lru = kv.second.get();
        if (!lru) break;
        free_set(*lru);
        ++stats.evictions;
      }
      note_bytes();
      if (b > room()) {
        if (!inflight.empty()) return false;  // wait for the batches in flight to free their room
        queue.erase(queue.begin() + long(qi));
        fail_request(r, VLB_ERR_OOM, "request exceeds the free device-memory budget");
        continue;
      }
    }
    take.push_back({r, r->next_off, cnt, 0});
    r->next_off += cnt;
    probes += cnt;
    bytes += b;
    keep_bytes += kb;
    if (src) src->last_use = ++use_clock;
    if (r->next_off >= r->n) queue.erase(queue.begin() + long(qi));
    else ++qi;
  }
  if (take.empty()) return false;

  // jobs (the lock stays held: the worker is the only user of ctx and of the
  // sets' device state; submitters only append to the queue)
  const size_t nj = take.size();
  std::vector<vlb_bake_job> jobs(nj);
  std::vector<vlbh::JobExt> ext(nj);
  std::vector<vlb_bake_params> jp(nj);
  Batch bt;
  size_t rows = 0;
  for (size_t i = 0; i < nj; ++i) {
    Slice& x = take[i];
    Request* r = x.r;
    if (x.off == 0) r->result.assign(size_t(r->n) * 3 * K, 0.f);
    jp[i] = r->params;
    jp[i].lmax = cfg.lmax;
    jp[i].precision = cfg.precision;
    vlb_bake_job& j = jobs[i];
    j.params = &jp[i];
    j.nprobes = x.cnt;
    if (r->relight_of) {
      HitSet* s = sets[r->relight_of].get();
      const size_t S = s->dirs->n;
      jp[i].dirs = s->dirs;
      jp[i].tmin = s->tmin;
      jp[i].tmax = s->tmax;
      j.scene = s->scene;
      if (x.off == 0) ++stats.relights;
      if (s->resident && !s->dropped) {
        j.probe_xyz = s->d_probes + size_t(x.off) * 3;
        ext[i].hits_in = s->d_hits + size_t(x.off) * S;
      } else {
        if (x.off == 0) ++stats.relights_rebaked;
        j.probe_xyz = s->h_probes.data() + size_t(x.off) * 3;
      }
    } else {
      j.scene = r->scene;
      j.probe_xyz = r->probes.data() + size_t(x.off) * 3;
      if (r->keep) {
        HitSet* s = sets[r->ticket].get();
        const size_t S = r->params.dirs->n;
        if (x.off == 0) {
          const size_t rays = size_t(r->n) * S;
          if (cudaMallocAsync(reinterpret_cast<void**>(&s->d_hits), rays * 8, ctx->stream) != cudaSuccess ||
              cudaMallocAsync(reinterpret_cast<void**>(&s->d_probes), size_t(r->n) * 12, ctx->stream) !=
                  cudaSuccess ||
              cudaMemcpyAsync(s->d_probes, r->probes.data(), size_t(r->n) * 12, cudaMemcpyHostToDevice,
                              ctx->stream) != cudaSuccess) {
            cudaGetLastError();
            if (s->d_hits) cudaFreeAsync(s->d_hits, ctx->stream);
            if (s->d_probes) cudaFreeAsync(s->d_probes, ctx->stream);
            s->d_hits = nullptr;
            s->d_probes = nullptr;
          } else {
            s->resident = true;  // a set released before its bake launched is freed right after
            s->bytes = hitset_bytes(r->n, S);
            set_bytes += s->bytes;
            s->last_use = ++use_clock;
          }
        }
        // later slices write into the set while it stays resident (an evicted
        // set is baked in full by its relights)
        if (s->resident) {
          ext[i].hits_out = s->d_hits + size_t(x.off) * S;
          j.probe_xyz = s->d_probes + size_t(x.off) * 3;
        }
      }
    }
    x.out = rows * 3 * K;
    rows += x.cnt;
    bt.rays += uint64_t(x.cnt) * jp[i].dirs->n;
  }
  // pinned staging for the outputs and the error counters
  const size_t need = std::max<size_t>(rows * 3 * K, 1);
  for (size_t i = 0; i < pinned_pool.size(); ++i)
    if (pinned_pool[i].second >= need) {
      bt.h_out = pinned_pool[i].first;
      bt.h_cap = pinned_pool[i].second;
      pinned_pool.erase(pinned_pool.begin() + long(i));
      break;
    }
  if (!bt.h_out) {
    if (cudaMallocHost(reinterpret_cast<void**>(&bt.h_out), need * 4) != cudaSuccess) {
      cudaGetLastError();
      fail_slices(take, VLB_ERR_OOM, "pinned staging allocation failed");
      return true;
    }
    bt.h_cap = need;
  }
  if (!err_pool.empty()) { bt.h_err = err_pool.back(); err_pool.pop_back(); }
  else if (cudaMallocHost(reinterpret_cast<void**>(&bt.h_err), vlbk::kErrSlots * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    pinned_pool.push_back({bt.h_out, bt.h_cap});
    fail_slices(take, VLB_ERR_OOM, "pinned staging allocation failed");
    return true;
  }
  for (size_t i = 0; i < nj; ++i) jobs[i].out = bt.h_out + take[i].out;
  if (!event_pool.empty()) { bt.done = event_pool.back(); event_pool.pop_back(); }
  else cudaEventCreateWithFlags(&bt.done, cudaEventDisableTiming);

  vlb_bake_params bp = jp[0];
  const vlb_batch_schedule sc{0, 1, 0};
  bool host_out = false;
  vlb_status st = vlbh::batch_launch(ctx, jobs.data(), ext.data(), uint32_t(nj), &bp, sc, &host_out);
  ctx->host_inputs_pending = false;  // pageable inputs were staged before the copies returned
  if (st == VLB_OK) {
    const cudaError_t e1 = cudaMemcpyAsync(bt.h_err, ctx->d_err, vlbk::kErrSlots * sizeof(int), cudaMemcpyDeviceToHost,
                                           ctx->stream);
    const cudaError_t e2 = cudaMemsetAsync(ctx->d_err, 0, vlbk::kErrSlots * sizeof(int), ctx->stream);
    const cudaError_t e3 = cudaEventRecord(bt.done, ctx->stream);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
      cudaGetLastError();
      st = VLB_ERR_CUDA;
      ctx->err = "service: enqueue failed";
    }
  }
  if (st != VLB_OK) {
    pinned_pool.push_back({bt.h_out, bt.h_cap});
    err_pool.push_back(bt.h_err);
    event_pool.push_back(bt.done);
    fail_slices(take, st, ctx->err);
    return true;
  }
  for (Slice& x : take) {
    x.r->state = Request::kRunning;
    ++x.r->pending;
  }
  bt.slices = std::move(take);
  bt.bytes = bytes - keep_bytes;
  flight_bytes += bt.bytes;
  ++stats.batches;
  note_bytes();
  inflight.push_back(std::move(bt));
  (void)lk;
  return true;
}

void vlb_service::retire(Batch& b, std::unique_lock<std::mutex>&) {
  bool bad = false;
  for (int i = 0; i < vlbk::kErrSlots; ++i) bad |= b.h_err[i] != 0;
  char msg[200] = "";
  if (bad)
    std::snprintf(msg, sizeof msg,
                  "device check failed in the batch (stack overflow %d, timeout %d, input %d, bounds %d)",
                  b.h_err[vlbk::kErrStackOverflow], b.h_err[vlbk::kErrTimeout], b.h_err[vlbk::kErrBadInput],
                  b.h_err[vlbk::kErrBounds]);
  for (Slice& x : b.slices) {
    Request* r = x.r;
    --r->pending;
    if (bad) {
      fail_request(r, VLB_ERR_INTERNAL, msg);
      continue;
    }
    if (!r->failed) {
      std::memcpy(r->result.data() + size_t(x.off) * 3 * K, b.h_out + x.out, size_t(x.cnt) * 3 * K * 4);
      stats.probes += x.cnt;
    }
    finalize(r);
  }
  if (!bad) stats.rays += b.rays;
  flight_bytes -= b.bytes;
  note_bytes();
  pinned_pool.push_back({b.h_out, b.h_cap});
  err_pool.push_back(b.h_err);
  event_pool.push_back(b.done);
  cv_done.notify_all();
}

void vlb_service::run() {
  cudaSetDevice(ctx->device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    // retire in stream order
    while (!inflight.empty()) {
      const cudaError_t q = cudaEventQuery(inflight.front().done);
      if (q == cudaErrorNotReady) break;
      if (q != cudaSuccess) {
        cudaGetLastError();
        for (Slice& x : inflight.front().slices) --x.r->pending;
        fail_slices(inflight.front().slices, VLB_ERR_CUDA, cudaGetErrorString(q));
        flight_bytes -= inflight.front().bytes;
        note_bytes();
      } else {
        retire(inflight.front(), lk);
      }
      inflight.pop_front();
    }
    // user-released sets: device copies go, the entry (host probes) stays
    for (auto& kv : sets)
      if (kv.second->dropped && kv.second->resident) free_set(*kv.second);
    note_bytes();
    if (!queue.empty() && inflight.size() < cfg.max_inflight && launch_next(lk)) continue;
    if (stop && queue.empty() && inflight.empty()) break;
    // wait for a submit or for the oldest batch (polled: new requests may arrive meanwhile)
    cv_work.wait_for(lk, std::chrono::microseconds(inflight.empty() ? 20000 : 50));
  }
  cudaStreamSynchronize(ctx->stream);
}

// ---- C ABI ---------------------------------------------------------------------------------
extern "C" {

vlb_status vlb_service_plan(const uint64_t* probes, const uint64_t* bytes, uint32_t n, uint64_t max_batch_probes,
                            uint64_t budget_bytes, uint32_t* out_batch, uint32_t* nbatches) {
  if ((!probes || !bytes || !out_batch) && n) return VLB_ERR_INVALID;
  if (!nbatches) return VLB_ERR_INVALID;
  uint32_t batch = 0;
  bool open = false;
  uint64_t cp = 0, cb = 0;
  for (uint32_t i = 0; i < n; ++i) {
    if (bytes[i] > budget_bytes) { out_batch[i] = UINT32_MAX; continue; }
    if (open && !joins(false, cp, cb, probes[i], bytes[i], max_batch_probes, budget_bytes)) {
      ++batch;
      cp = cb = 0;
    }
    out_batch[i] = batch;
    cp += probes[i];
    cb += bytes[i];
    open = true;
  }
  *nbatches = open ? batch + 1 : 0;
  return VLB_OK;
}

vlb_status vlb_service_create(vlb_ctx* ctx, const vlb_service_config* cfg, vlb_service** out) {
  if (!ctx || !out) return VLB_ERR_INVALID;
  *out = nullptr;
  vlb_service_config c = cfg ? *cfg : vlb_service_config{};
  if (c.lmax == 0) c.lmax = 2;
  if (c.lmax != 2 && c.lmax != 3) return sfail(VLB_ERR_INVALID, "service lmax must be 2 or 3");
  if (c.precision > VLB_PREC_BF16) return sfail(VLB_ERR_INVALID, "service precision must be a vlb_precision");
  if (!c.hbm_budget_bytes) c.hbm_budget_bytes = kDefaultBudget;
  if (!c.max_batch_probes) c.max_batch_probes = kDefaultMaxProbes;
  if (!c.max_inflight) c.max_inflight = kDefaultInflight;
  if (!c.slice_probes) c.slice_probes = kDefaultSlice;
  vlb_ctx* priv = nullptr;
  vlb_status st = vlb_ctx_create(ctx->device, &priv);
  if (st) return sfail(st, "service: private context creation failed");
  priv->parent = ctx;
  auto* s = new (std::nothrow) vlb_service();
  if (!s) { vlb_ctx_destroy(priv); return VLB_ERR_OOM; }
  s->user = ctx;
  s->ctx = priv;
  s->cfg = c;
  s->K = svc_k(c.lmax);
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return VLB_OK;
}

void vlb_service_destroy(vlb_service* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->ctx->device);
  for (auto& kv : s->sets) s->free_set(*kv.second);
  cudaStreamSynchronize(s->ctx->stream);
  for (auto& p : s->pinned_pool) cudaFreeHost(p.first);
  for (int* p : s->err_pool) cudaFreeHost(p);
  for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
  vlb_ctx_destroy(s->ctx);
  delete s;
}

vlb_status vlb_service_submit(vlb_service* s, const vlb_request* q, uint64_t* ticket) {
  if (!s || !q || !ticket) return VLB_ERR_INVALID;
  *ticket = 0;
  auto r = std::make_unique<Request>();
  if (!q->params || !q->params->dirs) return sfail(VLB_ERR_INVALID, "request params and dirs required");
  r->params = *q->params;
  r->relight_of = q->relight_of;
  r->keep = q->keep_hits != 0 && q->relight_of == 0;
  std::unique_lock<std::mutex> lk(s->mu);
  uint32_t n, S;
  if (q->relight_of) {
    auto it = s->sets.find(q->relight_of);
    if (it == s->sets.end()) return sfail(VLB_ERR_INVALID, "relight_of names no bake that keeps its hits");
    n = it->second->n;
    S = it->second->dirs->n;
    r->n = n;
  } else {
    if (!q->scene || (q->nprobes && !q->probe_xyz))
      return sfail(VLB_ERR_INVALID, "request needs a scene and probes");
    r->scene = q->scene;
    r->n = q->nprobes;
    r->probes.assign(q->probe_xyz, q->probe_xyz + size_t(q->nprobes) * 3);
    n = q->nprobes;
    S = q->params->dirs->n;
  }
  // parameter checks that the batch would otherwise report for the whole batch
  if (r->params.dirs->ctx != s->user || (r->params.sky && r->params.sky->ctx != s->user) ||
      (r->scene && r->scene->ctx != s->user))
    return sfail(VLB_ERR_INVALID, "request handles belong to another context");
  if (!(r->params.tmax > r->params.tmin) || r->params.tmin < 0.f)
    return sfail(VLB_ERR_INVALID, "bad ray interval");
  const double sl = double(r->params.sun_dir[0]) * r->params.sun_dir[0] +
                    double(r->params.sun_dir[1]) * r->params.sun_dir[1] + double(r->params.sun_dir[2]) * r->params.sun_dir[2];
  if (!(sl > 0.0)) return sfail(VLB_ERR_INVALID, "sun direction must be non-zero");
  uint64_t need = transient_bytes(n, S, s->K, s->cfg.precision) + (r->keep ? hitset_bytes(n, S) : 0);
  if (need > s->cfg.hbm_budget_bytes) {
    return sfail(VLB_ERR_OOM, "request exceeds the service's device-memory budget");
  }
  r->ticket = s->next_ticket++;
  r->t_submit = Clock::now();
  if (n == 0) {  // nothing to bake
    r->state = Request::kDone;
    ++s->stats.completed;
  }
  if (r->keep) {
    auto hs = std::make_unique<HitSet>();
    hs->scene = r->scene;
    hs->dirs = r->params.dirs;
    hs->tmin = r->params.tmin;
    hs->tmax = r->params.tmax;
    hs->n = n;
    hs->h_probes = r->probes;
    s->sets[r->ticket] = std::move(hs);
  }
  *ticket = r->ticket;
  ++s->stats.submitted;
  const bool queued = r->state == Request::kQueued;
  s->reqs[r->ticket] = std::move(r);
  if (queued) s->queue.push_back(*ticket);
  lk.unlock();
  s->cv_work.notify_one();
  return VLB_OK;
}

vlb_status vlb_service_wait(vlb_service* s, uint64_t ticket, uint32_t timeout_ms, float* out, double* latency_ms) {
  if (!s) return VLB_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(VLB_ERR_INVALID, "unknown or already collected ticket");
  Request* r = it->second.get();
  auto finished = [r] { return r->state == Request::kDone || r->state == Request::kFailed; };
  if (!finished()) {
    if (timeout_ms == 0 || !s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished))
      return VLB_ERR_TIMEOUT;
  }
  if (r->state == Request::kFailed) {
    const vlb_status st = r->status;
    const std::string msg = r->err;
    s->reqs.erase(it);
    return sfail(st, msg);
  }
  if (out && !r->result.empty()) std::memcpy(out, r->result.data(), r->result.size() * 4);
  if (latency_ms) *latency_ms = r->latency_ms;
  s->reqs.erase(it);
  return VLB_OK;
}

vlb_status vlb_service_release(vlb_service* s, uint64_t ticket) {
  if (!s) return VLB_ERR_INVALID;
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->sets.find(ticket);
    if (it == s->sets.end()) return sfail(VLB_ERR_INVALID, "ticket keeps no hits");
    it->second->dropped = true;
  }
  s->cv_work.notify_one();
  return VLB_OK;
}

const char* vlb_service_last_error(void) { return t_err.c_str(); }

vlb_status vlb_service_stats_read(vlb_service* s, vlb_service_stats* out) {
  if (!s || !out) return VLB_ERR_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->stats;
  return VLB_OK;
}

}  // extern "C"
