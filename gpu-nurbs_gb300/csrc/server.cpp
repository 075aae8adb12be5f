// Serving loop: continuous batching of point-inversion requests against a device-resident
// surface pool.  No counterpart in the reference (a one-shot program).
//
// Threads:
//  * scheduler — owns `slots` in-flight batches, each with its own CUDA stream, pinned host
//    staging and device buffers carved from the pool's budget.  In a loop it (1) retires slots
//    whose completion event fired, scattering uv/status/residual back to each request's host
//    buffers and releasing the requests, and (2) fills every free slot with the requests that
//    arrived meanwhile (FIFO, up to max_batch_queries), grouped by surface, then
//    H2D copy -> nurbs_pool_invert -> D2H copies -> event, all on the slot's stream.  Requests
//    arriving while batches run are admitted as soon as a slot frees: batches overlap on the GPU.
//  * uploader — converts uploaded surfaces into the pool on its own stream, all uploads queued
//    at that moment in one batch (nurbs_pool_add keeps the pool lock only to reserve and
//    publish, so inversions continue meanwhile).  When the budget is full it evicts
//    least-recently-used surfaces that no queued request references.
// Every wait is bounded; nothing spins on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <cstdlib>
#include <set>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gpu_nurbs.h"
#include "pool_internal.h"
#include "surface_host.h"

using namespace gnurbs;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
  uint64_t ticket = 0;
  int kind = 0;  // 0 invert, 1 upload
  int surf = -1;
  const double* P = nullptr;
  int64_t n = 0;
  double* uv = nullptr;
  int* status = nullptr;
  double* residual = nullptr;
  nurbs_surface_desc desc{};
  int* id_out = nullptr;
  double* latency_out = nullptr;
  Clock::time_point t_submit;
  int result = NURBS_OK;
  double latency_us = 0;
  bool done = false;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  cudaEvent_t begin = nullptr;  // timing: batch start on the slot's stream
  size_t off = 0, bytes = 0;
  char* dev = nullptr;
  double* hP = nullptr;
  double* huv = nullptr;
  int* hst = nullptr;
  double* hres = nullptr;
  std::vector<Request*> reqs;
  std::vector<int64_t> req_off;
  bool busy = false;
};

}  // namespace

struct nurbs_server_s {
  nurbs_pool_t pool = nullptr;
  nurbs_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_work;   // scheduler / uploader wake-up
  std::condition_variable cv_done;   // waiters on completions
  std::deque<Request*> incoming;     // invert requests not yet taken by the scheduler
  std::deque<Request*> uploads;      // upload requests
  std::unordered_map<uint64_t, Request*> live;  // submitted and not yet released by poll/wait
  std::vector<uint64_t> completed;   // tickets completed and not yet polled
  std::unordered_map<int, int> refs;            // surface id -> queued/in-flight requests
  std::unordered_map<int, Clock::time_point> last_use;
  std::vector<Slot> slots;
  std::thread sched, uploader;
  std::atomic<bool> stop{false};
  std::atomic<bool> paused{false};
  cudaStream_t up_stream = nullptr;
  uint64_t next_ticket = 1;
  int64_t n_batches = 0, n_batch_queries = 0, n_completed = 0;
  int in_flight_requests = 0;
  double gpu_ms = 0, dispatch_us = 0, retire_us = 0;
};

namespace {

void complete(nurbs_server_s* S, Request* r, int result) {
  // called with S->mu held
  r->result = result;
  r->done = true;
  r->latency_us = std::chrono::duration<double, std::micro>(Clock::now() - r->t_submit).count();
  if (r->latency_out) *r->latency_out = r->latency_us;
  S->completed.push_back(r->ticket);
  S->n_completed++;
  S->in_flight_requests--;
  if (r->kind == 0) {
    auto it = S->refs.find(r->surf);
    if (it != S->refs.end() && --it->second == 0) S->refs.erase(it);
    S->last_use[r->surf] = Clock::now();
  }
}

void retire(nurbs_server_s* S, Slot& sl, int result) {
  const Clock::time_point t0 = Clock::now();
  float ms = 0;
  if (result == NURBS_OK) cudaEventElapsedTime(&ms, sl.begin, sl.done);
  int64_t o = 0;
  for (size_t k = 0; k < sl.reqs.size(); ++k) {
    Request* r = sl.reqs[k];
    o = sl.req_off[k];
    if (result == NURBS_OK) {
      std::memcpy(r->uv, sl.huv + 2 * o, r->n * 2 * sizeof(double));
      std::memcpy(r->status, sl.hst + o, r->n * sizeof(int));
      std::memcpy(r->residual, sl.hres + o, r->n * sizeof(double));
    }
  }
  std::lock_guard<std::mutex> lock(S->mu);
  for (Request* r : sl.reqs) complete(S, r, result);
  sl.reqs.clear();
  sl.req_off.clear();
  sl.busy = false;
  S->gpu_ms += ms;
  S->retire_us += std::chrono::duration<double, std::micro>(Clock::now() - t0).count();
  S->cv_done.notify_all();
}

// Fills a free slot from the pending queue; returns true if a batch was launched.
bool dispatch(nurbs_server_s* S, Slot& sl, std::deque<Request*>& pending) {
  const Clock::time_point t0 = Clock::now();
  const int64_t cap = S->cfg.max_batch_queries;
  int64_t total = 0;
  while (!pending.empty() && total + pending.front()->n <= cap &&
         (int)sl.reqs.size() < S->cfg.max_batch_requests) {
    sl.reqs.push_back(pending.front());
    total += pending.front()->n;
    pending.pop_front();
  }
  if (sl.reqs.empty()) return false;
  // group by surface (stable), lay queries out contiguously per surface
  std::stable_sort(sl.reqs.begin(), sl.reqs.end(), [](const Request* a, const Request* b) { return a->surf < b->surf; });
  std::vector<int> ids;
  std::vector<int64_t> offs;
  sl.req_off.resize(sl.reqs.size());
  int64_t o = 0;
  for (size_t k = 0; k < sl.reqs.size(); ++k) {
    Request* r = sl.reqs[k];
    if (ids.empty() || ids.back() != r->surf) {
      ids.push_back(r->surf);
      offs.push_back(o);
    }
    sl.req_off[k] = o;
    std::memcpy(sl.hP + 3 * o, r->P, r->n * 3 * sizeof(double));
    o += r->n;
  }
  offs.push_back(o);
  const int64_t cap3 = cap;
  double* dP = (double*)sl.dev;
  double* duv = (double*)(sl.dev + align256(cap3 * 24));
  int* dst = (int*)(sl.dev + align256(cap3 * 24) + align256(cap3 * 16));
  double* dres = (double*)(sl.dev + align256(cap3 * 24) + align256(cap3 * 16) + align256(cap3 * 4));
  cudaError_t e = cudaEventRecord(sl.begin, sl.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dP, sl.hP, o * 24, cudaMemcpyHostToDevice, sl.stream);
  int rc = e == cudaSuccess ? NURBS_OK : NURBS_E_CUDA;
  if (rc == NURBS_OK)
    rc = nurbs_pool_invert(S->pool, (int)ids.size(), ids.data(), offs.data(), dP, duv, dst, dres, S->cfg.precision,
                           sl.stream);
  if (rc == NURBS_OK) {
    e = cudaMemcpyAsync(sl.huv, duv, o * 16, cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.hst, dst, o * 4, cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.hres, dres, o * 8, cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, sl.stream);
    if (e != cudaSuccess) rc = NURBS_E_CUDA;
  }
  if (rc != NURBS_OK) {
    cudaStreamSynchronize(sl.stream);
    retire(S, sl, rc);
    return false;
  }
  sl.busy = true;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->n_batches++;
    S->n_batch_queries += o;
    S->dispatch_us += std::chrono::duration<double, std::micro>(Clock::now() - t0).count();
  }
  return true;
}

constexpr int kPollUs = 20;  // the scheduler's sleep between polls of the in-flight batches

void scheduler_main(nurbs_server_s* S) {
  std::deque<Request*> pending;
  while (!S->stop.load()) {
    {
      std::unique_lock<std::mutex> lock(S->mu);
      bool any_busy = false;
      for (auto& sl : S->slots) any_busy |= sl.busy;
      if (S->incoming.empty() && pending.empty() && !any_busy)
        S->cv_work.wait_for(lock, std::chrono::microseconds(500));
      while (!S->incoming.empty()) {
        pending.push_back(S->incoming.front());
        S->incoming.pop_front();
      }
    }
    bool progress = false;
    for (auto& sl : S->slots) {
      if (!sl.busy) continue;
      cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaSuccess) {
        retire(S, sl, NURBS_OK);
        progress = true;
      } else if (q != cudaErrorNotReady) {
        retire(S, sl, NURBS_E_CUDA);
        progress = true;
      }
    }
    if (!S->paused.load())
      for (auto& sl : S->slots)
        if (!sl.busy && !pending.empty()) progress |= dispatch(S, sl, pending);
    if (!progress) {
      // Batches in flight and nothing to start: sleep until a request arrives (submit notifies
      // cv_work) or kPollUs passes, then poll the slots' events again.  A bounded wait: the
      // thread does not spin on a host core, and a completion is seen within kPollUs (plus the
      // timer's slack) of the GPU finishing.
      std::unique_lock<std::mutex> lock(S->mu);
      if (S->incoming.empty() && !S->stop.load()) S->cv_work.wait_for(lock, std::chrono::microseconds(kPollUs));
    }
  }
  // shutdown: finish what is in flight, fail what never started
  for (auto& sl : S->slots)
    if (sl.busy) {
      cudaStreamSynchronize(sl.stream);
      retire(S, sl, NURBS_OK);
    }
  std::lock_guard<std::mutex> lock(S->mu);
  for (Request* r : pending) complete(S, r, NURBS_E_STATE);
  for (Request* r : S->incoming) complete(S, r, NURBS_E_STATE);
  S->incoming.clear();
  S->cv_done.notify_all();
}

// One upload with LRU eviction when the budget is full.
int upload_one(nurbs_server_s* S, Request* r, int* id) {
  int rc = nurbs_pool_add(S->pool, 1, &r->desc, S->up_stream, id);
  while (rc == NURBS_E_BUDGET) {
    // Evict the least recently used surface no queued request references.  The choice and the
    // release happen under one hold of S->mu, the lock nurbs_server_submit_invert takes to check
    // that a surface is live and to count its reference: no request can reference the victim
    // between the check and the release (lock order S->mu, then the pool's lock, as in submit).
    int victim = -1;
    int released = NURBS_E_INVALID;
    {
      std::lock_guard<std::mutex> lock(S->mu);
      Clock::time_point oldest = Clock::time_point::max();
      for (auto& kv : S->last_use)
        if (!S->refs.count(kv.first) && kv.second < oldest) {
          oldest = kv.second;
          victim = kv.first;
        }
      if (victim >= 0) {
        S->last_use.erase(victim);
        released = pool_release_surface(S->pool, victim);
      }
    }
    if (victim < 0 || released != NURBS_OK) break;
    rc = nurbs_pool_add(S->pool, 1, &r->desc, S->up_stream, id);
  }
  return rc;
}

void uploader_main(nurbs_server_s* S) {
  constexpr int kMaxBatch = 64;  // uploads converted together (one copy, one launch per stage)
  std::vector<Request*> batch;
  std::vector<nurbs_surface_desc> descs;
  std::vector<int> ids;
  while (!S->stop.load()) {
    batch.clear();
    {
      std::unique_lock<std::mutex> lock(S->mu);
      S->cv_work.wait_for(lock, std::chrono::milliseconds(2), [&] { return !S->uploads.empty() || S->stop.load(); });
      while (!S->uploads.empty() && (int)batch.size() < kMaxBatch) {
        batch.push_back(S->uploads.front());
        S->uploads.pop_front();
      }
    }
    if (batch.empty()) continue;
    descs.resize(batch.size());
    ids.assign(batch.size(), -1);
    for (size_t k = 0; k < batch.size(); ++k) descs[k] = batch[k]->desc;
    std::vector<int> rcs(batch.size(), NURBS_OK);
    int rc = nurbs_pool_add(S->pool, (int)batch.size(), descs.data(), S->up_stream, ids.data());
    if (rc != NURBS_OK) {
      // a refusal of the whole batch (budget, or one invalid surface): one at a time, evicting
      for (size_t k = 0; k < batch.size(); ++k) rcs[k] = upload_one(S, batch[k], &ids[k]);
    }
    std::lock_guard<std::mutex> lock(S->mu);
    for (size_t k = 0; k < batch.size(); ++k) {
      Request* r = batch[k];
      if (rcs[k] == NURBS_OK) {
        r->surf = ids[k];
        if (r->id_out) *r->id_out = ids[k];
        S->last_use[ids[k]] = Clock::now();
      }
      complete(S, r, rcs[k]);
    }
    S->cv_done.notify_all();
  }
  std::lock_guard<std::mutex> lock(S->mu);
  for (Request* r : S->uploads) complete(S, r, NURBS_E_STATE);
  S->uploads.clear();
}

// Servers still alive at process exit are stopped by an exit handler: their threads call into
// the CUDA runtime, which tears itself down at exit (its handler was registered earlier, so it
// runs after this one).
std::mutex g_servers_mu;
std::set<nurbs_server_s*> g_servers;
bool g_exit_hook = false;

void stop_threads(nurbs_server_s* S) {
  S->stop.store(true);
  S->cv_work.notify_all();
  if (S->sched.joinable()) S->sched.join();
  if (S->uploader.joinable()) S->uploader.join();
}

void stop_all_servers_at_exit() {
  std::lock_guard<std::mutex> lock(g_servers_mu);
  for (nurbs_server_s* S : g_servers) stop_threads(S);
}

void free_slots(nurbs_server_s* S) {
  for (auto& sl : S->slots) {
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.begin) cudaEventDestroy(sl.begin);
    if (sl.hP) cudaFreeHost(sl.hP);
    if (sl.huv) cudaFreeHost(sl.huv);
    if (sl.hst) cudaFreeHost(sl.hst);
    if (sl.hres) cudaFreeHost(sl.hres);
    if (sl.dev) pool_arena_release(S->pool, sl.off, sl.bytes);
  }
  S->slots.clear();
}

}  // namespace

extern "C" {

int nurbs_server_create(nurbs_pool_t pool, const nurbs_server_config* cfg, nurbs_server_t* out) {
  if (!pool || !cfg || !out) return NURBS_E_INVALID;
  *out = nullptr;
  if (cfg->slots < 1 || cfg->slots > 16 || cfg->max_batch_queries < 32 || cfg->max_batch_requests < 1 ||
      (cfg->precision != NURBS_PREC_FP64 && cfg->precision != NURBS_PREC_MIXED))
    return NURBS_E_INVALID;
  nurbs_server_s* S = new (std::nothrow) nurbs_server_s();
  if (!S) return NURBS_E_NOMEM;
  S->pool = pool;
  S->cfg = *cfg;
  const int64_t cap = cfg->max_batch_queries;
  S->slots.resize(cfg->slots);
  int rc = NURBS_OK;
  for (auto& sl : S->slots) {
    sl.bytes = align256(cap * 24) + align256(cap * 16) + align256(cap * 4) + align256(cap * 8);
    sl.dev = pool_arena_alloc(pool, sl.bytes, &sl.off);
    if (!sl.dev) {
      rc = NURBS_E_BUDGET;
      break;
    }
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&sl.done) != cudaSuccess || cudaEventCreate(&sl.begin) != cudaSuccess ||
        cudaMallocHost((void**)&sl.hP, cap * 24) != cudaSuccess ||
        cudaMallocHost((void**)&sl.huv, cap * 16) != cudaSuccess ||
        cudaMallocHost((void**)&sl.hst, cap * 4) != cudaSuccess ||
        cudaMallocHost((void**)&sl.hres, cap * 8) != cudaSuccess) {
      rc = NURBS_E_NOMEM;
      break;
    }
  }
  if (rc == NURBS_OK && cudaStreamCreateWithFlags(&S->up_stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = NURBS_E_CUDA;
  if (rc != NURBS_OK) {
    free_slots(S);
    delete S;
    return rc;
  }
  S->sched = std::thread(scheduler_main, S);
  S->uploader = std::thread(uploader_main, S);
  {
    std::lock_guard<std::mutex> lock(g_servers_mu);
    if (!g_exit_hook) {
      std::atexit(stop_all_servers_at_exit);
      g_exit_hook = true;
    }
    g_servers.insert(S);
  }
  *out = S;
  return NURBS_OK;
}

int nurbs_server_destroy(nurbs_server_t S) {
  if (!S) return NURBS_OK;
  {
    std::lock_guard<std::mutex> lock(g_servers_mu);
    g_servers.erase(S);
  }
  stop_threads(S);
  if (S->up_stream) cudaStreamDestroy(S->up_stream);
  free_slots(S);
  for (auto& kv : S->live) delete kv.second;
  delete S;
  return NURBS_OK;
}

int nurbs_server_submit_invert(nurbs_server_t S, int surf_id, const double* P_host, int64_t n, double* uv_host,
                               int* status_host, double* residual_host, double* latency_us_out, uint64_t* ticket) {
  if (!S || !ticket || n < 0 || (n > 0 && (!P_host || !uv_host || !status_host || !residual_host))) return NURBS_E_INVALID;
  if (n > S->cfg.max_batch_queries) return NURBS_E_UNSUPPORTED;
  Request* r = new (std::nothrow) Request();
  if (!r) return NURBS_E_NOMEM;
  r->kind = 0;
  r->surf = surf_id;
  r->P = P_host;
  r->n = n;
  r->uv = uv_host;
  r->status = status_host;
  r->residual = residual_host;
  r->latency_out = latency_us_out;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->stop.load()) {
      delete r;
      return NURBS_E_STATE;
    }
    if (!pool_is_live(S->pool, surf_id)) {
      delete r;
      return NURBS_E_INVALID;
    }
    r->ticket = S->next_ticket++;
    S->live[r->ticket] = r;
    S->refs[surf_id]++;
    S->in_flight_requests++;
    if (n == 0) {
      complete(S, r, NURBS_OK);
    } else {
      S->incoming.push_back(r);
    }
    *ticket = r->ticket;
  }
  S->cv_work.notify_all();
  return NURBS_OK;
}

int nurbs_server_submit_upload(nurbs_server_t S, const nurbs_surface_desc* desc, int* surf_id_out,
                               double* latency_us_out, uint64_t* ticket) {
  if (!S || !desc || !ticket) return NURBS_E_INVALID;
  Request* r = new (std::nothrow) Request();
  if (!r) return NURBS_E_NOMEM;
  r->kind = 1;
  r->desc = *desc;
  r->id_out = surf_id_out;
  r->latency_out = latency_us_out;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->stop.load()) {
      delete r;
      return NURBS_E_STATE;
    }
    r->ticket = S->next_ticket++;
    S->live[r->ticket] = r;
    S->in_flight_requests++;
    S->uploads.push_back(r);
    *ticket = r->ticket;
  }
  S->cv_work.notify_all();
  return NURBS_OK;
}

int nurbs_server_wait(nurbs_server_t S, uint64_t ticket, int timeout_ms, int* result) {
  if (!S) return NURBS_E_INVALID;
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->live.find(ticket);
  if (it == S->live.end()) return NURBS_E_INVALID;
  Request* r = it->second;
  if (!S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms), [&] { return r->done; }))
    return NURBS_E_TIMEOUT;
  if (result) *result = r->result;
  S->live.erase(it);
  S->completed.erase(std::remove(S->completed.begin(), S->completed.end(), ticket), S->completed.end());
  delete r;
  return NURBS_OK;
}

int nurbs_server_poll(nurbs_server_t S, uint64_t* tickets, int* results, int max, int* count) {
  if (!S || !count || max < 0 || (max > 0 && (!tickets || !results))) return NURBS_E_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  int c = 0;
  while (c < max && !S->completed.empty()) {
    uint64_t t = S->completed.front();
    S->completed.erase(S->completed.begin());
    auto it = S->live.find(t);
    if (it == S->live.end()) continue;
    tickets[c] = t;
    results[c] = it->second->result;
    delete it->second;
    S->live.erase(it);
    ++c;
  }
  *count = c;
  return NURBS_OK;
}

int nurbs_server_drain(nurbs_server_t S, int timeout_ms) {
  if (!S) return NURBS_E_INVALID;
  std::unique_lock<std::mutex> lock(S->mu);
  if (!S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                           [&] { return S->in_flight_requests == 0; }))
    return NURBS_E_TIMEOUT;
  return NURBS_OK;
}

int nurbs_server_pause(nurbs_server_t S, int paused) {
  if (!S) return NURBS_E_INVALID;
  S->paused.store(paused != 0);
  S->cv_work.notify_all();
  return NURBS_OK;
}

int nurbs_server_stats(nurbs_server_t S, nurbs_server_stats_t* st) {
  if (!S || !st) return NURBS_E_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  st->completed = S->n_completed;
  st->batches = S->n_batches;
  st->batch_queries = S->n_batch_queries;
  st->in_flight = S->in_flight_requests;
  st->gpu_ms = S->gpu_ms;
  st->dispatch_us = S->dispatch_us;
  st->retire_us = S->retire_us;
  return NURBS_OK;
}

// Replays a request trace with native timing: request i is submitted at arrival_us[i] after the
// start (busy-waiting on the clock between arrivals).  kind[i] 0 = inversion of the queries
// [qoff[i], qoff[i+1]) of P against surf[i]; 1 = upload of uploads[upload_index[i]].  Latency
// counts from the scheduled arrival time, so a generator that falls behind does not hide queueing.
int nurbs_server_replay(nurbs_server_t S, int nreq, const double* arrival_us, const int* kind, const int* surf,
                        const int64_t* qoff, const double* P, double* uv, int* status, double* residual,
                        const nurbs_surface_desc* uploads, const int* upload_index, int* upload_ids, double* latency_us,
                        int* results, int timeout_ms) {
  if (!S || nreq < 0 || !arrival_us || !kind || !qoff || !latency_us || !results) return NURBS_E_INVALID;
  std::vector<uint64_t> tickets(nreq, 0);
  const Clock::time_point t0 = Clock::now();
  for (int i = 0; i < nreq; ++i) {
    const Clock::time_point due = t0 + std::chrono::nanoseconds((int64_t)(arrival_us[i] * 1e3));
    while (Clock::now() < due) {
    }
    int rc;
    if (kind[i] == 0) {
      int64_t a = qoff[i], b = qoff[i + 1];
      rc = nurbs_server_submit_invert(S, surf[i], P + 3 * a, b - a, uv + 2 * a, status + a, residual + a,
                                      &latency_us[i], &tickets[i]);
    } else {
      if (!uploads || !upload_index || !upload_ids) return NURBS_E_INVALID;
      rc = nurbs_server_submit_upload(S, &uploads[upload_index[i]], &upload_ids[upload_index[i]], &latency_us[i],
                                      &tickets[i]);
    }
    if (rc != NURBS_OK) {
      results[i] = rc;
      tickets[i] = 0;
      continue;
    }
    // latency from the scheduled arrival
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->live.find(tickets[i]);
    if (it != S->live.end() && !it->second->done) it->second->t_submit = due;
  }
  int rc = nurbs_server_drain(S, timeout_ms);
  for (int i = 0; i < nreq; ++i) {
    if (!tickets[i]) continue;
    int res = NURBS_E_TIMEOUT;
    if (nurbs_server_wait(S, tickets[i], 0, &res) != NURBS_OK) res = NURBS_E_TIMEOUT;
    results[i] = res;
  }
  return rc;
}

}  // extern "C"
