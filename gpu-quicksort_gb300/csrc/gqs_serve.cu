// The sort server (gqs_srv_* in include/gqs.h): continuous batching of sort requests of mixed
// size and key type on one GPU.
//
// No counterpart in the reference, which sorts one array per blocking call
// (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:835-906, driven by big_test<T> at 1192-1194). This
// is the serving form of the same sort path:
//
//   submit  -> pending (FIFO)
//   admit   -> when the request fits in the free part of the device arena (the memory budget):
//              space is taken for its keys and scratch and its keys are copied to the device at
//              once on the copy stream, so queued arrays wait on the device, not on the host
//   launch  -> whenever one of the lanes (batches in flight) is free: every resident request of
//              one key type, up to the batch limits, becomes one segment of one replay of the
//              lane's graph-captured segmented sort (gqs_graph.h); results are copied back on the
//              lane's stream
//   retire  -> a host function queued after the copies marks the batch finished; the dispatcher
//              frees its arena space and completes its requests
//
// Requests that arrive while batches run are admitted as memory frees up and launched as lanes
// free up, so their copies and sorts overlap the running work on the device. Segments of one
// batch never interact: each request's result is the same alone or in any mix.
//
// per_request mode is the comparison baseline: one request at a time through the plain context
// sort (copy in, gqs_sort_<type>_dev, copy out, wait), exactly what a caller looping over
// gqs_sort_<type> does.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gqs.h"
#include "gqs_arena.h"
#include "gqs_graph.h"
#include "gqs_host.h"

namespace {

uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

using gqs::ArenaAlloc;

struct Req {
  uint64_t id = 0;
  int dtype = 0;
  const void* in = nullptr;
  void* out = nullptr;
  size_t n = 0;
  size_t off = 0;      // arena byte offset once admitted
  uint64_t round = 0;  // admission round whose copy event covers its keys
  bool staged_out = false;  // out is pageable: copied back synchronously at retire
  gqs_request_info info{};
  bool done = false;
};

struct Round {
  cudaEvent_t ev = nullptr;
  uint32_t refs = 0;  // admitted requests of this round not yet launched
};

struct Lane {
  int index = 0;
  cudaStream_t stream = nullptr;
  std::unique_ptr<gqs::GraphSort> gs;
  std::vector<Req*> reqs;
  bool busy = false;
  bool finished = false;  // set by the host function at the end of the lane's work
  gqs_status launch_status = GQS_OK;
  struct gqs_server* srv = nullptr;
};

}  // namespace

struct gqs_server {
  int device = 0;
  int num_sms = 0;
  gqs_server_config cfg{};
  int variant[3] = {0, 0, 0};
  // device memory
  char* keys = nullptr;     // arena of arena_bytes
  char* scratch = nullptr;  // same layout
  size_t arena_bytes = 0;
  ArenaAlloc arena;
  cudaStream_t copy_stream = nullptr;
  std::vector<std::unique_ptr<Lane>> lanes;
  gqs_ctx* plain = nullptr;  // per_request mode
  // requests
  std::mutex mu;
  std::condition_variable cv_work;  // dispatcher: submissions, finished lanes, stop
  std::condition_variable cv_done;  // clients: completions
  std::deque<Req*> pending;
  std::deque<Req*> admitted[3];
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
  std::deque<uint64_t> completed;  // completion order, for wait_any
  std::map<uint64_t, Round> rounds;
  uint64_t next_id = 1, next_round = 1;
  uint64_t outstanding = 0;  // submitted, not yet completed
  bool stop = false;
  bool submitted = false;  // a request arrived since the dispatcher last looked
  gqs_status fatal = GQS_OK;
  gqs_server_stats stats{};
  std::thread dispatcher;
};

namespace {

void CUDART_CB lane_finished(void* p) {
  Lane* l = static_cast<Lane*>(p);
  gqs_server* s = l->srv;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    l->finished = true;
  }
  s->cv_work.notify_one();
}

void complete_locked(gqs_server* s, Req* r, gqs_status st) {
  r->info.status = (uint32_t)st;
  r->info.t_done_ns = now_ns();
  r->done = true;
  s->completed.push_back(r->id);
  --s->outstanding;
  ++s->stats.completed;
  if (st == GQS_OK) s->stats.completed_keys += r->n;
  if (st != GQS_OK && st != GQS_ERR_CANCELLED) ++s->stats.failed;
}

// Dispatcher: retire finished lanes. Lock held.
void retire_locked(gqs_server* s) {
  for (auto& lp : s->lanes) {
    Lane& l = *lp;
    if (!l.busy || !l.finished) continue;
    gqs_status st = l.launch_status;
    if (st == GQS_OK) {
      if (s->cfg.per_request) {
        gqs_stats ks{};
        st = gqs_last_stats(s->plain, &ks);
      } else {
        st = (gqs_status)l.gs->result().status;
      }
    }
    for (Req* r : l.reqs) {
      if (r->staged_out && st == GQS_OK) {
        const size_t es = gqs::kElemSize[r->dtype];
        cudaError_t e = cudaMemcpy(r->out, s->keys + r->off, r->n * es, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = gqs::cuda_status(e);
      }
      s->arena.release(r->off, r->n * gqs::kElemSize[r->dtype]);
      complete_locked(s, r, st);
    }
    l.reqs.clear();
    l.busy = false;
    l.finished = false;
  }
  s->stats.arena_used = s->arena.used();
  s->cv_done.notify_all();
}

// Dispatcher: move pending requests onto the device while the arena has room (FIFO: the
// oldest request that does not fit holds back the later ones). Lock held.
void admit_locked(gqs_server* s) {
  if (s->cfg.per_request) {  // the plain path copies at launch
    while (!s->pending.empty()) {
      Req* r = s->pending.front();
      size_t off = 0;
      if (!s->arena.alloc(r->n * gqs::kElemSize[r->dtype], &off)) break;
      r->off = off;
      r->info.t_admit_ns = now_ns();
      s->admitted[r->dtype].push_back(r);
      s->pending.pop_front();
    }
    return;
  }
  std::vector<Req*> batch;
  while (!s->pending.empty()) {
    Req* r = s->pending.front();
    size_t off = 0;
    if (!s->arena.alloc(r->n * gqs::kElemSize[r->dtype], &off)) break;
    r->off = off;
    batch.push_back(r);
    s->pending.pop_front();
  }
  if (batch.empty()) return;
  const uint64_t round = s->next_round++;
  Round rd;
  gqs_status st = gqs::cuda_status(cudaEventCreateWithFlags(&rd.ev, cudaEventDisableTiming));
  for (Req* r : batch) {
    const size_t es = gqs::kElemSize[r->dtype];
    if (st == GQS_OK)
      st = gqs::cuda_status(
          cudaMemcpyAsync(s->keys + r->off, r->in, r->n * es, cudaMemcpyHostToDevice, s->copy_stream));
  }
  if (st == GQS_OK) st = gqs::cuda_status(cudaEventRecord(rd.ev, s->copy_stream));
  const uint64_t t = now_ns();
  for (Req* r : batch) {
    if (st != GQS_OK) {
      s->arena.release(r->off, r->n * gqs::kElemSize[r->dtype]);
      complete_locked(s, r, st);
      continue;
    }
    r->round = round;
    r->info.t_admit_ns = t;
    s->admitted[r->dtype].push_back(r);
    ++rd.refs;
  }
  if (rd.refs) s->rounds[round] = rd;
  else if (rd.ev) cudaEventDestroy(rd.ev);
  if (st != GQS_OK) {
    s->fatal = st;
    s->cv_done.notify_all();
  }
  s->stats.arena_used = s->arena.used();
  s->stats.arena_peak = std::max(s->stats.arena_peak, s->stats.arena_used);
}

// The key type whose oldest resident request is oldest, or -1.
int pick_dtype_locked(gqs_server* s) {
  int best = -1;
  uint64_t t = 0;
  for (int d = 0; d < 3; ++d) {
    if (s->admitted[d].empty()) continue;
    const uint64_t id = s->admitted[d].front()->id;
    if (best < 0 || id < t) {
      best = d;
      t = id;
    }
  }
  return best;
}

gqs_status launch_plain(gqs_server* s, Lane& l, Req* r) {
  const size_t es = gqs::kElemSize[r->dtype];
  void* d = s->keys + r->off;
  void* dn = s->scratch + r->off;
  cudaError_t e = cudaMemcpyAsync(d, r->in, r->n * es, cudaMemcpyHostToDevice, l.stream);
  if (e != cudaSuccess) return gqs::cuda_status(e);
  gqs_status st;
  switch (r->dtype) {
    case GQS_U32:
      st = gqs_sort_u32_dev(s->plain, (uint32_t*)d, (uint32_t*)dn, r->n, l.stream);
      break;
    case GQS_F32:
      st = gqs_sort_f32_dev(s->plain, (float*)d, (float*)dn, r->n, l.stream);
      break;
    default:
      st = gqs_sort_f64_dev(s->plain, (double*)d, (double*)dn, r->n, l.stream);
      break;
  }
  if (st != GQS_OK) return st;
  if (!r->staged_out) {
    e = cudaMemcpyAsync(r->out, d, r->n * es, cudaMemcpyDeviceToHost, l.stream);
    if (e != cudaSuccess) return gqs::cuda_status(e);
  }
  return GQS_OK;
}

gqs_status launch_batch(gqs_server* s, Lane& l, int dtype, cudaEvent_t wait_ev) {
  const size_t es = gqs::kElemSize[dtype];
  if (wait_ev) {
    cudaError_t e = cudaStreamWaitEvent(l.stream, wait_ev, 0);
    if (e != cudaSuccess) return gqs::cuda_status(e);
  }
  unsigned long long* t = l.gs->table();
  for (size_t i = 0; i < l.reqs.size(); ++i) {
    const unsigned long long b = l.reqs[i]->off / es;
    t[2 * i] = b;
    t[2 * i + 1] = b + l.reqs[i]->n;
  }
  gqs_status st = l.gs->launch(dtype, s->variant[dtype], l.reqs.size(), l.stream);
  if (st != GQS_OK) return st;
  for (Req* r : l.reqs) {
    if (r->staged_out) continue;
    cudaError_t e = cudaMemcpyAsync(r->out, s->keys + r->off, r->n * es, cudaMemcpyDeviceToHost, l.stream);
    if (e != cudaSuccess) return gqs::cuda_status(e);
  }
  return GQS_OK;
}

// Dispatcher: fill free lanes. Called with the lock held; drops it around CUDA calls.
void launch_locked(gqs_server* s, std::unique_lock<std::mutex>& lk) {
  for (auto& lp : s->lanes) {
    Lane& l = *lp;
    if (l.busy) continue;
    const int dtype = pick_dtype_locked(s);
    if (dtype < 0) return;
    // take resident requests of that type, oldest first, up to the batch limits
    std::deque<Req*>& q = s->admitted[dtype];
    const size_t max_req = s->cfg.per_request ? 1 : s->cfg.batch_segments;
    uint64_t keys = 0, round = 0;
    while (!q.empty() && l.reqs.size() < max_req) {
      Req* r = q.front();
      if (!l.reqs.empty() && keys + r->n > s->cfg.batch_keys) break;
      keys += r->n;
      round = std::max(round, r->round);
      l.reqs.push_back(r);
      q.pop_front();
    }
    cudaEvent_t wait_ev = nullptr;
    if (round) {
      auto it = s->rounds.find(round);
      if (it != s->rounds.end()) wait_ev = it->second.ev;
    }
    const uint64_t t = now_ns();
    for (Req* r : l.reqs) {
      r->info.t_launch_ns = t;
      r->info.lane = (uint32_t)l.index;
      r->info.batch_requests = (uint32_t)l.reqs.size();
    }
    l.busy = true;
    l.finished = false;
    ++s->stats.batches;
    s->stats.max_batch_requests = std::max<uint64_t>(s->stats.max_batch_requests, l.reqs.size());
    lk.unlock();
    gqs_status st = s->cfg.per_request ? launch_plain(s, l, l.reqs[0]) : launch_batch(s, l, dtype, wait_ev);
    if (st == GQS_OK) st = gqs::cuda_status(cudaLaunchHostFunc(l.stream, lane_finished, &l));
    lk.lock();
    l.launch_status = st;
    if (st != GQS_OK) {
      // nothing is queued behind a failed launch that will signal: wait for the stream here
      lk.unlock();
      cudaStreamSynchronize(l.stream);
      lk.lock();
      l.finished = true;
      if (st == GQS_ERR_CUDA) s->fatal = st;
    }
    // rounds whose requests are all launched can go
    for (Req* r : l.reqs) {
      auto it = s->rounds.find(r->round);
      if (it != s->rounds.end() && --it->second.refs == 0) {
        cudaEventDestroy(it->second.ev);  // the stream wait above already captured it
        s->rounds.erase(it);
      }
    }
  }
}

bool lanes_idle_locked(gqs_server* s) {
  for (auto& l : s->lanes)
    if (l->busy) return false;
  return true;
}

void dispatcher_main(gqs_server* s) {
  gqs::DeviceGuard dg(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    retire_locked(s);
    if (s->fatal == GQS_OK) {
      admit_locked(s);
      launch_locked(s, lk);
    } else {
      // fail everything not on the GPU
      for (int d = 0; d < 3; ++d) {
        for (Req* r : s->admitted[d]) {
          s->arena.release(r->off, r->n * gqs::kElemSize[r->dtype]);
          complete_locked(s, r, s->fatal);
        }
        s->admitted[d].clear();
      }
      for (Req* r : s->pending) complete_locked(s, r, s->fatal);
      s->pending.clear();
      s->cv_done.notify_all();
    }
    const bool idle = lanes_idle_locked(s);
    if (s->stop && idle && s->pending.empty() && s->admitted[0].empty() && s->admitted[1].empty() &&
        s->admitted[2].empty())
      break;
    // sleep until a submission, a finished lane, or stop with nothing left on the GPU
    s->cv_work.wait(lk, [s] {
      for (auto& l : s->lanes)
        if (l->busy && l->finished) return true;
      return s->submitted || (s->stop && lanes_idle_locked(s));
    });
    s->submitted = false;
  }
}

}  // namespace

extern "C" {

void gqs_srv_config_default(gqs_server_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->budget_bytes = 64ull << 30;
  c->batch_keys = 1ull << 27;
  c->batch_segments = 4096;
  c->lanes = 3;
  c->timeout_ms = 4000;
  c->per_request = 0;
  c->variant[0] = c->variant[1] = c->variant[2] = -1;
}

uint64_t gqs_srv_now_ns(void) { return now_ns(); }

gqs_status gqs_srv_create(int device, const gqs_server_config* cfg, gqs_server** out) {
  if (!out) return GQS_ERR_INVALID;
  *out = nullptr;
  int num_sms = 0;
  gqs_status st = gqs::check_device(device, &num_sms);
  if (st != GQS_OK) return st;
  gqs_server_config c;
  gqs_srv_config_default(&c);
  if (cfg) c = *cfg;
  if (!c.budget_bytes) c.budget_bytes = 64ull << 30;
  if (!c.batch_keys) c.batch_keys = 1ull << 27;
  if (!c.batch_segments) c.batch_segments = 4096;
  if (!c.lanes) c.lanes = 3;
  if (c.per_request) {
    c.lanes = 1;
    c.batch_segments = 1;
  }
  if (c.lanes > 16 || c.batch_keys >= (1ull << 34) || c.batch_segments > (1u << 20)) return GQS_ERR_INVALID;
  gqs_server* s = new (std::nothrow) gqs_server();
  if (!s) return GQS_ERR_NOMEM;
  s->device = device;
  s->num_sms = num_sms;
  s->cfg = c;
  for (int t = 0; t < 3; ++t) {
    const int v = c.variant[t];
    s->variant[t] = (v >= 0 && v < gqs::variant_count(t)) ? v : 0;
  }
  gqs::DeviceGuard dg(device);
  do {
    st = gqs::cuda_status(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
    if (st != GQS_OK) break;
    // per-lane job records and rings come out of the budget first; the rest holds keys and
    // their scratch, half each
    size_t lane_bytes = 0;
    for (uint32_t i = 0; i < c.lanes && st == GQS_OK; ++i) {
      auto l = std::make_unique<Lane>();
      l->index = (int)i;
      l->srv = s;
      st = gqs::cuda_status(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking));
      if (st != GQS_OK) break;
      if (!c.per_request) {
        l->gs = std::make_unique<gqs::GraphSort>();
        st = l->gs->init(device, num_sms, c.batch_keys, c.batch_segments, true, c.timeout_ms);
        size_t cap = 0, ring = 0;
        for (int t = 0; t < 3; ++t)
          for (int v = 0; v < gqs::variant_count(t); ++v) {
            const gqs::VariantInfo vi = gqs::variant_info(t, v);
            cap = std::max(cap, gqs::job_capacity(vi, c.batch_keys, c.batch_segments));
            ring = std::max(ring, gqs::ticket_ring(vi, c.batch_keys, c.batch_segments));
          }
        lane_bytes += cap * sizeof(gqs::Job) + ring * 8;
      }
      s->lanes.push_back(std::move(l));
    }
    if (st != GQS_OK) break;
    if (c.per_request) {
      gqs_config pc;
      gqs_config_default(&pc);
      pc.sync = 0;
      pc.timeout_ms = c.timeout_ms;
      st = gqs_create(&s->plain, device, &pc);
      if (st != GQS_OK) break;
      for (int t = 0; t < 3; ++t) {
        st = gqs_set_variant(s->plain, t, s->variant[t]);
        if (st == GQS_OK) st = gqs_reserve(s->plain, t, c.batch_keys, 1, 0);
        if (st != GQS_OK) break;
      }
      if (st != GQS_OK) break;
      lane_bytes += 0;
    }
    if (c.budget_bytes <= lane_bytes + 2 * gqs::kArenaGrain) {
      st = GQS_ERR_INVALID;
      break;
    }
    s->arena_bytes = (c.budget_bytes - lane_bytes) / 2 / gqs::kArenaGrain * gqs::kArenaGrain;
    st = gqs::cuda_status(cudaMalloc(&s->keys, s->arena_bytes));
    if (st != GQS_OK) break;
    st = gqs::cuda_status(cudaMalloc(&s->scratch, s->arena_bytes));
    if (st != GQS_OK) break;
    s->arena.reset(s->arena_bytes);
    for (auto& l : s->lanes) {
      if (!l->gs) continue;
      l->gs->set_arena(s->keys, s->scratch, s->arena_bytes);
      for (int t = 0; t < 3 && st == GQS_OK; ++t)
        if (!l->gs->blocks_per_sm(t, s->variant[t])) st = GQS_ERR_NO_DEVICE;
    }
    if (st != GQS_OK) break;
    s->stats.arena_bytes = s->arena_bytes;
  } while (0);
  if (st != GQS_OK) {
    gqs_srv_destroy(s);
    return st;
  }
  try {
    s->dispatcher = std::thread(dispatcher_main, s);
  } catch (...) {
    gqs_srv_destroy(s);
    return GQS_ERR_NOMEM;
  }
  *out = s;
  return GQS_OK;
}

gqs_status gqs_srv_submit(gqs_server* s, int dtype, const void* in, void* out, size_t n, uint64_t* id) {
  if (!s || !id || dtype < 0 || dtype > 2) return GQS_ERR_INVALID;
  *id = 0;
  const size_t es = gqs::kElemSize[dtype];
  if (n == 0 || n > s->cfg.batch_keys || !in || !out) return GQS_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(in) % es) || (reinterpret_cast<uintptr_t>(out) % es)) return GQS_ERR_INVALID;
  if ((n * es + gqs::kArenaGrain - 1) / gqs::kArenaGrain * gqs::kArenaGrain > s->arena_bytes) return GQS_ERR_NOMEM;  // can never fit
  // Results go back asynchronously only into page-locked memory; pageable output is copied
  // back synchronously when the batch retires.
  bool out_pinned = false;
  {
    gqs::DeviceGuard dg(s->device);
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, out) == cudaSuccess)
      out_pinned = a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged;
    else
      (void)cudaGetLastError();
  }
  auto r = std::make_unique<Req>();
  r->dtype = dtype;
  r->in = in;
  r->out = out;
  r->n = n;
  r->staged_out = !out_pinned;
  r->info.dtype = (uint32_t)dtype;
  r->info.n = n;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return GQS_ERR_INVALID;
    if (s->fatal != GQS_OK) return s->fatal;
    r->id = s->next_id++;
    r->info.t_submit_ns = now_ns();
    *id = r->id;
    s->pending.push_back(r.get());
    s->reqs[r->id] = std::move(r);
    ++s->outstanding;
    ++s->stats.submitted;
    s->submitted = true;
  }
  s->cv_work.notify_one();
  return GQS_OK;
}

gqs_status gqs_srv_wait(gqs_server* s, uint64_t id, gqs_request_info* info) {
  if (!s) return GQS_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return GQS_ERR_INVALID;
  Req* r = it->second.get();
  s->cv_done.wait(lk, [r] { return r->done; });
  if (info) *info = r->info;
  const gqs_status st = (gqs_status)r->info.status;
  s->reqs.erase(it);
  return st;
}

gqs_status gqs_srv_wait_any(gqs_server* s, uint64_t* id, gqs_request_info* info, uint32_t timeout_ms) {
  if (!s || !id) return GQS_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  for (;;) {
    while (!s->completed.empty()) {
      const uint64_t k = s->completed.front();
      s->completed.pop_front();
      auto it = s->reqs.find(k);
      if (it == s->reqs.end()) continue;  // already collected by gqs_srv_wait
      *id = k;
      if (info) *info = it->second->info;
      const gqs_status st = (gqs_status)it->second->info.status;
      s->reqs.erase(it);
      return st;
    }
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && s->completed.empty())
      return GQS_ERR_TIMEOUT;
  }
}

gqs_status gqs_srv_cancel(gqs_server* s, uint64_t id) {
  if (!s) return GQS_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || it->second->done) return GQS_ERR_INVALID;
    Req* r = it->second.get();
    auto pit = std::find(s->pending.begin(), s->pending.end(), r);
    if (pit != s->pending.end()) {
      s->pending.erase(pit);
    } else {
      std::deque<Req*>& q = s->admitted[r->dtype];
      auto ait = std::find(q.begin(), q.end(), r);
      if (ait == q.end()) return GQS_ERR_INVALID;  // already on the GPU
      q.erase(ait);
      // its keys may still be on the way in; later copies into this space are ordered after
      // it on the same copy stream
      s->arena.release(r->off, r->n * gqs::kElemSize[r->dtype]);
      auto rd = s->rounds.find(r->round);
      if (rd != s->rounds.end() && --rd->second.refs == 0) {
        cudaEventDestroy(rd->second.ev);
        s->rounds.erase(rd);
      }
      s->stats.arena_used = s->arena.used();
    }
    complete_locked(s, r, GQS_ERR_CANCELLED);
    ++s->stats.cancelled;
  }
  s->cv_done.notify_all();
  s->cv_work.notify_one();
  return GQS_OK;
}

gqs_status gqs_srv_drain(gqs_server* s) {
  if (!s) return GQS_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [s] { return s->outstanding == 0; });
  return s->fatal;
}

gqs_status gqs_srv_stats(gqs_server* s, gqs_server_stats* out) {
  if (!s || !out) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->pending = s->pending.size();
  out->outstanding = s->outstanding;
  return s->fatal;
}

void gqs_srv_destroy(gqs_server* s) {
  if (!s) return;
  if (s->dispatcher.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_one();
    s->dispatcher.join();  // finishes every submitted request first
  }
  {
    gqs::DeviceGuard dg(s->device);
    for (auto& l : s->lanes) {
      if (l->stream) cudaStreamSynchronize(l->stream);
      l->gs.reset();
      if (l->stream) cudaStreamDestroy(l->stream);
    }
    s->lanes.clear();
    for (auto& kv : s->rounds) cudaEventDestroy(kv.second.ev);
    s->rounds.clear();
    if (s->plain) gqs_destroy(s->plain);
    if (s->copy_stream) {
      cudaStreamSynchronize(s->copy_stream);
      cudaStreamDestroy(s->copy_stream);
    }
    if (s->keys) cudaFree(s->keys);
    if (s->scratch) cudaFree(s->scratch);
  }
  delete s;
}

}  // extern "C"
