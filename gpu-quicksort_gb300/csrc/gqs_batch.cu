// Batched segmented sort as one replayable CUDA graph (gqs_batch_* in include/gqs.h), and the
// autotuner that picks its kernel variant.
//
// The reference sorts one array per call and drives every partition level from the host
// (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:835-906). A batch sorts thousands of independent
// arrays in one persistent launch: the seed kernel turns the segment table into root jobs and
// the persistent kernel drains all of them from one device queue. Everything one batch needs
// is captured once per (key type, variant) as a CUDA graph, so a batch costs one
// cudaGraphLaunch on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "gqs.h"
#include "gqs_graph.h"
#include "gqs_host.h"

namespace gqs {

GraphSort::~GraphSort() {
  if (ev_end_) cudaEventSynchronize(ev_end_);
  drop_graphs();
  if (jobs_) cudaFree(jobs_);
  if (ring_) cudaFree(ring_);
  if (q_) cudaFree(q_);
  if (hdr_dev_) cudaFree(hdr_dev_);
  if (q_host_) cudaFreeHost(q_host_);
  if (hdr_host_) cudaFreeHost(hdr_host_);
  if (ev_begin_) cudaEventDestroy(ev_begin_);
  if (ev_end_) cudaEventDestroy(ev_end_);
  if (cap_stream_) cudaStreamDestroy(cap_stream_);
}

void GraphSort::drop_graphs() {
  for (int t = 0; t < 3; ++t)
    for (int v = 0; v < kMaxVariantsPerType; ++v) {
      if (exec_[t][v]) cudaGraphExecDestroy(exec_[t][v]);
      if (graph_[t][v]) cudaGraphDestroy(graph_[t][v]);
      exec_[t][v] = nullptr;
      graph_[t][v] = nullptr;
    }
}

gqs_status GraphSort::init(int device, int num_sms, size_t max_keys, size_t max_segs, bool pairs,
                           uint32_t timeout_ms) {
  if (max_keys == 0 || max_segs == 0 || max_keys >= (1ull << 40) || max_segs >= (1ull << 30))
    return GQS_ERR_INVALID;
  device_ = device;
  num_sms_ = num_sms;
  max_keys_ = max_keys;
  max_segs_ = max_segs;
  pairs_ = pairs;
  timeout_ms_ = timeout_ms ? timeout_ms : 4000;
  table_words_ = 1 + (pairs ? 2 * max_segs : max_segs + 1);
  // Job records and ring entries for the most demanding variant of any key type.
  size_t cap = 0, ring = 0;
  for (int t = 0; t < 3; ++t)
    for (int v = 0; v < variant_count(t); ++v) {
      const VariantInfo vi = variant_info(t, v);
      cap = std::max(cap, job_capacity(vi, max_keys, max_segs));
      ring = std::max(ring, ticket_ring(vi, max_keys, max_segs));
    }
  if (cap >= (1ull << 32) || ring > (1ull << 31)) return GQS_ERR_INVALID;
  cudaError_t e;
  if ((e = cudaMalloc(&jobs_, cap * sizeof(Job))) != cudaSuccess) return cuda_status(e);
  job_cap_ = cap;
  if ((e = cudaMalloc(&ring_, ring * sizeof(unsigned long long))) != cudaSuccess) return cuda_status(e);
  ring_len_ = ring;
  if ((e = cudaMalloc(&q_, sizeof(Queue))) != cudaSuccess) return cuda_status(e);
  if ((e = cudaMalloc(&hdr_dev_, table_words_ * sizeof(unsigned long long))) != cudaSuccess) return cuda_status(e);
  if ((e = cudaMallocHost(&q_host_, sizeof(Queue))) != cudaSuccess) return cuda_status(e);
  if ((e = cudaMallocHost(&hdr_host_, table_words_ * sizeof(unsigned long long))) != cudaSuccess)
    return cuda_status(e);
  std::memset(hdr_host_, 0, table_words_ * sizeof(unsigned long long));
  std::memset(q_host_, 0, sizeof(Queue));
  if ((e = cudaStreamCreateWithFlags(&cap_stream_, cudaStreamNonBlocking)) != cudaSuccess) return cuda_status(e);
  if ((e = cudaEventCreate(&ev_begin_)) != cudaSuccess) return cuda_status(e);
  if ((e = cudaEventCreate(&ev_end_)) != cudaSuccess) return cuda_status(e);
  return GQS_OK;
}

void GraphSort::set_arena(void* keys, void* scratch, size_t arena_bytes) {
  if (keys == keys_ && scratch == scratch_ && arena_bytes == arena_bytes_) return;
  drop_graphs();
  keys_ = keys;
  scratch_ = scratch;
  arena_bytes_ = arena_bytes;
}

int GraphSort::blocks_per_sm(int dtype, int variant) {
  if (dtype < 0 || dtype > 2 || variant < 0 || variant >= variant_count(dtype)) return 0;
  if (!bps_[dtype][variant]) bps_[dtype][variant] = variant_prepare(dtype, variant);
  return bps_[dtype][variant];
}

gqs_status GraphSort::validate(int dtype, size_t nseg, unsigned long long* keys_out) const {
  if (nseg > max_segs_) return GQS_ERR_INVALID;
  const unsigned long long bound = arena_bytes_ / kElemSize[dtype];
  const unsigned long long* t = table();
  unsigned long long keys = 0;
  if (pairs_) {
    for (size_t i = 0; i < nseg; ++i) {
      if (t[2 * i] > t[2 * i + 1] || t[2 * i + 1] > bound) return GQS_ERR_INVALID;
      keys += t[2 * i + 1] - t[2 * i];
    }
  } else if (nseg) {
    for (size_t i = 0; i < nseg; ++i)
      if (t[i] > t[i + 1]) return GQS_ERR_INVALID;
    if (t[nseg] > bound) return GQS_ERR_INVALID;
    keys = t[nseg] - t[0];
  }
  if (keys > max_keys_) return GQS_ERR_INVALID;
  if (keys_out) *keys_out = keys;
  return GQS_OK;
}

gqs_status GraphSort::capture(int dtype, int variant) {
  if (exec_[dtype][variant]) return GQS_OK;
  const int bps = blocks_per_sm(dtype, variant);
  if (!bps) return GQS_ERR_NO_DEVICE;
  if (!keys_ || !scratch_) return GQS_ERR_INVALID;
  LaunchParams p{};
  p.d = keys_;
  p.dn = scratch_;
  p.jobs = jobs_;
  p.q = q_;
  p.tmap = ring_;
  p.capacity = (uint32_t)job_cap_;
  p.tmask = (uint32_t)(ring_len_ - 1);
  p.timeout_ns = (unsigned long long)timeout_ms_ * 1000000ull;
  p.offsets = hdr_dev_ + 1;
  p.nseg_dev = hdr_dev_;
  p.nseg = (uint32_t)max_segs_;
  p.pairs = pairs_ ? 1u : 0u;
  p.n = arena_bytes_ / kElemSize[dtype];
  p.variant = variant;
  p.grid = num_sms_ * bps;
  p.stream = cap_stream_;
  cudaError_t e = cudaStreamBeginCapture(cap_stream_, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_status(e);
  cudaError_t first = cudaSuccess;
  auto keep = [&first](cudaError_t r) {
    if (first == cudaSuccess && r != cudaSuccess) first = r;
  };
  keep(cudaMemcpyAsync(hdr_dev_, hdr_host_, table_words_ * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                       cap_stream_));
  keep(cudaMemsetAsync(q_, 0, sizeof(Queue), cap_stream_));
  keep(cudaMemsetAsync(ring_, 0, ring_len_ * sizeof(unsigned long long), cap_stream_));
  if (first == cudaSuccess) keep(launch_sort(dtype, p));
  keep(cudaMemcpyAsync(q_host_, q_, sizeof(Queue), cudaMemcpyDeviceToHost, cap_stream_));
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cap_stream_, &g);  // always ends the capture
  if (first == cudaSuccess) first = e;
  if (first != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_status(first);
  }
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_status(e);
  }
  graph_[dtype][variant] = g;
  exec_[dtype][variant] = x;
  return GQS_OK;
}

gqs_status GraphSort::launch(int dtype, int variant, size_t nseg, cudaStream_t stream) {
  if (dtype < 0 || dtype > 2 || variant < 0 || variant >= variant_count(dtype)) return GQS_ERR_INVALID;
  gqs_status st = validate(dtype, nseg, nullptr);
  if (st != GQS_OK) return st;
  st = capture(dtype, variant);
  if (st != GQS_OK) return st;
  hdr_host_[0] = nseg;
  cudaError_t e = cudaEventRecord(ev_begin_, stream);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec_[dtype][variant], stream);
  if (e == cudaSuccess) e = cudaEventRecord(ev_end_, stream);
  if (e != cudaSuccess) return cuda_status(e);
  last_dtype_ = dtype;
  last_variant_ = variant;
  return GQS_OK;
}

gqs_stats GraphSort::result() const {
  gqs_stats s = stats_from_queue(*q_host_, last_dtype_, last_variant_,
                                 num_sms_ * std::max(1, bps_[last_dtype_][last_variant_]));
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ev_begin_, ev_end_) == cudaSuccess) s.kernel_ms = ms;
  return s;
}

}  // namespace gqs

struct gqs_batch {
  int device = 0;
  int dtype = 0;
  int variant = 0;
  std::mutex mu;
  bool pending = false;
  void* keys = nullptr;
  void* scratch = nullptr;
  gqs_stats last{};
  std::unique_ptr<gqs::GraphSort> gs = std::make_unique<gqs::GraphSort>();
};

namespace {

gqs_status batch_wait_locked(gqs_batch* b) {
  if (!b->pending) return (gqs_status)b->last.status;
  cudaError_t e = cudaEventSynchronize(b->gs->end_event());
  b->pending = false;
  if (e != cudaSuccess) return gqs::cuda_status(e);
  b->last = b->gs->result();
  return (gqs_status)b->last.status;
}

}  // namespace

extern "C" {

gqs_status gqs_batch_create(int device, int dtype, size_t max_keys, size_t max_segments, const gqs_config* cfg,
                            gqs_batch** out) {
  if (!out) return GQS_ERR_INVALID;
  *out = nullptr;
  if (dtype < 0 || dtype > 2 || max_keys == 0 || max_segments == 0) return GQS_ERR_INVALID;
  int num_sms = 0;
  gqs_status st = gqs::check_device(device, &num_sms);
  if (st != GQS_OK) return st;
  gqs_config c;
  gqs_config_default(&c);
  if (cfg) c = *cfg;
  gqs_batch* b = new (std::nothrow) gqs_batch();
  if (!b) return GQS_ERR_NOMEM;
  b->device = device;
  b->dtype = dtype;
  b->variant = (c.variant >= 0 && c.variant < gqs::variant_count(dtype)) ? c.variant : 0;
  gqs::DeviceGuard dg(device);
  const size_t bytes = max_keys * gqs::kElemSize[dtype];
  st = b->gs->init(device, num_sms, max_keys, max_segments, false, c.timeout_ms);
  if (st == GQS_OK && cudaMalloc(&b->keys, bytes) != cudaSuccess) st = GQS_ERR_NOMEM;
  if (st == GQS_OK && cudaMalloc(&b->scratch, bytes) != cudaSuccess) st = GQS_ERR_NOMEM;
  if (st != GQS_OK) {
    (void)cudaGetLastError();
    gqs_batch_destroy(b);
    return st;
  }
  b->gs->set_arena(b->keys, b->scratch, bytes);
  b->last.status = GQS_OK;
  *out = b;
  return GQS_OK;
}

void gqs_batch_destroy(gqs_batch* b) {
  if (!b) return;
  {
    gqs::DeviceGuard dg(b->device);
    if (b->pending) cudaEventSynchronize(b->gs->end_event());
    b->gs.reset();  // frees its device buffers while the device is current
    if (b->keys) cudaFree(b->keys);
    if (b->scratch) cudaFree(b->scratch);
  }
  delete b;
}

void* gqs_batch_keys(gqs_batch* b) { return b ? b->keys : nullptr; }

uint64_t* gqs_batch_offsets(gqs_batch* b) { return b ? reinterpret_cast<uint64_t*>(b->gs->table()) : nullptr; }

gqs_status gqs_batch_launch(gqs_batch* b, size_t nseg, void* stream) {
  if (!b) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(b->mu);
  gqs::DeviceGuard dg(b->device);
  (void)batch_wait_locked(b);  // the table is reused: the previous replay must have read it
  gqs_status st = b->gs->launch(b->dtype, b->variant, nseg, static_cast<cudaStream_t>(stream));
  if (st != GQS_OK) return st;
  b->pending = true;
  return GQS_OK;
}

gqs_status gqs_batch_wait(gqs_batch* b, gqs_stats* out) {
  if (!b) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(b->mu);
  gqs::DeviceGuard dg(b->device);
  gqs_status st = batch_wait_locked(b);
  if (out) *out = b->last;
  return st;
}

static gqs_status batch_copy(gqs_batch* b, void* host, size_t first, size_t n, bool in) {
  if (!b || (!host && n)) return GQS_ERR_INVALID;
  if (first > b->gs->max_keys() || n > b->gs->max_keys() - first) return GQS_ERR_INVALID;
  if (!n) return GQS_OK;
  std::lock_guard<std::mutex> lk(b->mu);
  gqs::DeviceGuard dg(b->device);
  (void)batch_wait_locked(b);
  const size_t es = gqs::kElemSize[b->dtype];
  char* dev = static_cast<char*>(b->keys) + first * es;
  const cudaError_t e = in ? cudaMemcpy(dev, host, n * es, cudaMemcpyHostToDevice)
                           : cudaMemcpy(host, dev, n * es, cudaMemcpyDeviceToHost);
  return gqs::cuda_status(e);
}

gqs_status gqs_batch_copy_in(gqs_batch* b, const void* host, size_t first, size_t n) {
  return batch_copy(b, const_cast<void*>(host), first, n, true);
}

gqs_status gqs_batch_copy_out(gqs_batch* b, void* host, size_t first, size_t n) {
  return batch_copy(b, host, first, n, false);
}

gqs_status gqs_batch_set_variant(gqs_batch* b, int variant) {
  if (!b || variant < 0 || variant >= gqs::variant_count(b->dtype)) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(b->mu);
  gqs::DeviceGuard dg(b->device);
  if (!b->gs->blocks_per_sm(b->dtype, variant)) return GQS_ERR_NO_DEVICE;
  b->variant = variant;
  return GQS_OK;
}

int gqs_batch_get_variant(gqs_batch* b) { return b ? b->variant : -1; }

gqs_status gqs_batch_autotune(gqs_batch* b, size_t nseg, int reps, double* ms, int* best) {
  if (!b || reps < 1) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(b->mu);
  gqs::DeviceGuard dg(b->device);
  (void)batch_wait_locked(b);
  gqs_status st = b->gs->validate(b->dtype, nseg, nullptr);
  if (st != GQS_OK) return st;
  const uint64_t* t = reinterpret_cast<const uint64_t*>(b->gs->table());
  const size_t es = gqs::kElemSize[b->dtype];
  const size_t lo = nseg ? t[0] : 0, hi = nseg ? t[nseg] : 0;
  const size_t bytes = (hi - lo) * es;
  void* pristine = nullptr;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return GQS_ERR_CUDA;
  char* base = static_cast<char*>(b->keys) + lo * es;
  if (bytes && cudaMalloc(&pristine, bytes) != cudaSuccess) {
    (void)cudaGetLastError();
    cudaStreamDestroy(s);
    return GQS_ERR_NOMEM;
  }
  if (bytes) cudaMemcpyAsync(pristine, base, bytes, cudaMemcpyDeviceToDevice, s);
  const int nv = gqs::variant_count(b->dtype);
  int arg = -1;
  double best_ms = 0.0;
  gqs_status result = GQS_OK;
  for (int v = 0; v < nv; ++v) {
    double med = -1.0;
    if (b->gs->blocks_per_sm(b->dtype, v) > 0) {
      std::vector<double> times;
      for (int r = 0; r <= reps; ++r) {  // the first replay warms up (and captures the graph)
        if (bytes) cudaMemcpyAsync(base, pristine, bytes, cudaMemcpyDeviceToDevice, s);
        st = b->gs->launch(b->dtype, v, nseg, s);
        if (st == GQS_OK) {
          cudaError_t e = cudaStreamSynchronize(s);
          st = e == cudaSuccess ? (gqs_status)b->gs->result().status : gqs::cuda_status(e);
        }
        if (st != GQS_OK) break;
        if (r > 0) times.push_back(b->gs->result().kernel_ms);
      }
      if (st == GQS_OK && !times.empty()) {
        std::sort(times.begin(), times.end());
        med = times[times.size() / 2];
      } else if (st == GQS_ERR_CUDA || st == GQS_ERR_NOMEM) {
        result = st;  // the context may be unusable: stop tuning
      }
    }
    if (ms) ms[v] = med;
    if (med >= 0.0 && (arg < 0 || med < best_ms)) {
      arg = v;
      best_ms = med;
    }
    if (result != GQS_OK) break;
  }
  // leave the batch sorted by the chosen variant
  if (result == GQS_OK && arg >= 0) {
    if (bytes) cudaMemcpyAsync(base, pristine, bytes, cudaMemcpyDeviceToDevice, s);
    st = b->gs->launch(b->dtype, arg, nseg, s);
    if (st == GQS_OK) {
      cudaError_t e = cudaStreamSynchronize(s);
      st = e == cudaSuccess ? (gqs_status)b->gs->result().status : gqs::cuda_status(e);
    }
    b->last = b->gs->result();
    if (st != GQS_OK) result = st;
  }
  if (pristine) cudaFree(pristine);
  cudaStreamDestroy(s);
  if (arg < 0 && result == GQS_OK) result = GQS_ERR_NO_DEVICE;
  if (arg >= 0) b->variant = arg;
  if (best) *best = arg;
  return result;
}

}  // extern "C"
