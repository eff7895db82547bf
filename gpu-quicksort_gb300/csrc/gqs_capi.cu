// The C ABI (include/gqs.h): contexts, pools, argument checks, launches, status and stats.
//
// Host-side replacement for the reference's GPUQSort<T> driver
// (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:835-906). The reference rebuilds its records on the
// host and reads results back after every partition level (QuicksortMain.cpp:858-899); here one
// seed launch and one persistent launch sort the whole array, and the host only reads a small
// status block at the end.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>

#include "gqs.h"
#include "gqs_device.cuh"
#include "gqs_host.h"
#include "gqs_launch.h"
#include "gqs_tuning.h"

namespace gqs {

int variant_count(int dtype) {
  switch (dtype) {
    case DT_U32: return variant_count_u32();
    case DT_F32: return variant_count_f32();
    case DT_F64: return variant_count_f64();
    case DT_U64: return variant_count_u64();
    default: return 0;
  }
}
VariantInfo variant_info(int dtype, int v) {
  switch (dtype) {
    case DT_U32: return variant_info_u32(v);
    case DT_F32: return variant_info_f32(v);
    case DT_U64: return variant_info_u64(v);
    default: return variant_info_f64(v);
  }
}
int variant_prepare(int dtype, int v) {
  switch (dtype) {
    case DT_U32: return variant_prepare_u32(v);
    case DT_F32: return variant_prepare_f32(v);
    case DT_U64: return variant_prepare_u64(v);
    default: return variant_prepare_f64(v);
  }
}
cudaError_t launch_sort(int dtype, const LaunchParams& p) {
  switch (dtype) {
    case DT_U32: return launch_u32(p);
    case DT_F32: return launch_f32(p);
    case DT_U64: return launch_u64(p);
    default: return launch_f64(p);
  }
}

// The tuning table's variant for n keys of `dtype` on a GPU of `sms` SMs: the rows of the
// nearest SM count measured, then the nearest size class (ceil(log2 n)); 0 without a row.
int tuned_variant(int dtype, size_t n, int sms) {
  int lg = 0;
  while (lg < 63 && (1ull << lg) < (unsigned long long)n) ++lg;
  int best_sms = -1, v = 0, best = 1 << 30;
  for (const TuneRow& r : kTuneRows) {
    if (r.dtype != dtype) continue;
    const int d = r.sms > sms ? r.sms - sms : sms - r.sms;
    if (best_sms < 0 || d < (best_sms > sms ? best_sms - sms : sms - best_sms)) best_sms = r.sms;
  }
  for (const TuneRow& r : kTuneRows) {
    if (r.dtype != dtype || r.sms != best_sms) continue;
    const int d = r.log2n > lg ? r.log2n - lg : lg - r.log2n;
    if (d < best) {
      best = d;
      v = r.variant;
    }
  }
  return v >= 0 && v < variant_count(dtype) ? v : 0;
}

}  // namespace gqs

namespace {

constexpr int kMaxVariants = 16;
// Host-pointer sorts of at least kPipeMin keys are pipelined: the array is copied in kPieces
// pieces, each sorted as soon as it has arrived, then the sorted pieces are merged.
constexpr size_t kPipeMin = 1ull << 24;
constexpr int kPieces = 4;
// The last merge of a pipelined sort runs in kSlices launches; each slice of the result is copied
// back while the next one is merged.
constexpr int kSlices = 8;
using gqs::cuda_status;
using gqs::DeviceGuard;
using gqs::job_capacity;
using gqs::kElemSize;
using gqs::ticket_ring;

}  // namespace

struct gqs_ctx {
  int device = 0;
  int num_sms = 0;
  gqs_config cfg{};
  std::mutex mu;
  cudaStream_t stream = nullptr;       // used by the host-pointer calls
  cudaStream_t copy_stream = nullptr;  // host -> device pieces of a pipelined host sort
  cudaEvent_t ev_piece[4] = {};
  cudaEvent_t ev_slice[8] = {};        // slices of a pipelined sort's last merge, done
  gqs::Queue* q_acc = nullptr;         // statistics of a pipelined sort, summed over its pieces
  void* merge_splits = nullptr;        // merge-path splits of the pipelined sort's merges
  size_t merge_splits_bytes = 0;
  bool pending_acc = false;
  void* pool_d = nullptr;
  size_t pool_d_bytes = 0;
  void* pool_dn = nullptr;
  size_t pool_dn_bytes = 0;
  void* pool_kv = nullptr;  // packed (key, value) words of the pair sort
  size_t pool_kv_bytes = 0;
  void* pool_v = nullptr;   // values staged for the host-pointer pair sort
  size_t pool_v_bytes = 0;
  gqs::Job* jobs = nullptr;
  size_t job_cap = 0;
  gqs::Queue* q = nullptr;
  gqs::Queue* q_host = nullptr;  // pinned
  unsigned long long* offs = nullptr;
  size_t offs_cap = 0;
  unsigned long long* tmap = nullptr;  // ticket ring
  size_t tmap_len = 0;                 // entries (a power of two)
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr, ev_done = nullptr;
  bool pending = false;
  bool pending_timed = false;
  int pending_dtype = 0;
  int pending_variant = 0;
  int pending_grid = 0;
  unsigned long long pending_keys = 0;
  gqs_stats last{};
  uint64_t last_prof[32] = {};
  uint64_t last_phase[4] = {};  // the last sort's Queue::phase
#ifdef GQS_PROFILE
  unsigned long long last_lvl[gqs::kLevels][6] = {};  // per-level rows of the last sort
  unsigned long long last_lvl_start = 0;
#endif
  void* split_buf = nullptr;  // scratch of the top split of small sorts (gqs_split.cu)
  size_t split_bytes = 0;
  bool top_split = true;
  int variant[4] = {0, 0, 0, 0};  // per key type, and the internal packed pairs
  bool auto_variant[4] = {true, true, true, true};  // pick per call from the tuning table
  int blocks_per_sm[4][kMaxVariants] = {};
};

namespace {

// Grows a device buffer to at least `bytes`; callers have waited for pending work.
gqs_status grow(void** p, size_t* cap, size_t bytes) {
  if (*cap >= bytes && *p) return GQS_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  size_t want = std::max(bytes, (size_t)256);
  cudaError_t e = cudaMalloc(p, want);
  if (e != cudaSuccess) {
    *p = nullptr;
    (void)cudaGetLastError();
    return GQS_ERR_NOMEM;
  }
  *cap = want;
  return GQS_OK;
}

gqs_status wait_pending_locked(gqs_ctx* c) {
  if (!c->pending) return GQS_OK;
  cudaError_t e = cudaEventSynchronize(c->ev_done);
  if (e != cudaSuccess) return cuda_status(e);
  e = cudaMemcpy(c->q_host, c->pending_acc ? c->q_acc : c->q, sizeof(gqs::Queue), cudaMemcpyDeviceToHost);
  c->pending = false;
  c->pending_acc = false;
  if (e != cudaSuccess) return cuda_status(e);
  gqs_stats s = gqs::stats_from_queue(*c->q_host, c->pending_dtype, c->pending_variant, c->pending_grid);
  if (c->pending_timed) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev_begin, c->ev_end) == cudaSuccess) s.kernel_ms = ms;
  }
  c->last = s;
  for (int i = 0; i < 32; ++i) c->last_prof[i] = c->q_host->prof[i];
  for (int i = 0; i < 4; ++i) c->last_phase[i] = c->q_host->phase[i];
#ifdef GQS_PROFILE
  std::memcpy(c->last_lvl, c->q_host->lvl, sizeof(c->last_lvl));
  c->last_lvl_start = c->q_host->lvl_start;
#endif
  return (gqs_status)s.status;
}

// Returns `st` after a failure once copies of a caller's host array are queued, when neither
// stream can still read or write that array.
gqs_status drain(gqs_ctx* c, gqs_status st) {
  cudaStreamSynchronize(c->copy_stream);
  cudaStreamSynchronize(c->stream);
  (void)cudaGetLastError();
  // A sort enqueued before the failure has run (or still runs on a caller's stream): collect it
  // now, so that the next call neither reports its status as its own nor skips waiting for it.
  (void)wait_pending_locked(c);
  (void)cudaGetLastError();
  return st;
}

// Validates, grows pools, and enqueues one sort on `stream`. Caller holds the lock.
gqs_status enqueue_locked(gqs_ctx* c, int dtype, void* d, void* dn, size_t n, const unsigned long long* offsets,
                          size_t nseg, cudaStream_t stream, unsigned long long check_n = 0) {
  const size_t es = kElemSize[dtype];
  if (!d || (reinterpret_cast<uintptr_t>(d) % es) != 0) return GQS_ERR_INVALID;
  if (dn && (reinterpret_cast<uintptr_t>(dn) % es) != 0) return GQS_ERR_INVALID;
  if (n >= (1ull << 40) || nseg >= (1ull << 31)) return GQS_ERR_INVALID;
  const int v = c->auto_variant[dtype] ? gqs::tuned_variant(dtype, n, c->num_sms) : c->variant[dtype];
  const gqs::VariantInfo vi = gqs::variant_info(dtype, v);
  // Small plain sorts start with a multi-way split whose buckets become the segments.
  gqs::SplitPlan plan{};
  const bool split = !offsets && !check_n && c->top_split && gqs::split_plan(dtype, n, vi.tile, c->num_sms, &plan);
  const size_t segs = split ? plan.k : nseg;
  const size_t cap = job_capacity(vi, n, segs);
  const size_t ring = ticket_ring(vi, n, segs);
  if (cap >= (1ull << 32) || ring > (1ull << 31)) return GQS_ERR_INVALID;
  if (!c->blocks_per_sm[dtype][v]) {
    c->blocks_per_sm[dtype][v] = gqs::variant_prepare(dtype, v);
    if (!c->blocks_per_sm[dtype][v]) return GQS_ERR_NO_DEVICE;
  }
  gqs_status st = GQS_OK;
  const bool need_jobs = c->job_cap < cap;
  const bool need_dn = !dn && c->pool_dn_bytes < n * es;
  const bool need_ring = c->tmap_len < ring;
  const bool need_split = split && c->split_bytes < gqs::split_scratch_bytes(plan);
  if (need_jobs || need_dn || need_ring || need_split) {
    st = wait_pending_locked(c);
    if (st != GQS_OK && st != GQS_ERR_TIMEOUT && st != GQS_ERR_CAPACITY && st != GQS_ERR_INTERNAL) return st;
    size_t bytes = 0;
    if (need_jobs) {
      void* p = c->jobs;
      bytes = c->job_cap * sizeof(gqs::Job);
      st = grow(&p, &bytes, cap * sizeof(gqs::Job));
      c->jobs = static_cast<gqs::Job*>(p);
      c->job_cap = c->jobs ? bytes / sizeof(gqs::Job) : 0;
      if (st != GQS_OK) return st;
    }
    if (need_ring) {
      void* p = c->tmap;
      size_t bytes = c->tmap_len * sizeof(unsigned long long);
      st = grow(&p, &bytes, ring * sizeof(unsigned long long));
      c->tmap = static_cast<unsigned long long*>(p);
      c->tmap_len = c->tmap ? ring : 0;
      if (st != GQS_OK) return st;
    }
    if (need_dn) {
      st = grow(&c->pool_dn, &c->pool_dn_bytes, n * es);
      if (st != GQS_OK) return st;
    }
    if (need_split) {
      st = grow(&c->split_buf, &c->split_bytes, gqs::split_scratch_bytes(plan));
      if (st != GQS_OK) return st;
    }
  }
  if (!dn) dn = c->pool_dn;
  if (c->pending) {
    cudaError_t e = cudaStreamWaitEvent(stream, c->ev_done, 0);
    if (e != cudaSuccess) return cuda_status(e);
  }
  cudaError_t e = cudaMemsetAsync(c->q, 0, sizeof(gqs::Queue), stream);
  if (e != cudaSuccess) return cuda_status(e);
  // Only the part of the ring this sort can reach needs clearing.
  e = cudaMemsetAsync(c->tmap, 0, ring * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return cuda_status(e);
  gqs::LaunchParams p{};
  p.d = d;
  p.dn = dn;
  p.jobs = c->jobs;
  p.q = c->q;
  p.tmap = c->tmap;
  p.capacity = (uint32_t)c->job_cap;
  p.tmask = (uint32_t)(ring - 1);
  p.timeout_ns = (unsigned long long)(c->cfg.timeout_ms ? c->cfg.timeout_ms : 4000) * 1000000ull;
  p.offsets = offsets;
  p.n = n;
  p.nseg = (uint32_t)(offsets ? nseg : 1);
  p.variant = v;
  p.grid = c->num_sms * c->blocks_per_sm[dtype][v];
  p.stream = stream;
  p.ev_begin = c->cfg.timing ? c->ev_begin : nullptr;
  p.ev_end = c->cfg.timing ? c->ev_end : nullptr;
  p.check_n = check_n;
  if (split) {  // the timed interval starts with the split
    if (p.ev_begin && (e = cudaEventRecord(p.ev_begin, stream)) != cudaSuccess) return cuda_status(e);
    p.ev_begin = nullptr;
    unsigned long long* table = nullptr;
    e = gqs::split_launch(dtype, plan, d, dn, n, c->split_buf, &table, c->q, stream);
    if (e != cudaSuccess) return cuda_status(e);
    p.offsets = table;
    p.nseg = plan.k;
    p.from_dn = 1;
  }
  e = gqs::launch_sort(dtype, p);
  if (e != cudaSuccess) return cuda_status(e);
  e = cudaEventRecord(c->ev_done, stream);
  if (e != cudaSuccess) return cuda_status(e);
  c->pending = true;
  c->pending_timed = c->cfg.timing != 0;
  c->pending_dtype = dtype;
  c->pending_variant = v;
  c->pending_grid = p.grid;
  c->pending_keys = offsets ? 0 : n;
  return GQS_OK;
}

gqs_status sort_dev(gqs_ctx* c, int dtype, void* d, void* scratch, size_t n, void* stream) {
  if (!c) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  if (n <= 1) return d || n == 0 ? GQS_OK : GQS_ERR_INVALID;
  gqs_status st = enqueue_locked(c, dtype, d, scratch, n, nullptr, 1, static_cast<cudaStream_t>(stream));
  if (st != GQS_OK) return st;
  if (c->cfg.sync) return wait_pending_locked(c);
  return GQS_OK;
}

// Folds one piece's status block into the pipelined sort's totals (one thread).
__global__ void accumulate_queue(const gqs::Queue* __restrict__ q, gqs::Queue* __restrict__ acc) {
  acc->total += q->total;
  acc->done += q->done;
  acc->part_keys += q->part_keys;
  acc->local_keys += q->local_keys;
  acc->tiny_keys += q->tiny_keys;
  acc->fill_keys += q->fill_keys;
  acc->chunks += q->chunks;
  acc->part_jobs += q->part_jobs;
  acc->local_jobs += q->local_jobs;
  acc->fill_jobs += q->fill_jobs;
  if (q->max_depth > acc->max_depth) acc->max_depth = q->max_depth;
  for (int i = 0; i < 4; ++i) acc->phase[i] += q->phase[i];
  if (q->error && !acc->error) {
    acc->error = q->error;
    acc->error_info = q->error_info;
  }
#ifdef GQS_PROFILE
  if (!acc->lvl_start || (q->lvl_start && q->lvl_start < acc->lvl_start)) acc->lvl_start = q->lvl_start;
  for (int d = 0; d < gqs::kLevels; ++d) {
    for (int c = 0; c < 4; ++c) acc->lvl[d][c] += q->lvl[d][c];
    if (!acc->lvl[d][4] || (q->lvl[d][4] && q->lvl[d][4] < acc->lvl[d][4])) acc->lvl[d][4] = q->lvl[d][4];
    if (q->lvl[d][5] > acc->lvl[d][5]) acc->lvl[d][5] = q->lvl[d][5];
  }
#endif
}

// The host-pointer sort of a large array, overlapping the copies with the work: piece i is
// copied in on the copy stream while piece i - 1 is sorted; the sorted pieces are merged
// pairwise (two merge passes for four pieces), and the last merge runs in slices whose results
// are copied back while the next slice is merged. Lock held.
gqs_status sort_host_pipelined(gqs_ctx* c, int dtype, void* d, size_t n) {
  const size_t es = kElemSize[dtype];
  const size_t bytes = n * es;
  const size_t split_bytes = gqs::merge_split_words(n) * sizeof(unsigned long long);
  if (c->pool_d_bytes < bytes || c->pool_dn_bytes < bytes || c->merge_splits_bytes < split_bytes) {
    (void)wait_pending_locked(c);
    gqs_status st = grow(&c->pool_d, &c->pool_d_bytes, bytes);
    if (st == GQS_OK) st = grow(&c->pool_dn, &c->pool_dn_bytes, bytes);
    if (st == GQS_OK) st = grow(&c->merge_splits, &c->merge_splits_bytes, split_bytes);
    if (st != GQS_OK) return st;
  }
  unsigned long long* sp = static_cast<unsigned long long*>(c->merge_splits);
  size_t off[kPieces + 1];
  for (int i = 0; i <= kPieces; ++i) off[i] = n / kPieces * i;
  off[kPieces] = n;
  char* dd = static_cast<char*>(c->pool_d);
  char* dn = static_cast<char*>(c->pool_dn);
  char* hd = static_cast<char*>(d);
  cudaError_t e = cudaSuccess;
  if (c->pending) e = cudaStreamWaitEvent(c->copy_stream, c->ev_done, 0);  // pool_d is free again
  if (e == cudaSuccess) e = cudaMemsetAsync(c->q_acc, 0, sizeof(gqs::Queue), c->stream);
  if (e != cudaSuccess) return cuda_status(e);
  for (int i = 0; i < kPieces; ++i) {
    const size_t len = off[i + 1] - off[i];
    e = cudaMemcpyAsync(dd + off[i] * es, hd + off[i] * es, len * es, cudaMemcpyHostToDevice, c->copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_piece[i], c->copy_stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_piece[i], 0);
    if (e != cudaSuccess) return drain(c, cuda_status(e));
    gqs_status st = enqueue_locked(c, dtype, dd + off[i] * es, dn + off[i] * es, len, nullptr, 1, c->stream);
    if (st != GQS_OK) return drain(c, st);
    accumulate_queue<<<1, 1, 0, c->stream>>>(c->q, c->q_acc);
    if ((e = cudaGetLastError()) != cudaSuccess) return drain(c, cuda_status(e));
  }
  // pieces 0+1 and 2+3 into the scratch, then the two halves back into pool_d, in kSlices
  // launches: each slice of the result goes back to the host on the copy stream while the
  // next one is merged
  static_assert(kSlices <= (int)(sizeof(c->ev_slice) / sizeof(c->ev_slice[0])), "one event per slice");
  e = gqs::merge_runs(dtype, dd, off[1], dd + off[1] * es, off[2] - off[1], dn, sp, c->stream);
  if (e == cudaSuccess)
    e = gqs::merge_runs(dtype, dd + off[2] * es, off[3] - off[2], dd + off[3] * es, off[4] - off[3], dn + off[2] * es,
                        sp, c->stream);
  const size_t nlo = off[2], nhi = n - off[2];
  if (e == cudaSuccess) e = gqs::merge_plan(dtype, dn, nlo, dn + nlo * es, nhi, sp, c->stream);
  const size_t tk = gqs::merge_tile_keys(), tiles = (n + tk - 1) / tk;
  for (int sl = 0; sl < kSlices && e == cudaSuccess; ++sl) {
    const size_t t0 = tiles * (size_t)sl / kSlices, t1 = tiles * (size_t)(sl + 1) / kSlices;
    const size_t k0 = std::min(t0 * tk, n), k1 = std::min(t1 * tk, n);
    e = gqs::merge_tiles(dtype, dn, nlo, dn + nlo * es, nhi, dd, sp, t0, t1, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_slice[sl], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_stream, c->ev_slice[sl], 0);
    if (e == cudaSuccess && k1 > k0)
      e = cudaMemcpyAsync(hd + k0 * es, dd + k0 * es, (k1 - k0) * es, cudaMemcpyDeviceToHost, c->copy_stream);
  }
  // the last copy follows every kernel of this call (it waited for the last slice)
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_done, c->copy_stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  c->pending_acc = true;
  c->pending_timed = false;
  return wait_pending_locked(c);
}

gqs_status sort_host(gqs_ctx* c, int dtype, void* d, size_t n) {
  if (!c) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  if (n <= 1) return d || n == 0 ? GQS_OK : GQS_ERR_INVALID;
  if (!d) return GQS_ERR_INVALID;
  if (n >= kPipeMin && n < (1ull << 40)) return sort_host_pipelined(c, dtype, d, n);
  const size_t bytes = n * kElemSize[dtype];
  if (c->pool_d_bytes < bytes) {
    gqs_status st = wait_pending_locked(c);
    (void)st;
    st = grow(&c->pool_d, &c->pool_d_bytes, bytes);
    if (st != GQS_OK) return st;
  }
  cudaError_t e = cudaMemcpyAsync(c->pool_d, d, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  gqs_status st = enqueue_locked(c, dtype, c->pool_d, nullptr, n, nullptr, 1, c->stream);
  if (st != GQS_OK) return drain(c, st);
  e = cudaMemcpyAsync(d, c->pool_d, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  e = cudaEventRecord(c->ev_done, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  return wait_pending_locked(c);
}

gqs_status sort_segments_dev(gqs_ctx* c, int dtype, void* keys, void* scratch, size_t n, const uint64_t* offsets,
                             size_t nseg, void* stream) {
  if (!c) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  if (nseg == 0) return GQS_OK;
  if (!offsets || !keys) return GQS_ERR_INVALID;
  gqs_status st = enqueue_locked(c, dtype, keys, scratch, n, reinterpret_cast<const unsigned long long*>(offsets),
                                 nseg, static_cast<cudaStream_t>(stream));
  if (st != GQS_OK) return st;
  if (c->cfg.sync) return wait_pending_locked(c);
  return GQS_OK;
}

gqs_status sort_segments_host(gqs_ctx* c, int dtype, void* keys, size_t n, const uint64_t* offsets, size_t nseg) {
  if (!c) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  if (nseg == 0) return GQS_OK;
  if (!offsets || (!keys && n)) return GQS_ERR_INVALID;
  for (size_t i = 0; i < nseg; ++i)
    if (offsets[i + 1] < offsets[i]) return GQS_ERR_INVALID;
  if (offsets[nseg] > n || offsets[0] > offsets[nseg]) return GQS_ERR_INVALID;
  if (n == 0) return GQS_OK;
  const size_t bytes = n * kElemSize[dtype];
  const size_t obytes = (nseg + 1) * sizeof(uint64_t);
  if (c->pool_d_bytes < bytes || c->offs_cap < obytes) {
    (void)wait_pending_locked(c);
    gqs_status st = grow(&c->pool_d, &c->pool_d_bytes, bytes);
    if (st != GQS_OK) return st;
    void* po = c->offs;
    st = grow(&po, &c->offs_cap, obytes);
    c->offs = static_cast<unsigned long long*>(po);
    if (st != GQS_OK) return st;
  }
  cudaError_t e = cudaMemcpyAsync(c->pool_d, keys, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  e = cudaMemcpyAsync(c->offs, offsets, obytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  gqs_status st = enqueue_locked(c, dtype, c->pool_d, nullptr, n, c->offs, nseg, c->stream);
  if (st != GQS_OK) return drain(c, st);
  e = cudaMemcpyAsync(keys, c->pool_d, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  e = cudaEventRecord(c->ev_done, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  return wait_pending_locked(c);
}

// ---- pair sort: (key, value) packed into one 64-bit word --------------------------------
// word = (order-preserving key map << 32) | value, so sorting the words orders the pairs by key
// and pairs with equal keys by value (values 0..n-1: a stable argsort).
template <bool kFloat>
__global__ void __launch_bounds__(256) pack_pairs(const uint32_t* __restrict__ keys,
                                                  const uint32_t* __restrict__ vals,
                                                  unsigned long long* __restrict__ out, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t k = keys[i];
    if (kFloat) k ^= (uint32_t)((int32_t)k >> 31) | 0x80000000u;
    out[i] = ((unsigned long long)k << 32) | vals[i];
  }
}

template <bool kFloat>
__global__ void __launch_bounds__(256) unpack_pairs(const unsigned long long* __restrict__ in,
                                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                    size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const unsigned long long w = in[i];
    uint32_t k = (uint32_t)(w >> 32);
    if (kFloat) k ^= ~(uint32_t)((int32_t)k >> 31) | 0x80000000u;
    keys[i] = k;
    vals[i] = (uint32_t)w;
  }
}

// Enqueues pack -> sort of the words -> unpack on `stream` for device keys/values. Lock held.
gqs_status enqueue_pairs_locked(gqs_ctx* c, bool is_float, uint32_t* keys, uint32_t* vals, size_t n,
                                cudaStream_t stream) {
  if ((reinterpret_cast<uintptr_t>(keys) & 3u) || (reinterpret_cast<uintptr_t>(vals) & 3u)) return GQS_ERR_INVALID;
  if (n >= (1ull << 40)) return GQS_ERR_INVALID;
  if (c->pool_kv_bytes < n * 8) {
    (void)wait_pending_locked(c);
    gqs_status st = grow(&c->pool_kv, &c->pool_kv_bytes, n * 8);
    if (st != GQS_OK) return st;
  }
  const int blocks = c->num_sms * 8;
  unsigned long long* w = static_cast<unsigned long long*>(c->pool_kv);
  if (c->pending) {
    cudaError_t e = cudaStreamWaitEvent(stream, c->ev_done, 0);  // the previous sort may still use pool_kv
    if (e != cudaSuccess) return cuda_status(e);
  }
  if (is_float) pack_pairs<true><<<blocks, 256, 0, stream>>>(keys, vals, w, n);
  else pack_pairs<false><<<blocks, 256, 0, stream>>>(keys, vals, w, n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  gqs_status st = enqueue_locked(c, gqs::DT_U64, w, nullptr, n, nullptr, 1, stream);
  if (st != GQS_OK) return st;
  if (is_float) unpack_pairs<true><<<blocks, 256, 0, stream>>>(w, keys, vals, n);
  else unpack_pairs<false><<<blocks, 256, 0, stream>>>(w, keys, vals, n);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_done, stream);  // the call is done after the unpack
  return cuda_status(e);
}

gqs_status sort_pairs_dev(gqs_ctx* c, bool is_float, uint32_t* keys, uint32_t* vals, size_t n, void* stream) {
  if (!c) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  if (n <= 1) return (keys && vals) || n == 0 ? GQS_OK : GQS_ERR_INVALID;
  if (!keys || !vals) return GQS_ERR_INVALID;
  gqs_status st = enqueue_pairs_locked(c, is_float, keys, vals, n, static_cast<cudaStream_t>(stream));
  if (st != GQS_OK) return st;
  if (c->cfg.sync) return wait_pending_locked(c);
  return GQS_OK;
}

gqs_status sort_pairs_host(gqs_ctx* c, bool is_float, uint32_t* keys, uint32_t* vals, size_t n) {
  if (!c) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  if (n <= 1) return (keys && vals) || n == 0 ? GQS_OK : GQS_ERR_INVALID;
  if (!keys || !vals) return GQS_ERR_INVALID;
  const size_t bytes = n * 4;
  if (c->pool_d_bytes < bytes || c->pool_v_bytes < bytes) {
    (void)wait_pending_locked(c);
    gqs_status st = grow(&c->pool_d, &c->pool_d_bytes, bytes);
    if (st == GQS_OK) st = grow(&c->pool_v, &c->pool_v_bytes, bytes);
    if (st != GQS_OK) return st;
  }
  uint32_t* dk = static_cast<uint32_t*>(c->pool_d);
  uint32_t* dv = static_cast<uint32_t*>(c->pool_v);
  cudaError_t e = cudaMemcpyAsync(dk, keys, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dv, vals, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  gqs_status st = enqueue_pairs_locked(c, is_float, dk, dv, n, c->stream);
  if (st != GQS_OK) return drain(c, st);
  e = cudaMemcpyAsync(keys, dk, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(vals, dv, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_done, c->stream);
  if (e != cudaSuccess) return drain(c, cuda_status(e));
  return wait_pending_locked(c);
}

}  // namespace

extern "C" {

gqs_status gqs_sort_pairs_u32(gqs_ctx* c, uint32_t* keys, uint32_t* values, size_t n) {
  return sort_pairs_host(c, false, keys, values, n);
}
gqs_status gqs_sort_pairs_f32(gqs_ctx* c, float* keys, uint32_t* values, size_t n) {
  return sort_pairs_host(c, true, reinterpret_cast<uint32_t*>(keys), values, n);
}
gqs_status gqs_sort_pairs_u32_dev(gqs_ctx* c, uint32_t* keys, uint32_t* values, size_t n, void* stream) {
  return sort_pairs_dev(c, false, keys, values, n, stream);
}
gqs_status gqs_sort_pairs_f32_dev(gqs_ctx* c, float* keys, uint32_t* values, size_t n, void* stream) {
  return sort_pairs_dev(c, true, reinterpret_cast<uint32_t*>(keys), values, n, stream);
}

void gqs_config_default(gqs_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->variant = -1;
  cfg->timeout_ms = 4000;
  cfg->sync = 1;
  cfg->timing = 0;
}

gqs_status gqs_create(gqs_ctx** out, int device, const gqs_config* cfg) {
  if (!out) return GQS_ERR_INVALID;
  *out = nullptr;
  int num_sms = 0;
  const gqs_status dst = gqs::check_device(device, &num_sms);
  if (dst != GQS_OK) return dst;
  gqs_ctx* c = new (std::nothrow) gqs_ctx();
  if (!c) return GQS_ERR_NOMEM;
  c->device = device;
  c->num_sms = num_sms;
  gqs_config_default(&c->cfg);
  if (cfg) c->cfg = *cfg;
  DeviceGuard dg(device);
  gqs_status st = GQS_OK;
  do {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
      st = GQS_ERR_CUDA;
      break;
    }
    bool evs = true;
    for (cudaEvent_t& ev : c->ev_piece) evs = evs && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
    for (cudaEvent_t& ev : c->ev_slice) evs = evs && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
    if (!evs) { st = GQS_ERR_CUDA; break; }
    if (cudaMalloc(&c->q_acc, sizeof(gqs::Queue)) != cudaSuccess) { st = GQS_ERR_NOMEM; break; }
    if (cudaEventCreate(&c->ev_begin) != cudaSuccess || cudaEventCreate(&c->ev_end) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming) != cudaSuccess) {
      st = GQS_ERR_CUDA;
      break;
    }
    if (cudaMalloc(&c->q, sizeof(gqs::Queue)) != cudaSuccess) { st = GQS_ERR_NOMEM; break; }
    if (cudaMallocHost(&c->q_host, sizeof(gqs::Queue)) != cudaSuccess) { st = GQS_ERR_NOMEM; break; }
    for (int t = 0; t < 4; ++t) {
      int v = c->cfg.variant;
      c->auto_variant[t] = v < 0;
      if (v < 0 || v >= gqs::variant_count(t)) v = 0;
      c->variant[t] = v;
    }
  } while (0);
  if (st != GQS_OK) {
    (void)cudaGetLastError();
    gqs_destroy(c);
    return st;
  }
  *out = c;
  return GQS_OK;
}

void gqs_destroy(gqs_ctx* c) {
  if (!c) return;
  {
    DeviceGuard dg(c->device);
    if (c->pending && c->ev_done) cudaEventSynchronize(c->ev_done);
    if (c->pool_d) cudaFree(c->pool_d);
    if (c->pool_dn) cudaFree(c->pool_dn);
    if (c->pool_kv) cudaFree(c->pool_kv);
    if (c->pool_v) cudaFree(c->pool_v);
    if (c->jobs) cudaFree(c->jobs);
    if (c->q) cudaFree(c->q);
    if (c->offs) cudaFree(c->offs);
    if (c->tmap) cudaFree(c->tmap);
    if (c->q_host) cudaFreeHost(c->q_host);
    if (c->ev_begin) cudaEventDestroy(c->ev_begin);
    if (c->ev_end) cudaEventDestroy(c->ev_end);
    if (c->ev_done) cudaEventDestroy(c->ev_done);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    for (cudaEvent_t ev : c->ev_piece)
      if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : c->ev_slice)
      if (ev) cudaEventDestroy(ev);
    if (c->q_acc) cudaFree(c->q_acc);
    if (c->merge_splits) cudaFree(c->merge_splits);
    if (c->split_buf) cudaFree(c->split_buf);
  }
  delete c;
}

gqs_status gqs_reserve(gqs_ctx* c, int dtype, size_t n, size_t nseg, int with_buffers) {
  if (!c || dtype < 0 || dtype > 2) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  (void)wait_pending_locked(c);
  const int v = c->auto_variant[dtype] ? gqs::tuned_variant(dtype, n, c->num_sms) : c->variant[dtype];
  const gqs::VariantInfo vi = gqs::variant_info(dtype, v);
  if (!c->blocks_per_sm[dtype][v]) {
    c->blocks_per_sm[dtype][v] = gqs::variant_prepare(dtype, v);
    if (!c->blocks_per_sm[dtype][v]) return GQS_ERR_NO_DEVICE;
  }
  if (n >= (1ull << 40) || nseg >= (1ull << 31)) return GQS_ERR_INVALID;
  // a plain sort of this size may start with the top split: its buckets are segments, and it
  // has scratch of its own
  gqs::SplitPlan plan{};
  const bool split = nseg <= 1 && c->top_split && gqs::split_plan(dtype, n, vi.tile, c->num_sms, &plan);
  if (split) {
    nseg = plan.k;
    gqs_status st = grow(&c->split_buf, &c->split_bytes, gqs::split_scratch_bytes(plan));
    if (st != GQS_OK) return st;
  }
  const size_t cap = job_capacity(vi, n, nseg ? nseg : 1);
  if (cap >= (1ull << 32) || ticket_ring(vi, n, nseg ? nseg : 1) > (1ull << 31)) return GQS_ERR_INVALID;
  if (c->job_cap < cap) {
    void* p = c->jobs;
    size_t bytes = c->job_cap * sizeof(gqs::Job);
    gqs_status st = grow(&p, &bytes, cap * sizeof(gqs::Job));
    c->jobs = static_cast<gqs::Job*>(p);
    c->job_cap = c->jobs ? bytes / sizeof(gqs::Job) : 0;
    if (st != GQS_OK) return st;
  }
  const size_t ring = ticket_ring(vi, n, nseg ? nseg : 1);
  if (c->tmap_len < ring) {
    void* p = c->tmap;
    size_t bytes = c->tmap_len * sizeof(unsigned long long);
    gqs_status st = grow(&p, &bytes, ring * sizeof(unsigned long long));
    c->tmap = static_cast<unsigned long long*>(p);
    c->tmap_len = c->tmap ? ring : 0;
    if (st != GQS_OK) return st;
  }
  const size_t bytes = n * kElemSize[dtype];
  gqs_status st = grow(&c->pool_dn, &c->pool_dn_bytes, bytes);
  if (st != GQS_OK) return st;
  if (with_buffers) {
    st = grow(&c->pool_d, &c->pool_d_bytes, bytes);
    if (st != GQS_OK) return st;
    void* po = c->offs;
    st = grow(&po, &c->offs_cap, ((nseg ? nseg : 1) + 1) * sizeof(uint64_t));
    c->offs = static_cast<unsigned long long*>(po);
    if (st != GQS_OK) return st;
  }
  return GQS_OK;
}

gqs_status gqs_sort_u32(gqs_ctx* c, uint32_t* d, uint32_t*, size_t n) { return sort_host(c, gqs::DT_U32, d, n); }
gqs_status gqs_sort_f32(gqs_ctx* c, float* d, float*, size_t n) { return sort_host(c, gqs::DT_F32, d, n); }
gqs_status gqs_sort_f64(gqs_ctx* c, double* d, double*, size_t n) { return sort_host(c, gqs::DT_F64, d, n); }

gqs_status gqs_sort_u32_dev(gqs_ctx* c, uint32_t* d, uint32_t* s, size_t n, void* stream) {
  return sort_dev(c, gqs::DT_U32, d, s, n, stream);
}
gqs_status gqs_sort_f32_dev(gqs_ctx* c, float* d, float* s, size_t n, void* stream) {
  return sort_dev(c, gqs::DT_F32, d, s, n, stream);
}
gqs_status gqs_sort_f64_dev(gqs_ctx* c, double* d, double* s, size_t n, void* stream) {
  return sort_dev(c, gqs::DT_F64, d, s, n, stream);
}

gqs_status gqs_sort_segments_u32_dev(gqs_ctx* c, uint32_t* k, uint32_t* s, size_t n, const uint64_t* o, size_t ns,
                                     void* stream) {
  return sort_segments_dev(c, gqs::DT_U32, k, s, n, o, ns, stream);
}
gqs_status gqs_sort_segments_f32_dev(gqs_ctx* c, float* k, float* s, size_t n, const uint64_t* o, size_t ns,
                                     void* stream) {
  return sort_segments_dev(c, gqs::DT_F32, k, s, n, o, ns, stream);
}
gqs_status gqs_sort_segments_f64_dev(gqs_ctx* c, double* k, double* s, size_t n, const uint64_t* o, size_t ns,
                                     void* stream) {
  return sort_segments_dev(c, gqs::DT_F64, k, s, n, o, ns, stream);
}
gqs_status gqs_sort_segments_u32(gqs_ctx* c, uint32_t* k, size_t n, const uint64_t* o, size_t ns) {
  return sort_segments_host(c, gqs::DT_U32, k, n, o, ns);
}
gqs_status gqs_sort_segments_f32(gqs_ctx* c, float* k, size_t n, const uint64_t* o, size_t ns) {
  return sort_segments_host(c, gqs::DT_F32, k, n, o, ns);
}
gqs_status gqs_sort_segments_f64(gqs_ctx* c, double* k, size_t n, const uint64_t* o, size_t ns) {
  return sort_segments_host(c, gqs::DT_F64, k, n, o, ns);
}

gqs_status gqs_selftest_stalled_queue(gqs_ctx* c, int dtype, uint32_t timeout_ms) {
  if (!c || dtype < 0 || dtype > 2) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  (void)wait_pending_locked(c);
  const int v = c->variant[dtype];
  const gqs::VariantInfo vi = gqs::variant_info(dtype, v);
  if (!c->blocks_per_sm[dtype][v]) {
    c->blocks_per_sm[dtype][v] = gqs::variant_prepare(dtype, v);
    if (!c->blocks_per_sm[dtype][v]) return GQS_ERR_NO_DEVICE;
  }
  const size_t n = 1024;  // pools for a small sort; the kernel touches none of the keys
  const size_t cap = job_capacity(vi, n, 1), ring = ticket_ring(vi, n, 1);
  gqs_status st = GQS_OK;
  if (c->job_cap < cap) {
    void* p = c->jobs;
    size_t bytes = c->job_cap * sizeof(gqs::Job);
    st = grow(&p, &bytes, cap * sizeof(gqs::Job));
    c->jobs = static_cast<gqs::Job*>(p);
    c->job_cap = c->jobs ? bytes / sizeof(gqs::Job) : 0;
    if (st != GQS_OK) return st;
  }
  if (c->tmap_len < ring) {
    void* p = c->tmap;
    size_t bytes = c->tmap_len * sizeof(unsigned long long);
    st = grow(&p, &bytes, ring * sizeof(unsigned long long));
    c->tmap = static_cast<unsigned long long*>(p);
    c->tmap_len = c->tmap ? ring : 0;
    if (st != GQS_OK) return st;
  }
  if ((st = grow(&c->pool_dn, &c->pool_dn_bytes, n * kElemSize[dtype])) != GQS_OK) return st;
  void* po = c->offs;
  st = grow(&po, &c->offs_cap, 4 * sizeof(uint64_t));
  c->offs = static_cast<unsigned long long*>(po);
  if (st != GQS_OK) return st;
  // The queue claims one key (total = 1) while the segment count is zero: no job is ever seeded,
  // so done never reaches total and every wait runs into its limit.
  std::memset(c->q_host, 0, sizeof(gqs::Queue));
  c->q_host->total = 1;
  cudaError_t e = cudaMemcpyAsync(c->q, c->q_host, sizeof(gqs::Queue), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->offs, 0, 4 * sizeof(uint64_t), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->tmap, 0, ring * sizeof(unsigned long long), c->stream);
  if (e != cudaSuccess) return cuda_status(e);
  gqs::LaunchParams p{};
  p.d = c->pool_dn;
  p.dn = c->pool_dn;
  p.jobs = c->jobs;
  p.q = c->q;
  p.tmap = c->tmap;
  p.capacity = (uint32_t)c->job_cap;
  p.tmask = (uint32_t)(ring - 1);
  p.timeout_ns = (unsigned long long)(timeout_ms ? timeout_ms : (c->cfg.timeout_ms ? c->cfg.timeout_ms : 4000)) *
                 1000000ull;
  p.offsets = c->offs + 1;
  p.nseg_dev = c->offs;  // zero segments
  p.nseg = 1;
  p.n = n;
  p.variant = v;
  p.grid = c->num_sms * c->blocks_per_sm[dtype][v];
  p.stream = c->stream;
  e = gqs::launch_sort(dtype, p);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_done, c->stream);
  if (e != cudaSuccess) return cuda_status(e);
  c->pending = true;
  c->pending_timed = false;
  c->pending_dtype = dtype;
  c->pending_variant = v;
  c->pending_grid = p.grid;
  c->pending_keys = 0;
  return wait_pending_locked(c);
}

gqs_status gqs_selftest_bounds(gqs_ctx* c, int dtype) {
  if (!c || dtype < 0 || dtype > 2) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  const size_t n = 1u << 16, es = kElemSize[dtype];
  (void)wait_pending_locked(c);
  gqs_status st = grow(&c->pool_d, &c->pool_d_bytes, n * es);
  if (st != GQS_OK) return st;
  // equal keys (0x5a bytes: an ordinary value for every key type); any keys would do
  cudaError_t e = cudaMemsetAsync(c->pool_d, 0x5a, n * es, c->stream);
  if (e != cudaSuccess) return cuda_status(e);
  st = enqueue_locked(c, dtype, c->pool_d, nullptr, n, nullptr, 1, c->stream, n / 2);
  if (st != GQS_OK) return st;
  return wait_pending_locked(c);
}

gqs_status gqs_sync(gqs_ctx* c) {
  if (!c) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  if (!c->pending) return (gqs_status)c->last.status;
  return wait_pending_locked(c);
}

gqs_status gqs_last_stats(gqs_ctx* c, gqs_stats* out) {
  if (!c || !out) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  gqs_status st = wait_pending_locked(c);
  *out = c->last;
  return st == GQS_OK ? GQS_OK : st;
}

int gqs_last_profile(gqs_ctx* c, uint64_t* out, size_t n) {
  if (!c || !out) return 0;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  (void)wait_pending_locked(c);
  const size_t k = n < 32 ? n : 32;
  for (size_t i = 0; i < k; ++i) out[i] = c->last_prof[i];
  return (int)k;
}

gqs_status gqs_last_phases(gqs_ctx* c, gqs_phases* out) {
  if (!c || !out) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  const gqs_status st = wait_pending_locked(c);
  // partition chunks are not timed one by one (see Queue::phase): they are the remainder
  const uint64_t rest = c->last_phase[1] + c->last_phase[2];
  out->partition_cycles = c->last_phase[3] > rest ? c->last_phase[3] - rest : 0;
  out->onchip_cycles = c->last_phase[1];
  out->fill_cycles = c->last_phase[2];
  out->total_cycles = c->last_phase[3];
  return st;
}

int gqs_last_levels(gqs_ctx* c, gqs_level* out, int max) {
  if (!c || !out || max <= 0) return 0;
  std::lock_guard<std::mutex> lk(c->mu);
  DeviceGuard dg(c->device);
  (void)wait_pending_locked(c);
#ifdef GQS_PROFILE
  int k = 0;
  for (int d = 0; d < gqs::kLevels && k < max; ++d) {
    const unsigned long long* r = c->last_lvl[d];
    if (!r[0] && !r[2]) continue;
    gqs_level& L = out[k++];
    L.depth = (uint32_t)d;
    L.part_jobs = (uint32_t)r[0];
    L.part_keys = r[1];
    L.local_jobs = (uint32_t)r[2];
    L.reserved = 0;
    L.local_keys = r[3];
    const long long t0 = (long long)c->last_lvl_start;
    L.first_ms = r[4] ? (double)((long long)r[4] - t0) / 1e6 : 0.0;
    L.last_ms = r[5] ? (double)((long long)r[5] - t0) / 1e6 : 0.0;
  }
  return k;
#else
  return 0;
#endif
}

int gqs_variant_count(int dtype) { return gqs::variant_count(dtype); }

gqs_status gqs_variant_describe(int dtype, int v, gqs_variant_desc* out) {
  if (!out || dtype < 0 || dtype > 2 || v < 0 || v >= gqs::variant_count(dtype)) return GQS_ERR_INVALID;
  const gqs::VariantInfo vi = gqs::variant_info(dtype, v);
  out->threads = vi.threads;
  out->tile = vi.tile;
  out->chunk = vi.chunk;
  out->kpt = vi.kpt;
  out->stages = vi.stages;
  out->tiny = vi.tiny;
  out->smem_bytes = vi.smem;
  std::memset(out->name, 0, sizeof(out->name));
  std::strncpy(out->name, vi.name, sizeof(out->name) - 1);
  return GQS_OK;
}

gqs_status gqs_set_variant(gqs_ctx* c, int dtype, int v) {
  if (!c || dtype < 0 || dtype > 2 || v < 0 || v >= gqs::variant_count(dtype)) return GQS_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  c->variant[dtype] = v;
  c->auto_variant[dtype] = false;
  return GQS_OK;
}

int gqs_get_variant(gqs_ctx* c, int dtype) {
  if (!c || dtype < 0 || dtype > 2) return -1;
  return c->auto_variant[dtype] ? -1 : c->variant[dtype];
}

const char* gqs_strerror(gqs_status s) {
  switch (s) {
    case GQS_OK: return "ok";
    case GQS_ERR_INVALID: return "invalid argument";
    case GQS_ERR_CUDA: return "CUDA runtime error";
    case GQS_ERR_NOMEM: return "out of memory";
    case GQS_ERR_TIMEOUT: return "device wait timed out (no progress)";
    case GQS_ERR_CAPACITY: return "device job queue overflow";
    case GQS_ERR_NO_DEVICE: return "no sm_103 CUDA device";
    case GQS_ERR_INTERNAL: return "internal error";
    case GQS_ERR_CANCELLED: return "request cancelled";
    case GQS_ERR_BOUNDS: return "an index or record outside the sort's bounds (check build)";
  }
  return "unknown status";
}

int gqs_version(void) { return 1; }

}  // extern "C"
