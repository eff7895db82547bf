// Top split of a small plain sort: one multi-way partition of the whole array into buckets
// that the persistent kernel then sorts as segments (most of them as single on-chip tiles).
//
// Below a few million keys a binary partition level is bound by latency, not bandwidth: each
// level waits for its jobs' last chunks, the completer's pivot sampling and the publication of
// the children (about 11 us a level on a GB300), and 2^20 keys need seven levels before every
// range fits one on-chip tile. The split replaces those levels with four short kernels over an
// array that stays in L2:
//   split_pick     one CTA: sorts 8 samples per bucket (runs of 256 by warp networks, then
//                  merged pairwise by merge path) and keeps every 8th as a splitter, stored
//                  as a breadth-first search tree (the on-chip split's layout and bucket rule:
//                  bucket b holds splitter[b-1] < key <= splitter[b]);
//   split_count    every CTA walks the tree for each key of its slice, counts per bucket in
//                  shared memory and adds its counts to the bucket totals;
//   split_starts   one CTA: exclusive scan of the bucket totals into the segment table and the
//                  scatter cursors;
//   split_scatter  every CTA walks the tree again, reserves its share of each bucket with one
//                  atomic and appends each key to its bucket in dn.
// The split is the reference's partition generalised from one pivot to k - 1 (the sample split
// the on-chip sort already uses for a tile, applied once to the whole array); its pass is
// counted in the sort's partition keys.
#include <cuda_runtime.h>

#include <cstdint>

#include "gqs_device.cuh"
#include "gqs_launch.h"

namespace gqs {
namespace {

constexpr int kThreads = 512;
constexpr int kRun = 256;            // samples per warp-sorted run (8 per lane)
constexpr uint32_t kMaxK = 1024;     // buckets
constexpr uint32_t kMaxSamples = 4096;
constexpr uint32_t kOversample = 8;  // samples per bucket
constexpr uint32_t kMaxSlice = 16384;  // keys of one CTA's slice in the scatter (labels in shared memory)

template <class T>
using BOf = typename KeyOps<T>::B;

// Dynamic shared memory of split_pick: two sample buffers.
extern __shared__ __align__(16) unsigned char split_dyn[];

template <class T>
__global__ void __launch_bounds__(kThreads) split_pick(const BOf<T>* __restrict__ d, unsigned long long n, uint32_t k,
                                                        uint32_t lg, uint32_t ns, BOf<T>* __restrict__ tree,
                                                        uint32_t* __restrict__ total, Queue* q) {
  using B = BOf<T>;
  B* src = reinterpret_cast<B*>(split_dyn);
  B* dst = src + kMaxSamples;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  pdl_trigger();  // split_count may launch now; it waits for this grid before reading the tree
  for (uint32_t i = tid; i < k; i += kThreads) total[i] = 0u;
#ifdef GQS_PROFILE
  if (tid == 0) atomicCAS(&q->lvl_start, 0ull, (unsigned long long)global_timer_ns());  // per-level times start here
#else
  (void)q;
#endif
  const uint32_t nrun = ns / kRun;
  if ((uint32_t)warp < nrun) {
    B v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const unsigned long long i = (unsigned long long)warp * kRun + (unsigned long long)(r * 32 + lane);
      v[r] = KeyOps<T>::key(d[(i * n) / ns]);
    }
    warp_bitonic_n<8, 1, B>(v);  // element lane * 8 + r of the run
#pragma unroll
    for (int r = 0; r < 8; ++r) src[warp * kRun + lane * 8 + r] = v[r];
  }
  __syncthreads();
  // Merge the sorted runs pairwise until one run remains: each thread writes `per` consecutive
  // outputs of one pair, starting where merge path puts its first output (the number of keys
  // the first run contributes before it, by binary search on the diagonal).
  const uint32_t per = ns / kThreads;  // ns is 256 << j; with ns >= 512, per divides every pair
  for (uint32_t len = kRun; len < ns; len <<= 1) {
    if (per > 0) {
      const uint32_t o0 = (uint32_t)tid * per, base = o0 / (2u * len) * (2u * len), dg = o0 - base;
      const B* x = src + base;
      const B* y = x + len;
      uint32_t lo = dg > len ? dg - len : 0u, hi = dg < len ? dg : len;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (x[mid] <= y[dg - 1u - mid]) lo = mid + 1u;
        else hi = mid;
      }
      uint32_t i = lo, j = dg - lo;
      for (uint32_t t = 0; t < per; ++t) {
        const bool from_x = j >= len || (i < len && x[i] <= y[j]);
        dst[o0 + t] = from_x ? x[i++] : y[j++];
      }
    }
    __syncthreads();
    B* const tmp = src;
    src = dst;
    dst = tmp;
  }
  // splitter q1 - 1 is the sample of rank q1 * step - 1
  const uint32_t step = ns / k;
  for (uint32_t q1 = (uint32_t)tid + 1u; q1 < k; q1 += kThreads) {
    const uint32_t tz = (uint32_t)__ffs(q1) - 1u;
    tree[(1u << (lg - 1u - tz)) + (q1 >> (tz + 1u))] = src[q1 * step - 1u];
  }
}

template <class T>
__device__ __forceinline__ uint32_t bucket_of(const BOf<T>* t, uint32_t lg, BOf<T> key) {
  uint32_t b = 1u;
  for (uint32_t l = 0; l < lg; ++l) b = 2u * b + (t[b] < key ? 1u : 0u);
  return b;
}

// Buckets (0 .. k-1) of kBatch keys per thread at once: keys lo + tid + j * kThreads of
// [lo, hi); all loads are issued before the tree walks, which then run interleaved. Keys past
// hi get bucket kNone.
constexpr int kBatch = 8;
constexpr uint32_t kNone = 0xffffffffu;
template <class T>
__device__ __forceinline__ void buckets_of(const BOf<T>* __restrict__ d, unsigned long long i0, unsigned long long hi,
                                           const BOf<T>* t, uint32_t k, uint32_t lg, uint32_t (&b)[kBatch],
                                           BOf<T> (&raw)[kBatch]) {
  BOf<T> key[kBatch];
#pragma unroll
  for (int j = 0; j < kBatch; ++j) {
    const unsigned long long i = i0 + (unsigned long long)j * kThreads;
    raw[j] = i < hi ? d[i] : BOf<T>(0);
    key[j] = KeyOps<T>::key(raw[j]);
    b[j] = 1u;
  }
  for (uint32_t l = 0; l < lg; ++l) {
#pragma unroll
    for (int j = 0; j < kBatch; ++j) b[j] = 2u * b[j] + (t[b[j]] < key[j] ? 1u : 0u);
  }
#pragma unroll
  for (int j = 0; j < kBatch; ++j) b[j] = i0 + (unsigned long long)j * kThreads < hi ? b[j] - k : kNone;
}

// CTA c's slice of the keys: [c * n / ctas, (c + 1) * n / ctas).
__device__ __forceinline__ void slice_of(unsigned long long n, uint32_t ctas, unsigned long long& lo,
                                         unsigned long long& hi) {
  lo = n * blockIdx.x / ctas;
  hi = n * (blockIdx.x + 1ull) / ctas;
}

template <class T>
__global__ void __launch_bounds__(kThreads) split_count(const BOf<T>* __restrict__ d, unsigned long long n, uint32_t k,
                                                         uint32_t lg, const BOf<T>* __restrict__ tree,
                                                         uint32_t* __restrict__ total) {
  using B = BOf<T>;
  __shared__ B t[kMaxK];
  __shared__ uint32_t cnt[kMaxK];
  pdl_wait();
  pdl_trigger();
  for (uint32_t i = threadIdx.x; i < k; i += kThreads) {
    t[i] = tree[i];
    cnt[i] = 0u;
  }
  __syncthreads();
  unsigned long long lo, hi;
  slice_of(n, gridDim.x, lo, hi);
  for (unsigned long long i0 = lo + threadIdx.x; i0 < hi; i0 += (unsigned long long)kBatch * kThreads) {
    uint32_t b[kBatch];
    B raw[kBatch];
    buckets_of<T>(d, i0, hi, t, k, lg, b, raw);
#pragma unroll
    for (int j = 0; j < kBatch; ++j)
      if (b[j] != kNone) atomicAdd(&cnt[b[j]], 1u);
  }
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < k; b += kThreads)
    if (cnt[b]) atomicAdd(&total[b], cnt[b]);
}

// One CTA of kMaxK threads: bucket starts from the bucket totals (exclusive scan); they become
// the segment table (segs[k] = n) and the scatter cursors.
__global__ void __launch_bounds__(kMaxK) split_starts(const uint32_t* __restrict__ total, uint32_t k,
                                                      unsigned long long n, uint32_t* __restrict__ cursor,
                                                      unsigned long long* __restrict__ segs, Queue* q) {
  __shared__ uint32_t wsum[32];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  pdl_wait();
  pdl_trigger();
  const uint32_t c = tid < k ? total[tid] : 0u;
  uint32_t inc = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
    if ((int)lane >= o) inc += v;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = wsum[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, wi, o);
      if ((int)lane >= o) wi += v;
    }
    wsum[lane] = wi - w;
  }
  __syncthreads();
  if (tid < k) {
    const uint32_t start = wsum[warp] + inc - c;
    cursor[tid] = start;
    segs[tid] = start;
  }
  if (tid == 0) {
    segs[k] = n;
    atomicAdd(&q->part_keys, n);  // the split is one partition job and one pass over every key
    atomicAdd(&q->part_jobs, 1u);
#ifdef GQS_PROFILE
    level_note(q, 0, 0, n);  // and the depth-0 job of the profiling library's per-level rows
#endif
  }
}

// Every CTA labels the keys of its slice (labels kept in shared memory), reserves its share of
// every bucket with one global atomic per bucket, and appends each key to its bucket in dn. The
// order of the CTAs' shares inside a bucket does not matter: the bucket is sorted afterwards.
template <class T>
__global__ void __launch_bounds__(kThreads) split_scatter(const BOf<T>* __restrict__ d, BOf<T>* __restrict__ dn,
                                                           unsigned long long n, uint32_t k, uint32_t lg,
                                                           const BOf<T>* __restrict__ tree,
                                                           uint32_t* __restrict__ cursor) {
  using B = BOf<T>;
  __shared__ B t[kMaxK];
  __shared__ uint32_t cur[kMaxK];
  __shared__ uint16_t lab[kMaxSlice];
  pdl_wait();
  pdl_trigger();
  for (uint32_t i = threadIdx.x; i < k; i += kThreads) {
    t[i] = tree[i];
    cur[i] = 0u;
  }
  __syncthreads();
  unsigned long long lo, hi;
  slice_of(n, gridDim.x, lo, hi);  // hi - lo <= kMaxSlice (split_plan)
  for (unsigned long long i0 = lo + threadIdx.x; i0 < hi; i0 += (unsigned long long)kBatch * kThreads) {
    uint32_t b[kBatch];
    B raw[kBatch];
    buckets_of<T>(d, i0, hi, t, k, lg, b, raw);
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      if (b[j] == kNone) continue;
      lab[i0 + (unsigned long long)j * kThreads - lo] = (uint16_t)b[j];
      atomicAdd(&cur[b[j]], 1u);
    }
  }
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < k; b += kThreads)
    if (cur[b]) cur[b] = atomicAdd(&cursor[b], cur[b]);
  __syncthreads();
  for (unsigned long long i0 = lo + threadIdx.x; i0 < hi; i0 += (unsigned long long)kBatch * kThreads) {
    B raw[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const unsigned long long i = i0 + (unsigned long long)j * kThreads;
      raw[j] = i < hi ? d[i] : B(0);
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const unsigned long long i = i0 + (unsigned long long)j * kThreads;
      if (i >= hi) continue;
      const uint32_t pos = atomicAdd(&cur[lab[i - lo]], 1u);
      dn[pos] = raw[j];  // pos < n: the bucket's reserved range holds exactly these keys
    }
  }
}

// Scratch layout: tree (kMaxK keys of 8 bytes), segment table (kMaxK + 1), totals, cursors.
constexpr size_t kTreeBytes = kMaxK * 8;
constexpr size_t kSegBytes = ((kMaxK + 1) * 8 + 255) / 256 * 256;
constexpr size_t kCountBytes = kMaxK * 4;

template <class T>
cudaError_t launch_t(const SplitPlan& p, const void* d, void* dn, size_t n, void* scratch, unsigned long long** segs,
                     Queue* q, cudaStream_t s) {
  using B = BOf<T>;
  char* base = static_cast<char*>(scratch);
  B* tree = reinterpret_cast<B*>(base);
  unsigned long long* sg = reinterpret_cast<unsigned long long*>(base + kTreeBytes);
  uint32_t* total = reinterpret_cast<uint32_t*>(base + kTreeBytes + kSegBytes);
  uint32_t* cursor = total + kMaxK;
  const B* src = static_cast<const B*>(d);
  constexpr size_t kPickSmem = 2 * kMaxSamples * sizeof(B);
  static const cudaError_t attr =
      cudaFuncSetAttribute(split_pick<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPickSmem);
  if (attr != cudaSuccess) return attr;
  // Each kernel after the first is a programmatic dependent launch of the one before (and the
  // seed and persistent kernels follow the same way), so that each launches while the one
  // before it drains; split_pick also zeroes the bucket totals.
  split_pick<T><<<1, kThreads, kPickSmem, s>>>(src, n, p.k, p.lg, p.samples, tree, total, q);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = launch_kernel(true, split_count<T>, dim3(p.ctas), dim3(kThreads), 0, s, src, (unsigned long long)n, p.k, p.lg,
                      (const B*)tree, total);
  if (e == cudaSuccess)
    e = launch_kernel(true, split_starts, dim3(1), dim3(kMaxK), 0, s, (const uint32_t*)total, p.k,
                      (unsigned long long)n, cursor, sg, q);
  if (e == cudaSuccess)
    e = launch_kernel(true, split_scatter<T>, dim3(p.ctas), dim3(kThreads), 0, s, src, static_cast<B*>(dn),
                      (unsigned long long)n, p.k, p.lg, (const B*)tree, cursor);
  *segs = sg;
  return e;
}

}  // namespace

// Plain sorts of 2^15 .. 2^21 keys take the split (measured slower than the binary levels at
// 2^22 on a GB300): k = the power of two that gives buckets of
// about a third of a tile (so that nearly every bucket is one on-chip sort), at most kMaxK.
bool split_plan(int dtype, size_t n, int tile, int sms, SplitPlan* plan) {
  (void)dtype;
  if (n < (1u << 15) || n > (1u << 21)) return false;
  uint32_t k = 2, lg = 1;
  while (k < kMaxK && (unsigned long long)k * (unsigned long long)tile < 3ull * n) {
    k <<= 1;
    ++lg;
  }
  plan->k = k;
  plan->lg = lg;
  plan->samples = k * kOversample < (uint32_t)kRun ? (uint32_t)kRun : k * kOversample;
  if (plan->samples > kMaxSamples) plan->samples = kMaxSamples;
  size_t ctas = n / 4096;  // about 4096 keys per CTA, at most two CTAs per SM ...
  if (ctas > (size_t)(2 * sms)) ctas = (size_t)(2 * sms);
  const size_t need = (n + kMaxSlice - 1) / kMaxSlice;  // ... and never more than kMaxSlice keys
  if (ctas < need) ctas = need;
  plan->ctas = (uint32_t)(ctas < 1 ? 1 : ctas);
  return true;
}

size_t split_scratch_bytes(const SplitPlan& plan) {
  (void)plan;
  return kTreeBytes + kSegBytes + 2 * kCountBytes;
}

cudaError_t split_launch(int dtype, const SplitPlan& plan, const void* d, void* dn, size_t n, void* scratch,
                         unsigned long long** segs, Queue* q, cudaStream_t s) {
  switch (dtype) {
    case DT_U32: return launch_t<uint32_t>(plan, d, dn, n, scratch, segs, q, s);
    case DT_F32: return launch_t<float>(plan, d, dn, n, scratch, segs, q, s);
    case DT_F64: return launch_t<double>(plan, d, dn, n, scratch, segs, q, s);
    default: return launch_t<uint64_t>(plan, d, dn, n, scratch, segs, q, s);
  }
}

}  // namespace gqs
