// GPU-Quicksort for sm_103a: one persistent kernel that drains a device-resident
// queue of partition jobs, so the host never round-trips between levels.
//
// Reference mapping (GPU-Quicksort, rioffe/gpu-quicksort):
//   * partition job  <- gqsort_kernel (GPU-Quicksort_OpenCL_1.2/QuicksortKernels.cl:102-240;
//                       GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:547-710)
//   * local job      <- lqsort_kernel (QuicksortKernels.cl:267-421; QuicksortMain.cpp:286-542)
//   * warp bitonic   <- bitonic_sort / sort_threshold (QuicksortKernels.cl:40-97)
//   * job queue      <- the host level loop of GPUQSort<T> (QuicksortMain.cpp:835-906) and the
//                       OpenCL 2.0 device-side relaunch (GPU-Quicksort_OpenCL_2.0/QuicksortKernels.cl:132-222)
//   * Job            <- work_record / parent_record / block_record (GPU-Quicksort_Full_SYCL/Quicksort.h:145-184)
//
// Roles inside one CTA (one CTA per SM):
//   warps [0, NCW)  consumers: partition staged chunks, run local (on-chip) sorts, fill pivot runs
//   warp  NCW       producer:  takes work from the global queue and stages it in shared memory with
//                              bulk TMA copies (cp.async.bulk + mbarrier), STAGES deep
//   warp  NCW+1     completer: finishes a partition job once its last chunk is written (pivot run,
//                              child pivots, children pushed back to the queue or sorted in registers)
//
// Keys are compared through an order-preserving map to unsigned integers (identity for uint32;
// for float/double the sign-magnitude bit flip), so every comparison runs on the integer pipes
// and no float/double compare instruction is issued. Memory always holds the caller's raw bits.
#pragma once
#include <cstdint>
#include <cstring>
#include "gqs_ptx.cuh"

namespace gqs {

// ---------------------------------------------------------------------------
// Status codes written by the kernels (the C ABI uses the same numbers).
enum : uint32_t { ST_OK = 0, ST_INVALID = 1, ST_TIMEOUT = 4, ST_CAPACITY = 5, ST_INTERNAL = 7, ST_BOUNDS = 9 };

enum : uint32_t { JOB_PART = 1, JOB_LOCAL = 2, JOB_FILL = 3 };
enum : uint32_t { ITEM_PART = 1, ITEM_LOCAL = 2, ITEM_FILL = 3, ITEM_TERM = 4, ITEM_FLUSH = 5, ITEM_NONE = 6 };

// One queued unit of work. A partition job covers [start, end) of its source buffer and is
// cut into chunks on a grid aligned to 16 bytes of the source; its children are written
// to the other buffer. `dir` follows the reference's `direction`: 1 reads d, 0 reads dn.
// Every chunk of every job owns one ticket; tickets [t0, t0 + nchunks) belong to this job.
struct alignas(16) Job {
  unsigned long long start, end;
  unsigned long long sstart, send;  // reservation cursors: less-than grows up, greater-than down
  unsigned long long pivot;         // comparison key of the pivot
  long long grid;                   // element index of the chunk grid origin (may be < start)
  uint32_t kind, dir, nchunks, t0;
  uint32_t remaining, depth, pad0, pad1;
};
static_assert(sizeof(Job) == 80, "job record layout");

// Per-sort device state. Reset by the host (memset) before the seed kernel.
// Work is handed out by ticket: `grab` counts tickets taken, the low half of `alloc` counts
// tickets created and its high half job records created. The ticket map (SortArgs::tmap)
// holds ((ticket + 1) << 32 | job slot) at index ticket & tmask once the job is published.
constexpr int kLevels = 48;  // rows of the per-level statistics of a -DGQS_PROFILE build

struct Queue {
  unsigned long long total;  // keys in this sort
  unsigned long long done;   // keys in their final place
  unsigned long long alloc;  // (jobs << 32) | tickets
  uint32_t grab, error;
  unsigned long long error_info;
  unsigned long long part_keys, local_keys, tiny_keys, fill_keys, chunks;
  uint32_t part_jobs, local_jobs, fill_jobs, max_depth;
  // Cycles of each CTA's consumer leader thread, summed over CTAs: [1] on-chip sorts (tile wait,
  // sort, write-out), [2] queued pivot-run fills, [3] the whole consumer loop; the rest of [3] is
  // partition chunks, pipeline drains and waits for work ([0] is unused: a clock read per chunk
  // on the leader's path cost 5 % of a large sort).
  unsigned long long phase[4];
  unsigned long long prof[32];  // cycle counters of a -DGQS_PROFILE build (zero otherwise)
#ifdef GQS_PROFILE
  // Per partition level (job depth; the last row takes every deeper level) in a -DGQS_PROFILE
  // build, the counterpart of the reference's optional per-level timing: partition jobs and
  // their keys, on-chip jobs and their keys, and the global-timer times of a first and the
  // last completion at that depth; lvl_start is the first CTA's start.
  unsigned long long lvl_start;
  unsigned long long lvl[kLevels][6];
#endif
};

// Optional cycle accounting per role (compile with -DGQS_PROFILE); slots:
enum : int {
  PF_C_WAIT = 0,     // consumer leader: waiting for the next ring slot
  PF_C_PART = 1,     // consumers: partition chunk iterations
  PF_C_DRAIN = 2,    // consumers: draining before a non-partition item
  PF_C_LWAIT = 3,    // consumers: waiting for a local tile
  PF_C_LCTA = 4,     // local sort, CTA-wide phase (incl. key mapping)
  PF_C_LWARP = 5,    // local sort, warp phase
  PF_C_LSTORE = 6,   // local sort, write-out
  PF_C_FILL = 7,     // fill items
  PF_P_GRAB = 8,     // producer: taking work from the queue
  PF_P_EMPTY = 9,    // producer: waiting for a free stage
  PF_P_LEMPTY = 10,  // producer: waiting for the tile region
  PF_P_IDLE = 11,    // producer: no work available
  PF_Q_BUSY = 12,    // completer: finishing jobs
  PF_Q_IDLE = 13,    // completer: idle
  PF_N_LOCAL = 14,   // local jobs
  PF_C_TOTAL = 15,   // consumer leader: whole run
  PF_P_ISSUE = 16,   // producer: staging (descriptor + bulk copy issue)
  PF_N_GRAB = 17,    // producer: global queue operations
  PF_N_LCTA = 18,    // local sort: CTA-wide partitions
  PF_N_LWARP = 19,   // local sort: warp partitions
  PF_N_LBIT = 20,    // local sort: register sorts
  PF_N_ITEMS = 21,   // ring items consumed
  PF_C_COUNT = 22,   // consumers: load + count of a chunk, up to barrier #1
  PF_C_LEADER = 23,  // consumers: barrier #1 to barrier #2 (leader's reservation work)
  PF_C_SCATTER = 24, // consumers: scatter of the pending chunk
  PF_W_WAIT = 25,    // local sort, summed over warps: cycles inside slices (incl. finishing)
  PF_W_PART = 26,    // local sort: segments finished
  PF_W_BIT = 27,     // local sort, summed over warps: register sorts
  PF_W_SEGS = 28,    // (unused)
  PF_COUNT = 29
};
#ifdef GQS_PROFILE
#define GQS_PROF_DECL unsigned long long prof_[PF_COUNT] = {};
#define GQS_PROF_T(v) const long long v = clock64();
#define GQS_PROF_ADD(i, v) prof_[i] += (unsigned long long)(clock64() - (v));
#define GQS_PROF_CNT(i, n) prof_[i] += (unsigned long long)(n);
#define GQS_PROF_FLUSH(q)                                             \
  for (int i_ = 0; i_ < PF_COUNT; ++i_)                               \
    if (prof_[i_]) atomicAdd(&(q)->prof[i_], prof_[i_]);
#else
#define GQS_PROF_DECL
#define GQS_PROF_T(v)
#define GQS_PROF_ADD(i, v)
#define GQS_PROF_CNT(i, n)
#define GQS_PROF_FLUSH(q)
#endif

template <class T>
struct KeyOps;
template <>
struct KeyOps<uint32_t> {
  using B = uint32_t;
  static __device__ __forceinline__ B key(B v) { return v; }
  static __device__ __forceinline__ B raw(B k) { return k; }
  static constexpr bool kIdentity = true;
};
template <>
struct KeyOps<float> {
  using B = uint32_t;
  static __device__ __forceinline__ B key(B u) { return u ^ ((uint32_t)((int32_t)u >> 31) | 0x80000000u); }
  static __device__ __forceinline__ B raw(B k) { return k ^ (~(uint32_t)((int32_t)k >> 31) | 0x80000000u); }
  static constexpr bool kIdentity = false;
};
// 64-bit unsigned keys: the packed (key, value) words of the pair sort.
template <>
struct KeyOps<uint64_t> {
  using B = uint64_t;
  static __device__ __forceinline__ B key(B v) { return v; }
  static __device__ __forceinline__ B raw(B k) { return k; }
  static constexpr bool kIdentity = true;
};
template <>
struct KeyOps<double> {
  using B = uint64_t;
  static __device__ __forceinline__ B key(B u) {
    return u ^ ((uint64_t)((int64_t)u >> 63) | 0x8000000000000000ull);
  }
  static __device__ __forceinline__ B raw(B k) {
    return k ^ (~(uint64_t)((int64_t)k >> 63) | 0x8000000000000000ull);
  }
  static constexpr bool kIdentity = false;
};

template <class T>
struct SortArgs {
  typename KeyOps<T>::B* d;
  typename KeyOps<T>::B* dn;
  Job* jobs;
  Queue* q;
  unsigned long long* tmap;  // ticket -> job slot ring (zeroed before each sort)
  uint32_t capacity;         // job records
  uint32_t tmask;            // ticket ring size - 1 (a power of two)
  unsigned long long timeout_ns;
  unsigned long long n;      // every key index of the sort is below n (checked by -DGQS_CHECK builds)
};

// Kernel configuration. TILE keys fit one local (on-chip) sort; CHUNK keys are one staged
// partition chunk; TINY = 32*R keys are sorted in registers by one warp.
// Mean bucket size of the on-chip sample split, as a fraction of the register sort: TINY / 8
// (32 u32 keys, 16 f64 keys; at most NB_MAX buckets per tile).
#ifndef GQS_BUCKET_DIV
#define GQS_BUCKET_DIV 8
#endif

template <class T_, int NCW_, int TILE_, int CHUNK_, int STAGES_, int R_>
struct Cfg {
  using T = T_;
  using Ops = KeyOps<T>;
  using B = typename Ops::B;
  static constexpr int NCW = NCW_;
  static constexpr int NC = NCW * 32;
  static constexpr int NT = NC + 96;  // + producer, completer and reserver warps
  static constexpr int TILE = TILE_;
  static constexpr int CHUNK = CHUNK_;
  static constexpr int STAGES = STAGES_;
  static constexpr int R = R_;
  static constexpr int TINY = 32 * R;
  static constexpr int KPT = CHUNK / NC;
  static constexpr int E16 = 16 / (int)sizeof(B);
  static constexpr int STAGE_ELEMS = CHUNK + 2 * E16;
  static constexpr int TILE_ELEMS = TILE + 2 * E16;
  static constexpr int FILL_INLINE = 16384;  // pivot runs up to this many keys are written by the completer
  static constexpr int FILL_CHUNK = 32768;   // longer runs become queued fill jobs of this grain
  static constexpr int CQ = 128;             // completer queue slots
  static constexpr int RQ = 32;              // reservation request slots
  // Local sort: segments are cut into slices of SLICE_KPL keys per lane (32 * SLICE_KPL per
  // slice) that any warp may partition; LREC segment records live in shared memory per tile.
  static constexpr int SLICE_KPL = sizeof(B) == 8 ? 8 : 16;
  static constexpr int SLICE = 32 * SLICE_KPL;
  static constexpr int LREC = 4 * TILE / TINY + 64;
  // Local sort, first level: a sample split into up to NB_MAX buckets (mean TINY / 4 keys),
  // used for tiles of at least SPLIT_MIN keys; SPLIT_SAMPLES keys are sorted to pick pivots.
  static constexpr int NB_MAX = 256;
  static constexpr int SPLIT_MIN = 8 * TINY;
  static constexpr int SPLIT_SAMPLES = 256;
  static constexpr int BUCKET = TINY / GQS_BUCKET_DIV;  // mean bucket size the split aims for
  static constexpr int NCLASS = 7;                     // bucket classes (network sizes), see sample_split
  static_assert(CHUNK % NC == 0, "chunk must be a multiple of the consumer threads");
  static_assert(NCW >= 3 && NCW <= 32, "the partition loop's bookkeeping uses consumer warps 0, 1 and 2");
  static_assert((CHUNK * sizeof(B)) % 16 == 0, "chunk must be a multiple of 16 bytes");
  static_assert(TILE > TINY, "tile must exceed the register sort");
  static_assert(NB_MAX <= 256 && NB_MAX >= 32, "bucket labels are bytes; the scan takes 32..256 buckets");
  static_assert(NB_MAX == 256, "8 bucket counts per lane of one warp in the scan");
  static_assert(SPLIT_SAMPLES >= NB_MAX && NC >= SPLIT_SAMPLES, "one pivot per bucket; one thread per sample");
};

// A segment of the on-chip tile being partitioned slice by slice (shared memory).
struct LRec {
  unsigned long long pivot;
  uint32_t s, e, buf, nsl;  // [s, e) of buffer `buf`, cut into nsl slices
  uint32_t cursor;          // slices taken
  uint32_t remaining;       // slices not yet scattered
  uint32_t lt, gt;          // keys reserved below / above the pivot
  uint32_t seq;             // index + 1 once the record is published
  uint32_t pad;
};

struct Desc {
  unsigned long long gbeg;  // first element (global index) of the staged range
  unsigned long long pivot;
  uint32_t len, off, job, kind, dir, pad;
#ifdef GQS_CHECK
  unsigned long long jlo, jhi;  // the job's range: every key this item writes stays inside it
#endif
};

template <class C>
struct alignas(128) Smem {
  typename C::B stage[C::STAGES][C::STAGE_ELEMS];
  typename C::B tileA[C::TILE_ELEMS];
  typename C::B tileB[C::TILE_ELEMS];
  uint64_t full[C::STAGES], empty[C::STAGES], lfull, lempty;
  Desc desc[C::STAGES];
  uint32_t wlt[3][C::NCW], wgt[3][C::NCW];  // per-warp totals: count (k), scatter (k-1), free (k-2)
  uint32_t cq[C::CQ];
  uint32_t cq_head, cq_tail, term, cons_ok, slot_ok, lok;
  unsigned long long ph[5];  // consumer leader's phase cycles: partition, on-chip, fill; item start; loop start
  // output-range reservations: consumer leader -> reserver warp -> consumers
  uint32_t rq_job[C::RQ], rq_ls[C::RQ], rq_gs[C::RQ], rs_done[C::RQ];
  unsigned long long rs_lb[C::RQ], rs_gb[C::RQ];
  uint32_t rq_tail;
  // local sort: segment records and their queue
  uint32_t lr_head, lr_tail, ls_done;
  LRec lrec[C::LREC];
  // local sort, first level: pivots, bucket counts (then cursors), bucket starts, labels
  typename C::B spl[C::NB_MAX];
  alignas(16) uint32_t bcnt[C::NB_MAX];
  alignas(16) uint32_t bstart[C::NB_MAX + 4];
  // the buckets of each network class (appended in any order) and their numbers
  uint8_t cls_list[C::NCLASS][C::NB_MAX];
  uint32_t cls_cnt[8];
  uint32_t task_next;  // the next bucket task to take
  uint8_t lb[C::TILE];
};

// ---------------------------------------------------------------------------
// Error reporting and bounded waits.

__device__ __forceinline__ void set_error(Queue* q, uint32_t code, unsigned long long info) {
  if (atomicCAS(&q->error, 0u, code) == 0u) q->error_info = info;
}

#ifdef GQS_PROFILE
// Counts one finished job of `keys` keys at `depth` in the per-level rows (col 0: partition
// jobs, col 2: on-chip sorts) and notes the time. One thread per job.
__device__ __forceinline__ void level_note(Queue* q, uint32_t depth, int col, unsigned long long keys) {
  unsigned long long* r = q->lvl[depth < (uint32_t)kLevels ? depth : (uint32_t)kLevels - 1u];
  atomicAdd(&r[col], 1ull);
  atomicAdd(&r[col + 1], keys);
  const unsigned long long now = global_timer_ns();
  atomicCAS(&r[4], 0ull, now);
  atomicMax(&r[5], now);
}
#endif

// Debug builds (-DGQS_CHECK) test every job record, staged range and global write index
// against the sort's bounds; a failed test records ST_BOUNDS with the site's code in
// error_info, the access is skipped, and every role then winds down through its error path.
// Product builds compile the tests out.
#ifdef GQS_CHECK
#define GQS_OK(cond, q, code) ((cond) || (set_error((q), ST_BOUNDS, (code)), false))
#define GQS_CHECK_PARAMS , unsigned long long chk_lo, unsigned long long chk_hi, Queue* chk_q
#define GQS_CHECK_ARGS(lo, hi, q) , (lo), (hi), (q)
#else
#define GQS_OK(cond, q, code) true
#define GQS_CHECK_PARAMS
#define GQS_CHECK_ARGS(lo, hi, q)
#endif

__device__ __forceinline__ unsigned long long progress_word(Queue* q) {
  return ld_relaxed(&q->done) + ld_relaxed(&q->alloc) * 0x9E3779B97F4A7C15ull +
         ((unsigned long long)ld_relaxed(&q->grab) << 40);
}

// A wait that gives up (and records a timeout) only when the whole sort has made no
// progress for `timeout_ns`, or when another CTA has already recorded an error.
struct Waiter {
  // The shared progress counters are sampled at most every kPollNs (the SM-local global timer
  // is read in between), so waiting warps do not flood the queue's hot cache lines.
  static constexpr unsigned long long kPollNs = 20000;
  unsigned long long t0, tcheck, last;
  uint32_t spins;
  __device__ __forceinline__ explicit Waiter(Queue*) : t0(global_timer_ns()), tcheck(t0), last(~0ull), spins(0) {}
  __device__ __forceinline__ bool step(Queue* q, unsigned long long timeout_ns, uint32_t where, bool sleep) {
    ++spins;
    if ((spins & 15u) == 0u) {
      const unsigned long long now = global_timer_ns();
      if (now - tcheck >= kPollNs) {
        tcheck = now;
        if (ld_relaxed(&q->error)) return false;
        const unsigned long long p = progress_word(q);
        if (p != last) {
          last = p;
          t0 = now;
        } else if (now - t0 > timeout_ns) {
          set_error(q, ST_TIMEOUT, where);
          return false;
        }
      }
    }
    if (sleep) __nanosleep(spins < 64 ? 64 : 512);
    return true;
  }
};

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, Queue* q, unsigned long long tmo,
                                          uint32_t where) {
  if (mbar_test(bar, parity)) return true;
  Waiter w(q);
  while (!mbar_test(bar, parity)) {
    if (!w.step(q, tmo, where, false)) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Warp-level bitonic sort of NET keys held R per lane by NET / R lanes (a power of two); network
// element e = (lane % (NET / R)) * R + r, so one warp runs 32 * R / NET networks side by side, one
// per group of NET / R consecutive lanes (every shuffle stays inside its group). (Replaces the
// reference's work-group bitonic network, QuicksortKernels.cl:40-68.)
// Flip form: each merge of size k starts by comparing e with its mirror e ^ (k-1), then
// half-cleaners compare e with e ^ j; the lower index always keeps the minimum, so no
// compare-exchange needs a per-element direction. Stages with j < R compare two registers of one
// lane (no shuffle), so more keys per lane means fewer shuffles per key. N independent sets of
// networks run interleaved, which multiplies the independent work in every stage by N (the
// stages are a latency chain).
template <int R, int N, class K, int NET = 32 * R>
__device__ __forceinline__ void warp_bitonic_n(K (&v)[N * R]) {
  static_assert(NET >= R && NET <= 32 * R && (NET & (NET - 1)) == 0, "a network of 1 to 32 lanes");
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= NET; k <<= 1) {
    if (k <= R) {
#pragma unroll
      for (int n = 0; n < N; ++n)
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int pr = r ^ (k - 1);
          if (pr > r) {
            const K a = v[n * R + r], b = v[n * R + pr];
            v[n * R + r] = a < b ? a : b;
            v[n * R + pr] = a < b ? b : a;
          }
        }
    } else {
      const int lj = (k - 1) / R;
      const bool lower = (lane & (k / R / 2)) == 0;
      K t[N * R];
#pragma unroll
      for (int n = 0; n < N; ++n)
#pragma unroll
        for (int r = 0; r < R; ++r) t[n * R + r] = __shfl_xor_sync(0xffffffffu, v[n * R + R - 1 - r], lj);
#pragma unroll
      for (int n = 0; n < N; ++n)
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const K a = v[n * R + r], b = t[n * R + r];
          v[n * R + r] = ((a > b) == lower) ? b : a;
        }
    }
#pragma unroll
    for (int j = k >> 2; j > 0; j >>= 1) {
      if (j < R) {
#pragma unroll
        for (int n = 0; n < N; ++n)
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int pr = r ^ j;
            if (pr > r) {
              const K a = v[n * R + r], b = v[n * R + pr];
              v[n * R + r] = a < b ? a : b;
              v[n * R + pr] = a < b ? b : a;
            }
          }
      } else {
        const int lj = j / R;
        const bool lower = (lane & lj) == 0;
        K t[N * R];
#pragma unroll
        for (int n = 0; n < N; ++n)
#pragma unroll
          for (int r = 0; r < R; ++r) t[n * R + r] = __shfl_xor_sync(0xffffffffu, v[n * R + r], lj);
#pragma unroll
        for (int n = 0; n < N; ++n)
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const K a = v[n * R + r], b = t[n * R + r];
            v[n * R + r] = ((a > b) == lower) ? b : a;
          }
      }
    }
  }
}

template <int R, class K>
__device__ __forceinline__ void warp_bitonic(K (&v)[R]) {
  warp_bitonic_n<R, 1>(v);
}

template <class K>
__device__ __forceinline__ K kmax() {
  return ~K(0);
}

// ---------------------------------------------------------------------------
// Queue operations.

// Publishes `njobs` (1 or 2) jobs with one allocation: consecutive record slots, and each
// job's tickets after the previous job's. Called by all 32 lanes of a warp with the same
// arguments. Lane 0 writes the records, then every lane writes a share of the ticket-map
// entries. The two children of a finished partition go out together, so the completer pays
// one allocation round trip and one fence for both.
template <class C>
__device__ bool push_jobs(const SortArgs<typename C::T>& a, uint32_t njobs, const uint32_t (&kind)[2], uint32_t dir,
                          const unsigned long long (&start)[2], const unsigned long long (&end)[2],
                          const unsigned long long (&pivot)[2], uint32_t depth) {
  using B = typename C::B;
  const int lane = threadIdx.x & 31;
  long long grid[2];
  uint32_t nch[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    grid[i] = (long long)start[i];
    nch[i] = 0;
    if ((uint32_t)i >= njobs) continue;
    nch[i] = 1;
    if (kind[i] == JOB_PART) {
      const B* src = dir ? a.d : a.dn;
      grid[i] -= (long long)((reinterpret_cast<uintptr_t>(src + start[i]) & 15u) / sizeof(B));
      nch[i] = (uint32_t)(((long long)end[i] - grid[i] + C::CHUNK - 1) / C::CHUNK);
    } else if (kind[i] == JOB_FILL) {
      grid[i] -= (long long)((reinterpret_cast<uintptr_t>(a.d + start[i]) & 15u) / sizeof(B));
      nch[i] = (uint32_t)(((long long)end[i] - grid[i] + C::FILL_CHUNK - 1) / C::FILL_CHUNK);
    }
  }
  const uint32_t total = nch[0] + nch[1];
  unsigned long long old = 0;
  uint32_t ok = 1;
  if (lane == 0) {
    // `grab` is read before the allocation: an older value only overstates the untaken tickets
    const uint32_t grab = ld_relaxed(&a.q->grab);
    old = atomicAdd(&a.q->alloc, ((unsigned long long)njobs << 32) | (unsigned long long)total);
    const uint32_t slot = (uint32_t)(old >> 32), t0 = (uint32_t)old;
    // the ring must still hold every ticket not yet taken once these are added (producers
    // may hold tickets ahead of the last one created, so `grab` can exceed t0 + total)
    const long long untaken = (long long)t0 + (long long)total - (long long)grab;
    if ((unsigned long long)slot + njobs > a.capacity || untaken > (long long)a.tmask + 1) {
      set_error(a.q, ST_CAPACITY, slot);
      ok = 0;
    } else if (!GQS_OK(start[0] <= end[0] && end[0] <= a.n && (njobs < 2 || (start[1] <= end[1] && end[1] <= a.n)),
                       a.q, 0xB001ull)) {
      ok = 0;
    } else {
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        if ((uint32_t)i >= njobs) continue;
        Job* j = a.jobs + slot + i;
        j->start = start[i];
        j->end = end[i];
        j->sstart = start[i];
        j->send = end[i];
        j->pivot = pivot[i];
        j->grid = grid[i];
        j->kind = kind[i];
        j->dir = dir;
        j->nchunks = nch[i];
        j->t0 = t0 + (i ? nch[0] : 0u);
        j->remaining = nch[i];
        j->depth = depth;
      }
    }
  }
  ok = __shfl_sync(0xffffffffu, ok, 0);
  old = __shfl_sync(0xffffffffu, old, 0);
  if (!ok) return false;
  __syncwarp();
  __threadfence();  // the records (written by lane 0, ordered by the warp barrier) before their tickets
  const uint32_t slot = (uint32_t)(old >> 32), t0 = (uint32_t)old;
  for (uint32_t i = lane; i < total; i += 32) {
    const uint32_t t = t0 + i;
    st_relaxed(a.tmap + (t & a.tmask), ((unsigned long long)(t + 1) << 32) | (slot + (i < nch[0] ? 0u : 1u)));
  }
  return true;
}

// Publishes one job (see push_jobs).
template <class C>
__device__ bool push_job(const SortArgs<typename C::T>& a, uint32_t kind, uint32_t dir,
                         unsigned long long start, unsigned long long end, unsigned long long pivot,
                         uint32_t depth) {
  const uint32_t k[2] = {kind, 0u};
  const unsigned long long s[2] = {start, 0ull}, e[2] = {end, 0ull}, p[2] = {pivot, 0ull};
  return push_jobs<C>(a, 1u, k, dir, s, e, p, depth);
}

// Median of 32*RS evenly spaced samples of src[a, a+m) (global memory, L2 reads).
template <class C, int RS>
__device__ typename C::B sample_pivot_global(const typename C::B* src, unsigned long long a,
                                             unsigned long long m) {
  using B = typename C::B;
  const int lane = threadIdx.x & 31;
  B v[RS];
#pragma unroll
  for (int r = 0; r < RS; ++r) {
    const unsigned long long idx = (unsigned long long)(lane * RS + r);
    v[r] = C::Ops::key(__ldcg(src + a + (idx * m) / (32ull * RS)));
  }
  warp_bitonic<RS>(v);
  return __shfl_sync(0xffffffffu, v[0], 16);
}

// The pivots of two ranges at once (each as sample_pivot_global computes it): every lane
// issues its loads for both ranges before either network runs. `use0`/`use1` are warp-uniform.
template <class C, int RS>
__device__ void sample_pivots_global2(const typename C::B* src, unsigned long long a0, unsigned long long m0,
                                      bool use0, unsigned long long a1, unsigned long long m1, bool use1,
                                      typename C::B& p0, typename C::B& p1) {
  using B = typename C::B;
  const int lane = threadIdx.x & 31;
  B v0[RS], v1[RS];
#pragma unroll
  for (int r = 0; r < RS; ++r) {
    const unsigned long long idx = (unsigned long long)(lane * RS + r);
    v0[r] = use0 ? C::Ops::key(__ldcg(src + a0 + (idx * m0) / (32ull * RS))) : B(0);
    v1[r] = use1 ? C::Ops::key(__ldcg(src + a1 + (idx * m1) / (32ull * RS))) : B(0);
  }
  if (use0) {
    warp_bitonic<RS>(v0);
    p0 = __shfl_sync(0xffffffffu, v0[0], 16);
  }
  if (use1) {
    warp_bitonic<RS>(v1);
    p1 = __shfl_sync(0xffffffffu, v1[0], 16);
  }
}

// One warp sorts src[a, a+m) (m <= 32*R) into d[a, a+m) with a network of 32*R keys.
template <class C, int R>
__device__ __noinline__ void warp_sort_global_r(const typename C::B* src, typename C::B* d, unsigned long long a,
                                                uint32_t m) {
  using B = typename C::B;
  const int lane = threadIdx.x & 31;
  B v[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const uint32_t e = r * 32 + lane;  // input layout is free; this one coalesces
    v[r] = e < m ? C::Ops::key(__ldcg(src + a + e)) : kmax<B>();
  }
  warp_bitonic<R>(v);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const uint32_t e = lane * R + r;
    if (e < m) d[a + e] = C::Ops::raw(v[r]);
  }
}

// One warp sorts src[a, a+m) (m <= TINY) into d[a, a+m), with the smallest network that fits.
template <class C>
__device__ __forceinline__ void warp_sort_global(const typename C::B* src, typename C::B* d, unsigned long long a,
                                                 uint32_t m) {
  if (m <= 64u) warp_sort_global_r<C, 2>(src, d, a, m);
  else if (m <= 128u || C::R <= 4) warp_sort_global_r<C, (C::R < 4 ? C::R : 4)>(src, d, a, m);
  else warp_sort_global_r<C, C::R>(src, d, a, m);
}

// What becomes of a range of m keys: 0 = placed at once by place_small (at most TINY keys),
// else the kind of job it becomes.
template <class C>
__device__ __forceinline__ uint32_t range_kind(unsigned long long m) {
  return m <= (unsigned long long)C::TINY ? 0u : m <= (unsigned long long)C::TILE ? (uint32_t)JOB_LOCAL
                                                                                  : (uint32_t)JOB_PART;
}

// Places a range of at most TINY keys whose keys sit in d (dir 1) or dn (dir 0): one key is
// copied, more are sorted by the calling warp. Returns the number of keys placed.
template <class C>
__device__ unsigned long long place_small(const SortArgs<typename C::T>& a, uint32_t dir, unsigned long long s,
                                          unsigned long long m, unsigned long long& tiny_keys) {
  const int lane = threadIdx.x & 31;
  const typename C::B* src = dir ? a.d : a.dn;
  if (m == 0) return 0;
  if (!GQS_OK(s + m <= a.n, a.q, 0xB002ull)) return 0;
  if (m == 1) {
    if (!dir && lane == 0) a.d[s] = __ldcg(src + s);
    return 1;
  }
  warp_sort_global<C>(src, a.d, s, (uint32_t)m);
  tiny_keys += m;
  return m;
}

// Decide what to do with a range whose keys sit in d (dir 1) or dn (dir 0).
// Called by a whole warp. Returns the number of keys placed in their final position.
template <class C>
__device__ unsigned long long dispatch_range(const SortArgs<typename C::T>& a, uint32_t dir,
                                             unsigned long long s, unsigned long long e, uint32_t depth,
                                             unsigned long long& tiny_keys) {
  using B = typename C::B;
  const unsigned long long m = e - s;
  const uint32_t kind = range_kind<C>(m);
  if (!kind) return place_small<C>(a, dir, s, m, tiny_keys);
  if (kind == JOB_LOCAL) {
    push_job<C>(a, JOB_LOCAL, dir, s, e, 0, depth);
    return 0;
  }
  const B pv = sample_pivot_global<C, 4>(dir ? a.d : a.dn, s, m);
  push_job<C>(a, JOB_PART, dir, s, e, (unsigned long long)pv, depth);
  return 0;
}

// ---------------------------------------------------------------------------
// Seed kernel: one warp per segment turns the segment table into root jobs.

// Segment i is [offsets[i], offsets[i+1]) or, with `pairs`, [offsets[2i], offsets[2i+1]) (the
// segments then need not be adjacent); without offsets, the one segment [0, n). Every segment
// must lie in [0, n). The keys are in d, or with `from_dn` in dn (the buckets of a top split);
// either way the sorted keys end in d.
template <class C>
__global__ void __launch_bounds__(256) seed_kernel(SortArgs<typename C::T> a, const unsigned long long* offsets,
                                                   const unsigned long long* nseg_dev, uint32_t nseg,
                                                   unsigned long long n, uint32_t pairs, uint32_t from_dn) {
  const uint32_t seg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  pdl_wait();     // the segment table and the zeroed queue are written by the work before it
  pdl_trigger();  // the persistent kernel may launch; it waits for this grid before starting
  if (nseg_dev) {  // a replayable launch: the count is data, at most the launch's capacity
    const unsigned long long m = *nseg_dev;
    if (m > nseg) {
      if (seg == 0 && lane == 0) set_error(a.q, ST_INVALID, m);
      return;
    }
    nseg = (uint32_t)m;
  }
  if (seg >= nseg) return;
  const unsigned long long s = offsets ? offsets[pairs ? 2ull * seg : seg] : 0ull;
  const unsigned long long e = offsets ? offsets[pairs ? 2ull * seg + 1 : seg + 1] : n;
  if (s > e || e > n) {  // malformed segment table
    if (lane == 0) set_error(a.q, ST_INVALID, seg);
    return;
  }
  if (e == s) return;
  if (lane == 0) atomicAdd(&a.q->total, e - s);
  unsigned long long tiny = 0;
  // the buckets of a top split are its children: depth 1
  const unsigned long long placed = dispatch_range<C>(a, from_dn ? 0u : 1u, s, e, from_dn ? 1u : 0u, tiny);
  if (lane == 0) {
    if (placed) atomicAdd(&a.q->done, placed);
    if (tiny) atomicAdd(&a.q->tiny_keys, tiny);
  }
}

// ---------------------------------------------------------------------------
// Persistent sort kernel.

template <class C>
struct Persistent {
  using T = typename C::T;
  using B = typename C::B;
  using Ops = typename C::Ops;

  static __device__ __forceinline__ void cbar() { named_bar_sync(1, C::NC); }

  // ---- producer ---------------------------------------------------------
  // Work is taken by ticket: one atomic on the queue's grab counter reserves kTake consecutive
  // tickets, and lanes 0..kTake-1 resolve them through the ticket map in parallel. Each ticket
  // is one chunk of one job, so no two producers ever contend for the same chunk.
  static constexpr uint32_t kTake = 4;

  struct Ticket {
    unsigned long long js, je, pivot;
    long long grid;
    uint32_t slot, kind, dir, chunk;
  };

  // Resolves this lane's ticket if it is published; returns whether it is.
  static __device__ __forceinline__ bool resolve(const SortArgs<T>& a, uint32_t t, Ticket& tk) {
    const unsigned long long e = ld_acquire(a.tmap + (t & a.tmask));
    if ((uint32_t)(e >> 32) != t + 1u) return false;
    const uint32_t slot = (uint32_t)e;
    if (!GQS_OK(slot < a.capacity, a.q, 0xB003ull)) return false;
    const Job* j = a.jobs + slot;
    tk.slot = slot;
    tk.kind = __ldcg(&j->kind);
    tk.dir = __ldcg(&j->dir);
    tk.js = __ldcg(&j->start);
    tk.je = __ldcg(&j->end);
    tk.pivot = __ldcg(&j->pivot);
    tk.grid = __ldcg(&j->grid);
    tk.chunk = t - __ldcg(&j->t0);
    if (!GQS_OK(tk.kind >= JOB_PART && tk.kind <= JOB_FILL && tk.js <= tk.je && tk.je <= a.n, a.q, 0xB004ull))
      return false;
    return true;
  }

  // Stage src[cs, ce) into shared memory at `dst`, rounded out to whole 16-byte granules of
  // global memory (a granule never straddles a page, so the rounding cannot fault; the extra
  // bytes are never read). Returns the element offset of src[cs] inside `dst`.
  // The keys were written with plain stores by other warps and CTAs, made visible to this
  // thread by the acquire of the job's ticket; the global proxy fence extends that to the bulk
  // copy, which reads through the async proxy.
  static __device__ __forceinline__ uint32_t stage_range(const B* src, unsigned long long cs,
                                                         unsigned long long ce, B* dst, uint64_t* bar) {
    const uintptr_t lo = reinterpret_cast<uintptr_t>(src + cs);
    const uintptr_t ga = lo & ~uintptr_t(15);
    const uintptr_t gb = (reinterpret_cast<uintptr_t>(src + ce) + 15) & ~uintptr_t(15);
    const uint32_t bytes = (uint32_t)(gb - ga);
    fence_proxy_async_global();
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, bytes);
    bulk_load(dst, reinterpret_cast<const void*>(ga), bytes, bar);
    return (uint32_t)((lo - ga) / sizeof(B));
  }

  static __device__ void producer(const SortArgs<T>& a, Smem<C>& sm) {
    const int lane = threadIdx.x & 31;
    GQS_PROF_DECL
    uint32_t k = 0, nloc = 0, nops = 0;
    bool need_flush = false;  // partition chunks were handed out since the last drain
    uint32_t failed = 0;
    Waiter idle(a.q);
    bool idling = false;
    // Tickets per grab: this CTA's share of the tickets waiting at the last grab, from one to
    // kTake, so that a new job's chunks spread over all CTAs instead of queueing kTake deep on
    // a few, while a deep queue is still taken kTake at a time (one atomic, and the tickets
    // resolved in parallel lanes). At the
    // frontier (the last grab ran past every ticket allocated so far) the producer takes its
    // next ticket only once this CTA is idle, so that new work goes to CTAs that can start it
    // at once rather than behind a local sort.
    uint32_t tb = 0, take = 1, take_next = 1, next = 1, resolved = 0;
    bool frontier = false;
    Ticket mine;
    mine.slot = 0;
    for (;;) {
      GQS_PROF_T(t0)
      uint32_t kind = ITEM_NONE;
      if (next == take) {
        // need_flush is lane 0's; the branch below must be taken by the whole warp
        if (frontier && __shfl_sync(0xffffffffu, need_flush ? 1u : 0u, 0) != 0u) {
          kind = ITEM_FLUSH;  // hand the consumers their last chunk before waiting for idle
        } else {  // take the next batch of tickets
          uint32_t b = 0, ok = 1, fr = 0, nt = take_next;
          if (lane == 0) {
            if (frontier) {
              // the most recent item released by the consumers, and the tile region free
              if (k && !mbar_wait(&sm.empty[(k - 1) % C::STAGES], ((k - 1) / C::STAGES) & 1u, a.q, a.timeout_ns, 2))
                ok = 0;
              if (ok && nloc && !mbar_wait(&sm.lempty, (nloc - 1) & 1u, a.q, a.timeout_ns, 3)) ok = 0;
            }
            if (ok) {
              b = atomicAdd(&a.q->grab, take_next);
              const uint32_t alloc_tickets = (uint32_t)ld_relaxed(&a.q->alloc);
              const int avail = (int)(alloc_tickets - (b + take_next));
              fr = avail < 0 ? 1u : 0u;
              const int share = avail / (int)gridDim.x;  // this CTA's share of the waiting tickets
              nt = share >= (int)kTake ? kTake : share > 1 ? (uint32_t)share : 1u;
            }
          }
          if (!__shfl_sync(0xffffffffu, ok, 0)) {
            failed = 1;
            break;
          }
          tb = __shfl_sync(0xffffffffu, b, 0);
          take = take_next;
          take_next = __shfl_sync(0xffffffffu, nt, 0);
          frontier = __shfl_sync(0xffffffffu, fr, 0) != 0u;
          next = 0;
          resolved = 0;
          ++nops;
        }
      }
      if (kind == ITEM_NONE) {
        if (!((resolved >> next) & 1u)) {
          bool ok = false;
          if (lane < (int)take && !((resolved >> lane) & 1u)) ok = resolve(a, tb + lane, mine);
          resolved |= __ballot_sync(0xffffffffu, ok);
        }
        GQS_PROF_ADD(PF_P_GRAB, t0)
        if ((resolved >> next) & 1u) {
          kind = __shfl_sync(0xffffffffu, mine.kind, next);  // job kinds double as item kinds
          idling = false;
        } else {
          // The next ticket is not published yet: more work is coming, or the sort is over.
          if (lane == 0) {
            GQS_PROF_T(t1)
            if (ld_relaxed(&a.q->error) || ld_relaxed(&a.q->done) >= ld_relaxed(&a.q->total)) {
              kind = ITEM_TERM;
            } else if (need_flush) {
              kind = ITEM_FLUSH;  // let the consumers finish what they hold before idling
            } else {
              if (!idling) {
                idle = Waiter(a.q);
                idling = true;
              }
              if (!idle.step(a.q, a.timeout_ns, 1, true)) kind = ITEM_TERM;
            }
            GQS_PROF_ADD(PF_P_IDLE, t1)
          }
          kind = __shfl_sync(0xffffffffu, kind, 0);
          if (kind == ITEM_NONE) continue;
        }
      }
      const bool real = kind == ITEM_PART || kind == ITEM_LOCAL || kind == ITEM_FILL;
      const uint32_t src_lane = real ? next : 0u;
      const uint32_t slot = __shfl_sync(0xffffffffu, mine.slot, src_lane);
      const uint32_t dir = __shfl_sync(0xffffffffu, mine.dir, src_lane);
      const uint32_t chunk = __shfl_sync(0xffffffffu, mine.chunk, src_lane);
      const unsigned long long js = __shfl_sync(0xffffffffu, mine.js, src_lane);
      const unsigned long long je = __shfl_sync(0xffffffffu, mine.je, src_lane);
      const unsigned long long pivot = __shfl_sync(0xffffffffu, mine.pivot, src_lane);
      const long long grid = __shfl_sync(0xffffffffu, mine.grid, src_lane);
      const uint32_t s = k % C::STAGES;
      if (lane == 0) {
        GQS_PROF_T(t2)
        const bool got = mbar_wait(&sm.empty[s], ((k / C::STAGES) & 1u) ^ 1u, a.q, a.timeout_ns, 2);
        GQS_PROF_ADD(PF_P_EMPTY, t2)
        GQS_PROF_T(t3)
        if (!got) {
          failed = 1;
        } else if (!real) {
          sm.desc[s].kind = kind;
          mbar_arrive(&sm.full[s]);
          need_flush = false;
        } else {
          Desc& dd = sm.desc[s];
          dd.kind = kind;
          dd.job = slot;
          dd.dir = dir;
          dd.pivot = pivot;
          const B* src = dir ? a.d : a.dn;
          if (kind == ITEM_PART || kind == ITEM_FILL) {
            const long long grain = kind == ITEM_PART ? C::CHUNK : C::FILL_CHUNK;
            const long long g0 = grid + (long long)chunk * grain;
            const unsigned long long cs = (long long)js > g0 ? js : (unsigned long long)g0;
            const unsigned long long ce0 = (unsigned long long)(g0 + grain);
            const unsigned long long ce = ce0 < je ? ce0 : je;
            dd.gbeg = cs;
            dd.len = (uint32_t)(ce - cs);
#ifdef GQS_CHECK
            dd.jlo = js;
            dd.jhi = je;
#endif
            if (!GQS_OK(cs < ce && ce - cs <= (unsigned long long)grain, a.q, 0xB005ull)) {
              failed = 1;  // nothing staged; the whole warp leaves the loop below
            } else if (kind == ITEM_PART) {
              dd.off = stage_range(src, cs, ce, sm.stage[s], &sm.full[s]);
              need_flush = true;
            } else {
              dd.off = 0;
              mbar_arrive(&sm.full[s]);
              need_flush = false;
            }
          } else {  // ITEM_LOCAL: the tile region is single-buffered
            GQS_PROF_T(t4)
            const bool free_tile = mbar_wait(&sm.lempty, (nloc & 1u) ^ 1u, a.q, a.timeout_ns, 3);
            GQS_PROF_ADD(PF_P_LEMPTY, t4)
            if (!free_tile || !GQS_OK(je - js <= (unsigned long long)C::TILE, a.q, 0xB006ull)) {
              failed = 1;
            } else {
              dd.gbeg = js;
              dd.len = (uint32_t)(je - js);
              dd.off = stage_range(src, js, je, sm.tileA, &sm.lfull);
              mbar_arrive(&sm.full[s]);
              ++nloc;
              need_flush = false;
            }
          }
        }
        GQS_PROF_ADD(PF_P_ISSUE, t3)
      }
      failed = __shfl_sync(0xffffffffu, failed, 0);
      if (failed) break;
      ++k;
      if (real) ++next;
      if (kind == ITEM_TERM) break;
    }
    if (failed && lane == 0) {
      // Leave no bulk copy in flight into this CTA's shared memory: each stage's most recent
      // load completes on its full barrier, the most recent tile load on lfull.
      for (uint32_t i = 0; i < (uint32_t)C::STAGES && i < k; ++i) {
        const uint32_t kk = k - 1 - i;
        mbar_wait(&sm.full[kk % C::STAGES], (kk / C::STAGES) & 1u, a.q, 200000000ull, 9);
      }
      if (nloc) mbar_wait(&sm.lfull, (nloc - 1) & 1u, a.q, 200000000ull, 9);
      sts_release(&sm.term, 2u);
    }
    if (lane == 0) {
      GQS_PROF_CNT(PF_N_GRAB, nops)
      GQS_PROF_FLUSH(a.q)
    }
  }

  // ---- completer --------------------------------------------------------
  static __device__ void complete_job(const SortArgs<T>& a, uint32_t slot, unsigned long long& st_tiny,
                                      unsigned long long& st_fill, uint32_t& st_depth) {
    const int lane = threadIdx.x & 31;
    const Job* j = a.jobs + slot;
    const unsigned long long js = __ldcg(&j->start), je = __ldcg(&j->end);
    const unsigned long long ss = __ldcg(&j->sstart), se = __ldcg(&j->send);
    const B pv = (B)__ldcg(&j->pivot);
    const uint32_t dir = __ldcg(&j->dir), depth = __ldcg(&j->depth);
    if (!GQS_OK(js <= ss && ss <= se && se <= je && je <= a.n, a.q, 0xB00Aull)) return;
#ifdef GQS_PROFILE
    if (lane == 0) level_note(a.q, depth, 0, je - js);
#endif
    unsigned long long placed = 0;
    // Pivot run [ss, se) -> d (the reference's last block writes it serially,
    // QuicksortKernels.cl:214-216; here a warp writes short runs and long runs become
    // fill jobs that every CTA shares).
    const unsigned long long plen = se - ss;
    if (plen) {
      if (plen <= (unsigned long long)C::FILL_INLINE) {
        const B raw = Ops::raw(pv);
        for (unsigned long long i = ss + lane; i < se; i += 32) a.d[i] = raw;
        placed += plen;
        st_fill += plen;
      } else {
        push_job<C>(a, JOB_FILL, 0u, ss, se, (unsigned long long)pv, depth);
      }
    }
    // Children [js, ss) and [se, je) live in this job's destination buffer; they are read the
    // other way next. Both pivots are sampled together and both jobs published with one
    // allocation; children of at most TINY keys are sorted here, after the publication.
    const uint32_t cdir = dir ^ 1u;
    const uint32_t k0 = range_kind<C>(ss - js), k1 = range_kind<C>(je - se);
    B p0 = 0, p1 = 0;
    sample_pivots_global2<C, 4>(cdir ? a.d : a.dn, js, ss - js, k0 == JOB_PART, se, je - se, k1 == JOB_PART, p0,
                                p1);
    const uint32_t nj = (k0 ? 1u : 0u) + (k1 ? 1u : 0u);
    if (nj) {
      const uint32_t kinds[2] = {k0 ? k0 : k1, k1};
      const unsigned long long cs[2] = {k0 ? js : se, se}, ce[2] = {k0 ? ss : je, je};
      const unsigned long long cp[2] = {(unsigned long long)(k0 ? p0 : p1), (unsigned long long)p1};
      push_jobs<C>(a, nj, kinds, cdir, cs, ce, cp, depth + 1);
    }
    if (!k0) placed += place_small<C>(a, cdir, js, ss - js, st_tiny);
    if (!k1) placed += place_small<C>(a, cdir, se, je - se, st_tiny);
    if (lane == 0 && placed) atomicAdd(&a.q->done, placed);
    if (depth + 1 > st_depth) st_depth = depth + 1;
  }

  // The completer takes up to 32 posted chunks at once; each lane retires one with an
  // acquire-release decrement of its job's chunk count, and the warp finishes every job
  // whose count reached zero.
  static __device__ void completer(const SortArgs<T>& a, Smem<C>& sm) {
    const int lane = threadIdx.x & 31;
    GQS_PROF_DECL
    unsigned long long st_tiny = 0, st_fill = 0;
    uint32_t st_depth = 0, st_jobs = 0;
    uint32_t head = 0;
    Waiter w(a.q);
    bool idling = false;
    for (;;) {
      uint32_t navail = 0, state = 0;  // state: 0 none, 1 items, 2 exit
      GQS_PROF_T(tq)
      if (lane == 0) {
        const uint32_t t = lds_acquire(&sm.cq_tail);
        if (t != head) {
          navail = min(t - head, 32u);
          state = 1;
          idling = false;
        } else if (lds_acquire(&sm.term)) {
          state = 2;
        } else {
          if (!idling) {
            w = Waiter(a.q);
            idling = true;
          }
          if (!w.step(a.q, a.timeout_ns, 4, true)) state = 2;  // the sort failed; nothing left to finish
        }
      }
      state = __shfl_sync(0xffffffffu, state, 0);
      if (state == 2) break;
      if (state == 0) {
        GQS_PROF_ADD(PF_Q_IDLE, tq)
        continue;
      }
      GQS_PROF_T(tb)
      navail = __shfl_sync(0xffffffffu, navail, 0);
      __syncwarp();
      uint32_t slot = 0, old = 0;
      if ((uint32_t)lane < navail) {
        slot = sm.cq[(head + lane) % C::CQ];
        old = atom_add_acq_rel(&a.jobs[slot].remaining, 0xffffffffu);
      }
      head += navail;
      __syncwarp();
      if (lane == 0) sts_release(&sm.cq_head, head);
      uint32_t last = __ballot_sync(0xffffffffu, (uint32_t)lane < navail && old == 1u);
      while (last) {
        const int l = __ffs(last) - 1;
        last &= last - 1;
        const uint32_t js = __shfl_sync(0xffffffffu, slot, l);
        __threadfence();
        complete_job(a, js, st_tiny, st_fill, st_depth);
        ++st_jobs;
      }
      GQS_PROF_ADD(PF_Q_BUSY, tb)
    }
    if (lane == 0) {
      GQS_PROF_FLUSH(a.q)
      if (st_tiny) atomicAdd(&a.q->tiny_keys, st_tiny);
      if (st_fill) atomicAdd(&a.q->fill_keys, st_fill);
      if (st_jobs) atomicAdd(&a.q->part_jobs, st_jobs);
      atomicMax(&a.q->max_depth, st_depth);
    }
  }

  // ---- reserver ---------------------------------------------------------
  // Reserves each counted chunk's output ranges in its job (the reference's two atomics on
  // parent.sstart / parent.send, QuicksortKernels.cl:183-186). Lane l of the warp serves
  // request next + l, so up to 32 reservations are in flight and no consumer thread ever
  // waits on a global atomic.
  static __device__ void reserver(const SortArgs<T>& a, Smem<C>& sm) {
    const int lane = threadIdx.x & 31;
    uint32_t next = 0;
    Waiter w(a.q);
    bool idling = false;
    for (;;) {
      uint32_t n = 0, state = 0;
      if (lane == 0) {
        const uint32_t t = lds_acquire(&sm.rq_tail);
        if (t != next) {
          n = min(t - next, 32u);
          state = 1;
          idling = false;
        } else if (lds_acquire(&sm.term)) {
          state = 2;
        } else {
          if (!idling) {
            w = Waiter(a.q);
            idling = true;
          }
          if (!w.step(a.q, a.timeout_ns, 8, true)) state = 2;
        }
      }
      state = __shfl_sync(0xffffffffu, state, 0);
      if (state == 2) break;
      if (state == 0) continue;
      n = __shfl_sync(0xffffffffu, n, 0);
      __syncwarp();
      if ((uint32_t)lane < n) {
        const uint32_t i = next + lane, e = i % C::RQ;
        Job* j = a.jobs + sm.rq_job[e];
        const uint32_t ls = sm.rq_ls[e], gs = sm.rq_gs[e];
        const unsigned long long lb = atomicAdd(&j->sstart, (unsigned long long)ls);
        const unsigned long long gb = atomicAdd(&j->send, (unsigned long long)(-(long long)gs)) - gs;
        sm.rs_lb[e] = lb;
        sm.rs_gb[e] = gb;
        sts_release(&sm.rs_done[e], i + 1);
      }
      next += n;
    }
  }

  // Consumer leader: waits (bounded) for reservation `id`; false if the sort has failed.
  static __device__ __forceinline__ bool leader_wait_reservation(const SortArgs<T>& a, Smem<C>& sm, uint32_t id) {
    const uint32_t e = id % C::RQ;
    if (lds_acquire(&sm.rs_done[e]) == id + 1) return true;
    Waiter w(a.q);
    while (lds_acquire(&sm.rs_done[e]) != id + 1) {
      if (!w.step(a.q, a.timeout_ns, 10, false)) return false;
    }
    return true;
  }

  // ---- consumers: partition chunks --------------------------------------
  // Post a finished chunk of job `slot` to this CTA's completer.
  static __device__ void post_chunk(const SortArgs<T>& a, Smem<C>& sm, uint32_t slot) {
    const uint32_t t = sm.cq_tail;
    if (t - lds_acquire(&sm.cq_head) >= (uint32_t)C::CQ) {
      Waiter w(a.q);
      while (t - lds_acquire(&sm.cq_head) >= (uint32_t)C::CQ) {
        if (!w.step(a.q, a.timeout_ns, 5, false)) return;
      }
    }
    sm.cq[t % C::CQ] = slot;
    sts_release(&sm.cq_tail, t + 1);
  }

  // Scatter one counted chunk whose keys are in registers: keys below the pivot go to
  // [lb + warp prefix, ...), keys above to [gb + warp prefix, ...). Keys equal to the pivot
  // (and the pivot-valued padding of a partial chunk) are dropped; the completer writes the
  // pivot run. (gqsort_kernel pass 2, QuicksortKernels.cl:190-203.)
  static __device__ __forceinline__ void scatter_chunk(const B (&keys)[C::KPT], B p, B* dst, unsigned long long lb,
                                                       unsigned long long gb, const uint32_t* wlt,
                                                       const uint32_t* wgt GQS_CHECK_PARAMS) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t vl = lane < C::NCW ? wlt[lane] : 0u, vg = lane < C::NCW ? wgt[lane] : 0u;
    uint32_t il = vl, ig = vg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t tl = __shfl_up_sync(0xffffffffu, il, o), tg = __shfl_up_sync(0xffffffffu, ig, o);
      if (lane >= o) {
        il += tl;
        ig += tg;
      }
    }
    B* const lbase = dst + lb + __shfl_sync(0xffffffffu, il - vl, warp);
    B* const gbase = dst + gb + __shfl_sync(0xffffffffu, ig - vg, warp);
    const uint32_t ltm = lanemask_lt();
    uint32_t lo = 0, go = 0;
#pragma unroll
    for (int j = 0; j < C::KPT; ++j) {
      const B kk = Ops::key(keys[j]);
      const bool isl = kk < p, isg = kk > p;
      const uint32_t bl = __ballot_sync(0xffffffffu, isl), bg = __ballot_sync(0xffffffffu, isg);
      const uint32_t r = __popc((isl ? bl : bg) & ltm);  // rank among the lanes of its side
#ifdef GQS_CHECK
      B* const to = (isl ? lbase + lo : gbase + go) + r;
      const unsigned long long ix = (unsigned long long)(to - dst);
      const bool inside = !(isl || isg) || GQS_OK(ix >= chk_lo && ix < chk_hi, chk_q, 0xB007ull);
      if ((isl || isg) && inside) *to = keys[j];
#else
      // (this exact form: computing the address outside the branch measured 6 % slower)
      if (isl || isg) (isl ? lbase + lo : gbase + go)[r] = keys[j];
#endif
      lo += __popc(bl);
      go += __popc(bg);
    }
  }

  // ---- consumers: local (on-chip) sort -----------------------------------
  // lqsort_kernel (QuicksortKernels.cl:267-421) re-done for one CTA. Like the global
  // partition, every segment of the tile is cut into slices that any consumer warp may take:
  // the warp counts its slice in registers, reserves output positions at both ends of the
  // segment with two shared-memory atomics, and scatters into the other buffer. The warp that
  // scatters a segment's last slice writes its pivot run and publishes the children; children
  // of at most TINY keys are sorted in registers by that warp at once. No CTA barrier is
  // needed between levels, so all warps stay busy from the first segment on.
  // Keys are comparison keys in A (buffer 0) and B (buffer 1); every final key lands in A.
  static __device__ __forceinline__ B* bufp(Smem<C>& sm, B* A, uint32_t buf) { return buf ? sm.tileB : A; }

  // One warp sorts X[s, s+n) (n <= 32*R) into A[s, s+n) with a network of 32*R keys.
  template <int R>
  static __device__ __noinline__ void warp_sort_smem_r(const B* X, B* A, uint32_t s, uint32_t n) {
    const int lane = threadIdx.x & 31;
    B v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint32_t e = r * 32 + lane;  // any input layout is valid; this one is bank-conflict free
      v[r] = e < n ? X[s + e] : kmax<B>();
    }
    __syncwarp();
    warp_bitonic<R>(v);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint32_t e = lane * R + r;
      if (e < n) A[s + e] = v[r];
    }
    __syncwarp();
  }

  // One warp sorts X[s, s+n) (n <= TINY) into A[s, s+n), with the smallest network that fits.
  static __device__ __forceinline__ void warp_sort_smem(const B* X, B* A, uint32_t s, uint32_t n) {
    if (n <= 32u) warp_sort_smem_r<1>(X, A, s, n);
    else if (n <= 64u) warp_sort_smem_r<2>(X, A, s, n);
    else if (n <= 128u || C::R <= 4) warp_sort_smem_r<(C::R < 4 ? C::R : 4)>(X, A, s, n);
    else warp_sort_smem_r<C::R>(X, A, s, n);
  }

  // Median of 32 evenly spaced samples of X[s, s+n), computed by one warp.
  static __device__ __forceinline__ B sample32_smem(const B* X, uint32_t s, uint32_t n) {
    const int lane = threadIdx.x & 31;
    B v[1];
    v[0] = X[s + (uint32_t)(((unsigned long long)lane * n) >> 5)];
    warp_bitonic<1>(v);
    return __shfl_sync(0xffffffffu, v[0], 16);
  }

  // Publishes segment [s, e) of buffer `buf` (longer than TINY) for slicing. Whole warp.
  static __device__ void lrec_push(const SortArgs<T>& a, Smem<C>& sm, B* A, uint32_t s, uint32_t e,
                                   uint32_t buf) {
    const int lane = threadIdx.x & 31;
    const B p = sample32_smem(bufp(sm, A, buf), s, e - s);
    if (lane == 0) {
      const uint32_t idx = atomicAdd(&sm.lr_tail, 1u);
      if (idx >= (uint32_t)C::LREC) {
        set_error(a.q, ST_INTERNAL, 0x1EC0ull);
      } else {
        LRec& r = sm.lrec[idx];
        r.pivot = (unsigned long long)p;
        r.s = s;
        r.e = e;
        r.buf = buf;
        r.nsl = (e - s + C::SLICE - 1) / C::SLICE;
        r.cursor = 0;
        r.remaining = r.nsl;
        r.lt = 0;
        r.gt = 0;
        __threadfence_block();
        *(volatile uint32_t*)&r.seq = idx + 1u;
      }
    }
    __syncwarp();
  }

  // Places one child of a finished segment: singletons go to A, small children are sorted in
  // registers now, larger ones become records. Returns the keys it finalised. Whole warp.
  static __device__ uint32_t place_child(const SortArgs<T>& a, Smem<C>& sm, B* A, uint32_t s, uint32_t e,
                                         uint32_t buf, unsigned long long* lp) {
    const int lane = threadIdx.x & 31;
    const uint32_t n = e - s;
    if (n <= 1) {
      if (n == 1 && buf && lane == 0) A[s] = sm.tileB[s];
      return n;
    }
    if (n <= (uint32_t)C::TINY) {
#ifdef GQS_PROFILE
      const long long tb0 = clock64();
#endif
      warp_sort_smem(bufp(sm, A, buf), A, s, n);
#ifdef GQS_PROFILE
      if (lane == 0) lp[7] += (unsigned long long)(clock64() - tb0);
#endif
      return n;
    }
    lrec_push(a, sm, A, s, e, buf);
    return 0;
  }

  // Partitions slice `c` of record `ri` (whole warp); the warp scattering the last slice
  // finishes the segment.
  static __device__ void run_slice(const SortArgs<T>& a, Smem<C>& sm, B* A, uint32_t ri, uint32_t c,
                                   unsigned long long* lp) {
    const int lane = threadIdx.x & 31;
    const uint32_t ltm = lanemask_lt();
    LRec& r = sm.lrec[ri];
    const uint32_t rs = r.s, re = r.e, buf = r.buf;
    const B p = (B)r.pivot;
    const B* X = bufp(sm, A, buf);
    B* Y = bufp(sm, A, buf ^ 1u);
    const uint32_t s0 = rs + c * (uint32_t)C::SLICE;
    B k[C::SLICE_KPL];
    if (s0 + (uint32_t)C::SLICE <= re) {
#pragma unroll
      for (int j = 0; j < C::SLICE_KPL; ++j) k[j] = X[s0 + (uint32_t)(j * 32 + lane)];
    } else {  // the segment's last, partial slice: the pivot value pads it and is dropped
#pragma unroll
      for (int j = 0; j < C::SLICE_KPL; ++j) {
        const uint32_t i = s0 + (uint32_t)(j * 32 + lane);
        k[j] = i < re ? X[i] : p;
      }
    }
    uint32_t cl = 0, cg = 0;
#pragma unroll
    for (int j = 0; j < C::SLICE_KPL; ++j) {
      cl += k[j] < p;
      cg += k[j] > p;
    }
    const uint32_t wl = __reduce_add_sync(0xffffffffu, cl), wg = __reduce_add_sync(0xffffffffu, cg);
    uint32_t ol = 0, og = 0;
    if (lane == 0) {
      ol = atomicAdd(&r.lt, wl);
      og = atomicAdd(&r.gt, wg);
    }
    ol = __shfl_sync(0xffffffffu, ol, 0);
    og = __shfl_sync(0xffffffffu, og, 0);
    uint32_t lpos = rs + ol, gpos = re - 1u - og;
#pragma unroll
    for (int j = 0; j < C::SLICE_KPL; ++j) {
      const bool isl = k[j] < p, isg = k[j] > p;
      const uint32_t bl = __ballot_sync(0xffffffffu, isl), bg = __ballot_sync(0xffffffffu, isg);
      if (isl || isg) Y[isl ? lpos + __popc(bl & ltm) : gpos - __popc(bg & ltm)] = k[j];
      lpos += __popc(bl);
      gpos -= __popc(bg);
    }
    __syncwarp();
    uint32_t last = 0;
    if (lane == 0) {
      __threadfence_block();
      last = atomicSub(&r.remaining, 1u) == 1u;
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return;
    __threadfence_block();
    // every slice is scattered: [rs, rs+L) < p <= ... < [re-G, re) in Y, pivot run to A
    const uint32_t L = *(volatile uint32_t*)&r.lt, G = *(volatile uint32_t*)&r.gt;
    for (uint32_t i = rs + L + lane; i < re - G; i += 32) A[i] = p;
    __syncwarp();
    uint32_t fin = (re - G) - (rs + L);
    fin += place_child(a, sm, A, rs, rs + L, buf ^ 1u, lp);
    fin += place_child(a, sm, A, re - G, re, buf ^ 1u, lp);
    if (lane == 0) atomicAdd(&sm.ls_done, fin);
#ifdef GQS_PROFILE
    if (lane == 0) lp[6] += 1;
#endif
  }

  // Sorts `cnt` buckets of class log2(G) at once: bucket cls_list[log2 G][first + g] (keys
  // tileB[bstart[b], bstart[b+1]), at most G * R of them) is sorted by lanes [g * G, g * G + G)
  // into A at the same place, with a network of G * R keys padded with the key maximum. Whole
  // warp; returns the keys placed.
  template <int G>
  static __device__ __noinline__ uint32_t bucket_networks(Smem<C>& sm, B* A, const uint8_t* list, uint32_t cnt) {
    constexpr int R = C::R;
    const uint32_t lane = threadIdx.x & 31, g = lane / G, gl = lane % G;
    uint32_t bs = 0, n = 0;
    if (g < cnt) {
      const uint32_t b = list[g];
      bs = sm.bstart[b];
      n = sm.bstart[b + 1] - bs;
    }
    B v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint32_t e = (uint32_t)r * G + gl;  // any input layout is valid; this one spreads the banks
      v[r] = e < n ? sm.tileB[bs + e] : kmax<B>();
    }
    warp_bitonic_n<R, 1, B, G * R>(v);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint32_t e = gl * R + (uint32_t)r;
      if (e < n) A[bs + e] = v[r];
    }
    return __reduce_add_sync(0xffffffffu, gl == 0 ? n : 0u);
  }

  // First level of the on-chip sort for tiles of SPLIT_MIN keys or more: one multi-pivot
  // partition of the whole tile into nb buckets (nb a power of two, buckets of about BUCKET keys),
  // then every bucket sorted in registers. Whole CTA; returns the keys this warp finalised.
  //  1. Pivots. SPLIT_SAMPLES evenly spaced keys, each ranked by one thread that compares it with
  //     all of them; the sample of rank (q + 1) * (SPLIT_SAMPLES / nb) - 1 becomes pivot q. The
  //     pivots are stored as an implicit search tree in breadth-first order (node i has children
  //     2i and 2i + 1), so the lanes of a warp reading one level hit distinct banks.
  //  2. Every consumer thread labels its keys with their bucket (bucket b holds
  //     pivot[b-1] < key <= pivot[b]) and counts them.
  //  3. Warp 0 scans the counts (16-byte loads and stores): bucket starts, and scatter cursors.
  //  4. Every key is scattered into tileB at its bucket's place; meanwhile each bucket is entered
  //     in the list of its class: class c <= 5 is sorted by a group of 2^c lanes holding R keys
  //     each (2^c * R keys at most), class 6 holds the buckets longer than TINY.
  //  5. Tasks, largest class first, each taken by the next free warp: a class-6 bucket becomes a
  //     slice-partitioned segment; a class-c task sorts 32 >> c buckets of that class at once.
  // The buckets are disjoint ranges in final order. (Inlined: as a called function its register
  // demand made the kernel keep partition-loop values in local memory.)
  static __device__ __forceinline__ uint32_t sample_split(const SortArgs<T>& a, Smem<C>& sm, B* A, uint32_t m,
                                                       unsigned long long* lp) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t nb = 2, lg = 1;
    while (nb < (uint32_t)C::NB_MAX && nb * (uint32_t)C::BUCKET < m) {
      nb <<= 1;
      ++lg;
    }
    for (uint32_t i = tid; i < (uint32_t)C::NB_MAX; i += C::NC) sm.bcnt[i] = 0u;
    if (tid < 8) sm.cls_cnt[tid] = 0u;
    if (tid == 0) sm.task_next = 0u;
    // Pivots by rank: SPLIT_SAMPLES evenly spaced keys, each ranked by one thread against all of
    // them (16-byte broadcast reads; equal keys ordered by index, so the ranks are a permutation).
    // Pivot q is the sample of rank (q + 1) * step - 1; with q1 = q + 1 = (2p + 1) << (lg - l - 1)
    // it is tree node 2^l + p.
    B* smp = sm.tileB;  // free until the scatter
    if (tid < C::SPLIT_SAMPLES)
      smp[tid] = A[(uint32_t)(((unsigned long long)tid * m) / (unsigned long long)C::SPLIT_SAMPLES)];
    cbar();
    if (tid < C::SPLIT_SAMPLES) {
      const B x = smp[tid];
      uint32_t rank = 0;
      constexpr int PER16 = 16 / (int)sizeof(B);
      const uint4* v4 = reinterpret_cast<const uint4*>(smp);
#pragma unroll 4
      for (int q = 0; q < C::SPLIT_SAMPLES / PER16; ++q) {
        const uint4 w = v4[q];
        B y[PER16];
        memcpy(y, &w, 16);
#pragma unroll
        for (int u = 0; u < PER16; ++u) rank += (y[u] < x) | ((y[u] == x) & (q * PER16 + u < tid));
      }
      const uint32_t step = (uint32_t)C::SPLIT_SAMPLES / nb;
      const uint32_t q1 = (rank + 1u) / step;
      if ((rank + 1u) % step == 0u && q1 < nb) {
        const uint32_t tz = (uint32_t)__ffs(q1) - 1u;
        sm.spl[(1u << (lg - 1u - tz)) + (q1 >> (tz + 1u))] = x;
      }
    }
    cbar();
    // KU keys per thread in flight: their tree walks (one dependent shared load per level) and
    // the scatter's atomic-then-store chains overlap (four 32-bit keys; two 64-bit keys, where
    // four measured slower)
    constexpr uint32_t KU = sizeof(B) == 4 ? 4u : 2u;
    uint32_t i0 = tid;
    for (; i0 + (KU - 1u) * (uint32_t)C::NC < m; i0 += KU * (uint32_t)C::NC) {
      B k[KU];
      uint32_t b[KU];
#pragma unroll
      for (uint32_t u = 0; u < KU; ++u) {
        k[u] = A[i0 + u * (uint32_t)C::NC];
        b[u] = 1u;
      }
      for (uint32_t l = 0; l < lg; ++l) {
#pragma unroll
        for (uint32_t u = 0; u < KU; ++u) b[u] = 2u * b[u] + (sm.spl[b[u]] < k[u] ? 1u : 0u);
      }
#pragma unroll
      for (uint32_t u = 0; u < KU; ++u) {
        sm.lb[i0 + u * (uint32_t)C::NC] = (uint8_t)(b[u] - nb);
        atomicAdd(&sm.bcnt[b[u] - nb], 1u);
      }
    }
    for (uint32_t i = i0; i < m; i += C::NC) {
      const B k = A[i];
      uint32_t b = 1u;
      for (uint32_t l = 0; l < lg; ++l) b = 2u * b + (sm.spl[b] < k ? 1u : 0u);
      sm.lb[i] = (uint8_t)(b - nb);
      atomicAdd(&sm.bcnt[b - nb], 1u);
    }
    cbar();
    if (warp == 0) {
      // lane l owns buckets 8l .. 8l + 7 (counts past nb are zero)
      const uint4 c0 = reinterpret_cast<const uint4*>(sm.bcnt)[2 * lane];
      const uint4 c1 = reinterpret_cast<const uint4*>(sm.bcnt)[2 * lane + 1];
      const uint32_t sum = c0.x + c0.y + c0.z + c0.w + c1.x + c1.y + c1.z + c1.w;
      uint32_t inc = sum;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += t;
      }
      uint4 s0, s1;
      s0.x = inc - sum;
      s0.y = s0.x + c0.x;
      s0.z = s0.y + c0.y;
      s0.w = s0.z + c0.z;
      s1.x = s0.w + c0.w;
      s1.y = s1.x + c1.x;
      s1.z = s1.y + c1.y;
      s1.w = s1.z + c1.z;
      reinterpret_cast<uint4*>(sm.bstart)[2 * lane] = s0;
      reinterpret_cast<uint4*>(sm.bstart)[2 * lane + 1] = s1;
      reinterpret_cast<uint4*>(sm.bcnt)[2 * lane] = s0;
      reinterpret_cast<uint4*>(sm.bcnt)[2 * lane + 1] = s1;
      if (lane == 31) sm.bstart[C::NB_MAX] = inc;  // = m
    }
    cbar();
    if ((uint32_t)tid < nb) {  // enter bucket tid in the list of its class
      const uint32_t c = sm.bstart[tid + 1] - sm.bstart[tid];
      if (c) {
        const uint32_t k = c > (uint32_t)C::TINY ? 6u : 32u - (uint32_t)__clz((c - 1u) / (uint32_t)C::R);
        sm.cls_list[k][atomicAdd(&sm.cls_cnt[k], 1u)] = (uint8_t)tid;
      }
    }
    uint32_t j0 = tid;
    for (; j0 + (KU - 1u) * (uint32_t)C::NC < m; j0 += KU * (uint32_t)C::NC) {
      uint32_t pos[KU];
#pragma unroll
      for (uint32_t u = 0; u < KU; ++u) pos[u] = atomicAdd(&sm.bcnt[sm.lb[j0 + u * (uint32_t)C::NC]], 1u);
#pragma unroll
      for (uint32_t u = 0; u < KU; ++u)
        if (GQS_OK(pos[u] < m, a.q, 0xB00Bull)) sm.tileB[pos[u]] = A[j0 + u * (uint32_t)C::NC];
    }
    for (uint32_t i = j0; i < m; i += C::NC) {
      const uint32_t pos = atomicAdd(&sm.bcnt[sm.lb[i]], 1u);
      if (GQS_OK(pos < m, a.q, 0xB00Bull)) sm.tileB[pos] = A[i];
    }
    cbar();
    // Tasks in the order class 6, 5, ..., 0 (largest networks first); each warp takes the next
    // task from a shared counter whenever it is free, so the long tasks spread first and the
    // short ones fill the gaps.
    uint32_t fin = 0;
    for (;;) {
      uint32_t t = 0;
      if (lane == 0) t = atomicAdd(&sm.task_next, 1u);
      t = __shfl_sync(0xffffffffu, t, 0);
      int k = 6;
      uint32_t per = 1u, ntk = sm.cls_cnt[6];
      while (t >= ntk && k > 0) {  // skip whole classes: t becomes the index within class k
        t -= ntk;
        --k;
        per = 32u >> k;
        ntk = (sm.cls_cnt[k] + per - 1u) >> (5 - k);
      }
      if (t >= ntk) break;  // past the last task of class 0
      const uint8_t* list = sm.cls_list[k] + t * per;
      const uint32_t cnt = min(per, sm.cls_cnt[k] - t * per);
      switch (k) {
        case 6: {
          const uint32_t b = list[0];
          fin += place_child(a, sm, A, sm.bstart[b], sm.bstart[b + 1], 1u, lp);  // a slice-partitioned segment
          break;
        }
        case 5: fin += bucket_networks<32>(sm, A, list, cnt); break;
        case 4: fin += bucket_networks<16>(sm, A, list, cnt); break;
        case 3: fin += bucket_networks<8>(sm, A, list, cnt); break;
        case 2: fin += bucket_networks<4>(sm, A, list, cnt); break;
        case 1: fin += bucket_networks<2>(sm, A, list, cnt); break;
        default: fin += bucket_networks<1>(sm, A, list, cnt); break;
      }
    }
    return fin;
  }

  // Sorts A[0, m) (comparison keys) with all consumer warps. On return A holds the keys sorted.
  static __device__ __forceinline__ void local_sort(const SortArgs<T>& a, Smem<C>& sm, B* A, uint32_t m,
                                                 unsigned long long* lp) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#ifdef GQS_PROFILE
    const long long t0 = clock64();
#endif
    if (tid == 0) {
      sm.lr_head = 0;
      sm.lr_tail = 0;
      sm.ls_done = 0;
    }
    for (uint32_t i = tid; i < (uint32_t)C::LREC; i += C::NC) sm.lrec[i].seq = 0u;
    cbar();
    if (m >= (uint32_t)C::SPLIT_MIN) {
      const uint32_t fin = sample_split(a, sm, A, m, lp);
      if (lane == 0 && fin) atomicAdd(&sm.ls_done, fin);
    } else if (warp == 0) {
      const uint32_t fin = place_child(a, sm, A, 0, m, 0u, lp);
      if (lane == 0 && fin) atomicAdd(&sm.ls_done, fin);
    }
    // every warp takes slices until every key of the tile is placed
    uint32_t spins = 0;
    for (;;) {
      uint32_t ri = 0, c = 0, state = 0;  // 0 nothing yet, 1 slice, 2 done
      if (lane == 0) {
        const uint32_t h = *(volatile uint32_t*)&sm.lr_head;
        const uint32_t t = *(volatile uint32_t*)&sm.lr_tail;
        if (h < t && h < (uint32_t)C::LREC) {
          if (*(volatile uint32_t*)&sm.lrec[h].seq == h + 1u) {
            const uint32_t cc = atomicAdd(&sm.lrec[h].cursor, 1u);
            if (cc < sm.lrec[h].nsl) {
              ri = h;
              c = cc;
              state = 1;
            } else {
              atomicCAS(&sm.lr_head, h, h + 1u);
              state = 3;  // retry at once
            }
          }
        } else if (*(volatile uint32_t*)&sm.ls_done >= m) {
          state = 2;
        } else if (h >= (uint32_t)C::LREC) {
          state = 2;  // record overflow was reported; stop
        }
        if (state == 0) {
          if (++spins > (1u << 24) || ((spins & 1023u) == 0u && ld_relaxed(&a.q->error))) {
            set_error(a.q, ST_TIMEOUT, 0x15ull);
            state = 2;
          }
        }
      }
      state = __shfl_sync(0xffffffffu, state, 0);
      if (state == 2) break;
      if (state != 1) continue;
      ri = __shfl_sync(0xffffffffu, ri, 0);
      c = __shfl_sync(0xffffffffu, c, 0);
      __threadfence_block();
#ifdef GQS_PROFILE
      const long long ts = clock64();
#endif
      run_slice(a, sm, A, ri, c, lp);
#ifdef GQS_PROFILE
      if (lane == 0) lp[5] += (unsigned long long)(clock64() - ts);
#endif
    }
    cbar();
#ifdef GQS_PROFILE
    if (tid == 0) lp[1] += (unsigned long long)(clock64() - t0);
#endif
  }

  // Leader-only bounded wait for ring slot k; every consumer reads the verdict after the
  // next named barrier, so all consumer threads always take the same path.
  static __device__ __forceinline__ void leader_wait_slot(const SortArgs<T>& a, Smem<C>& sm, uint32_t k) {
    sm.cons_ok = mbar_wait(&sm.full[k % C::STAGES], (k / C::STAGES) & 1u, a.q, a.timeout_ns, 6) ? 1u : 0u;
  }

  static __device__ void consumers(const SortArgs<T>& a, Smem<C>& sm) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t k = 0, nloc = 0, npart = 0;
    // pend: counted, offsets requested, scattered next iteration; scat: scattered last
    // iteration, posted to the completer at the next barrier.
    bool have_pend = false, have_scat = false;
    B pend[C::KPT];
    uint32_t pend_len = 0, pend_job = 0, pend_par = 0, scat_job = 0;
    B pend_p = 0;
    B* pend_dst = nullptr;
#ifdef GQS_CHECK
    unsigned long long pend_lo = 0, pend_hi = 0;
#endif
    unsigned long long st_part = 0, st_local = 0, st_chunks = 0;
    uint32_t st_local_jobs = 0, st_fill_jobs = 0;
    // Leader cycles by item kind (Queue::phase), kept in shared memory by thread 0 alone, so that
    // no register is held across the loop for them; partition chunks are not timed.
    if (tid == 0) {
      sm.ph[0] = sm.ph[1] = sm.ph[2] = 0ull;
      sm.ph[4] = (unsigned long long)clock64();
    }
    GQS_PROF_DECL
    GQS_PROF_T(t_all)

    if (tid == 0) leader_wait_slot(a, sm, 0);
    cbar();
    for (;;) {
      if (!sm.cons_ok) break;
      GQS_PROF_T(t_it)
      GQS_PROF_CNT(PF_N_ITEMS, 1)
      const uint32_t s = k % C::STAGES;
      (void)mbar_test(&sm.full[s], (k / C::STAGES) & 1u);  // completed; gives this thread acquire order
      const Desc dd = sm.desc[s];
      if (dd.kind == ITEM_PART) {
        // The stage holds the chunk's 16-byte granules: keys [off, off + len) of an aligned
        // window of CHUNK keys. Each thread reads 16-byte vectors; positions outside the chunk
        // take the pivot's value, which neither side counts or keeps.
        const B p = (B)dd.pivot;
        B cur[C::KPT];
        constexpr int VEC = 16 / (int)sizeof(B);
        const uint4* win = reinterpret_cast<const uint4*>(sm.stage[s]);
#pragma unroll
        for (int v = 0; v < C::KPT / VEC; ++v) {
          const uint4 w = win[v * C::NC + tid];
          B t[VEC];
          memcpy(t, &w, 16);
#pragma unroll
          for (int q = 0; q < VEC; ++q) cur[v * VEC + q] = t[q];
        }
        if (dd.off != 0 || dd.len != (uint32_t)C::CHUNK) {
          const B praw = Ops::raw(p);
#pragma unroll
          for (int v = 0; v < C::KPT / VEC; ++v) {
#pragma unroll
            for (int q = 0; q < VEC; ++q) {
              const uint32_t idx = (uint32_t)((v * C::NC + tid) * VEC + q);
              if (idx < dd.off || idx >= dd.off + dd.len) cur[v * VEC + q] = praw;
            }
          }
        }
        uint32_t cl = 0, cg = 0;
#pragma unroll
        for (int j = 0; j < C::KPT; ++j) {
          const B kk = Ops::key(cur[j]);
          cl += kk < p;
          cg += kk > p;
        }
        const uint32_t par = npart % 3u;
        cl = __reduce_add_sync(0xffffffffu, cl);
        cg = __reduce_add_sync(0xffffffffu, cg);
        if (lane == 0) {
          sm.wlt[par][warp] = cl;
          sm.wgt[par][warp] = cg;
        }
        GQS_PROF_ADD(PF_C_COUNT, t_it)
        cbar();  // #1: stage s read into registers; the previous scatter is complete
        GQS_PROF_T(t_l)
        // The bookkeeping between the two barriers is split over three threads of different
        // warps, so that its waits overlap: warp 0 releases the stage, sums the warp counts,
        // asks the reserver warp for this chunk's output ranges (used one iteration later, when
        // this chunk is scattered) and waits for the pending chunk's ranges; lane 0 of warp 1
        // posts the chunk scattered last iteration to the completer; lane 0 of warp 2 waits for
        // the next stage. Each publishes its verdict before barrier #2.
        if (warp == 0) {
          uint32_t ls = lane < C::NCW ? sm.wlt[par][lane] : 0u, gs = lane < C::NCW ? sm.wgt[par][lane] : 0u;
          ls = __reduce_add_sync(0xffffffffu, ls);
          gs = __reduce_add_sync(0xffffffffu, gs);
          if (lane == 0) {
            mbar_arrive(&sm.empty[s]);
            const uint32_t e = npart % C::RQ;
            sm.rq_job[e] = dd.job;
            sm.rq_ls[e] = ls;
            sm.rq_gs[e] = gs;
            sts_release(&sm.rq_tail, npart + 1);
            GQS_PROF_T(tw)
            sm.cons_ok = (!have_pend || leader_wait_reservation(a, sm, npart - 1)) ? 1u : 0u;
            GQS_PROF_ADD(PF_C_WAIT, tw)
          }
        } else if (tid == 32) {
          if (have_scat) post_chunk(a, sm, scat_job);
        } else if (tid == 64) {
          sm.slot_ok = mbar_wait(&sm.full[(k + 1) % C::STAGES], ((k + 1) / C::STAGES) & 1u, a.q, a.timeout_ns, 6)
                           ? 1u : 0u;
        }
        cbar();  // #2: the pending chunk's ranges are reserved; next slot verdict published
        GQS_PROF_ADD(PF_C_LEADER, t_l)
        if (!sm.cons_ok || !sm.slot_ok) break;
        GQS_PROF_T(t_sc)
        have_scat = false;
        if (have_pend) {
          const uint32_t e = (npart - 1) % C::RQ;
          scatter_chunk(pend, pend_p, pend_dst, sm.rs_lb[e], sm.rs_gb[e], sm.wlt[pend_par],
                        sm.wgt[pend_par] GQS_CHECK_ARGS(pend_lo, pend_hi, a.q));
          have_scat = true;
          scat_job = pend_job;
        }
        GQS_PROF_ADD(PF_C_SCATTER, t_sc)
#pragma unroll
        for (int j = 0; j < C::KPT; ++j) pend[j] = cur[j];
        pend_len = dd.len;
        pend_job = dd.job;
        pend_par = par;
        pend_p = p;
        pend_dst = dd.dir ? a.dn : a.d;
#ifdef GQS_CHECK
        pend_lo = dd.jlo;
        pend_hi = dd.jhi;
#endif
        have_pend = true;
        st_part += dd.len;
        ++st_chunks;
        ++npart;
        ++k;
        GQS_PROF_ADD(PF_C_PART, t_it)
        continue;
      }

      // Any other item first drains the pipeline of partition chunks.
      if (tid == 0) {
        if (have_scat) post_chunk(a, sm, scat_job);
        if (have_pend && !leader_wait_reservation(a, sm, npart - 1)) sm.cons_ok = 0;
      }
      cbar();
      if (!sm.cons_ok) break;
      if (have_pend) {
        const uint32_t e = (npart - 1) % C::RQ;
        scatter_chunk(pend, pend_p, pend_dst, sm.rs_lb[e], sm.rs_gb[e], sm.wlt[pend_par],
                      sm.wgt[pend_par] GQS_CHECK_ARGS(pend_lo, pend_hi, a.q));
      }
      cbar();
      if (tid == 0) {
        if (have_pend) post_chunk(a, sm, pend_job);
        mbar_arrive(&sm.empty[s]);  // every thread copied the descriptor before the barriers above
      }
      have_pend = false;
      have_scat = false;
      // The pending keys are dead now; giving them a constant lets the compiler reuse their
      // registers in the on-chip sort and the fills below (otherwise they stay live around the loop).
#pragma unroll
      for (int j = 0; j < C::KPT; ++j) pend[j] = B(0);
      GQS_PROF_ADD(PF_C_DRAIN, t_it)

      if (dd.kind == ITEM_TERM) break;
      if (tid == 0) sm.ph[3] = (unsigned long long)clock64();
      if (dd.kind == ITEM_FILL) {
        // Queued pivot-run fill: write the raw pivot over d[gbeg, gbeg + len).
        GQS_PROF_T(tf)
        const B raw = Ops::raw((B)dd.pivot);
        B* out = a.d + dd.gbeg;
        const uint32_t flen = GQS_OK(dd.gbeg + dd.len <= a.n, a.q, 0xB008ull) ? dd.len : 0u;
        for (uint32_t i = tid; i < flen; i += C::NC) out[i] = raw;
        ++st_fill_jobs;
        GQS_PROF_ADD(PF_C_FILL, tf)
        if (tid == 0) atomicAdd(&a.q->done, (unsigned long long)dd.len);
        if (tid == 0) sm.ph[2] += (unsigned long long)clock64() - sm.ph[3];
      } else if (dd.kind == ITEM_LOCAL) {
        GQS_PROF_T(tl)
        if (tid == 0) sm.lok = mbar_wait(&sm.lfull, nloc & 1u, a.q, a.timeout_ns, 7) ? 1u : 0u;
        cbar();
        if (!sm.lok) break;
        GQS_PROF_ADD(PF_C_LWAIT, tl)

        (void)mbar_test(&sm.lfull, nloc & 1u);
        B* A = sm.tileA + dd.off;
        const uint32_t m = dd.len;
        if (!Ops::kIdentity) {
          for (uint32_t i = tid; i < m; i += C::NC) A[i] = Ops::key(A[i]);
          cbar();
        }
        unsigned long long lp[14] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        local_sort(a, sm, A, m, lp);
        GQS_PROF_CNT(PF_C_LCTA, lp[0])
        GQS_PROF_CNT(PF_C_LWARP, lp[1])
        GQS_PROF_CNT(PF_N_LCTA, lp[2])
        GQS_PROF_CNT(PF_N_LWARP, lp[3])
        GQS_PROF_CNT(PF_N_LBIT, lp[4])
#ifdef GQS_PROFILE
        if (lane == 0) {  // per-warp totals of the warp phase
          atomicAdd(&a.q->prof[PF_W_WAIT], lp[5]);
          atomicAdd(&a.q->prof[PF_W_PART], lp[6]);
          atomicAdd(&a.q->prof[PF_W_BIT], lp[7]);
          atomicAdd(&a.q->prof[PF_W_SEGS], lp[8]);
        }
#endif
        GQS_PROF_CNT(PF_N_LOCAL, 1)
        GQS_PROF_T(ts)

        if (!Ops::kIdentity) {
          for (uint32_t i = tid; i < m; i += C::NC) A[i] = Ops::raw(A[i]);
        }
        // Write the sorted tile to d: one bulk TMA store for the 16-byte-aligned body,
        // plain stores for the ragged ends (a bulk store must not touch bytes outside).
        B* out = a.d + dd.gbeg;
        const uint32_t mw = GQS_OK(dd.gbeg + m <= a.n, a.q, 0xB009ull) ? m : 0u;  // keys written
        const uintptr_t olo = reinterpret_cast<uintptr_t>(out);
        const uintptr_t ohi = reinterpret_cast<uintptr_t>(out + mw);
        const uintptr_t ga = (olo + 15) & ~uintptr_t(15), gb = ohi & ~uintptr_t(15);
        const uint32_t head = (uint32_t)((ga - olo) / sizeof(B));
        const bool tma_ok = ga < gb && ((smem_addr(A + head) & 15u) == 0u);
        if (tma_ok) {
          fence_proxy_async_smem();
          cbar();
          const uint32_t tail0 = (uint32_t)((gb - olo) / sizeof(B));
          if (tid == 0) {
            bulk_store(reinterpret_cast<void*>(ga), A + head, (uint32_t)(gb - ga));
            bulk_commit();
          }
          for (uint32_t i = tid; i < head; i += C::NC) out[i] = A[i];
          for (uint32_t i = tail0 + tid; i < mw; i += C::NC) out[i] = A[i];
          if (tid == 0) bulk_wait_read_all();
        } else {
          cbar();
          for (uint32_t i = tid; i < mw; i += C::NC) out[i] = A[i];
        }
        cbar();  // every read of the tile is done before the producer may refill it
        if (tid == 0) {
          mbar_arrive(&sm.lempty);
          atomicAdd(&a.q->done, (unsigned long long)m);
#ifdef GQS_PROFILE
          level_note(a.q, __ldcg(&a.jobs[dd.job].depth), 2, m);
#endif
        }
        GQS_PROF_ADD(PF_C_LSTORE, ts)
        st_local += m;
        ++st_local_jobs;
        ++nloc;
        if (tid == 0) sm.ph[1] += (unsigned long long)clock64() - sm.ph[3];
      }
      // ITEM_FLUSH needs nothing beyond the drain above.
      if (tid == 0) leader_wait_slot(a, sm, k + 1);
      cbar();
      ++k;
    }
    GQS_PROF_ADD(PF_C_TOTAL, t_all)
    if (tid == 0) {
      GQS_PROF_FLUSH(a.q)
      bulk_wait_all();
      sts_release(&sm.term, 1u);
      if (st_part) atomicAdd(&a.q->part_keys, st_part);
      if (st_local) atomicAdd(&a.q->local_keys, st_local);
      if (st_chunks) atomicAdd(&a.q->chunks, st_chunks);
      if (st_local_jobs) atomicAdd(&a.q->local_jobs, st_local_jobs);
      if (st_fill_jobs) atomicAdd(&a.q->fill_jobs, st_fill_jobs);
      atomicAdd(&a.q->phase[1], sm.ph[1]);
      atomicAdd(&a.q->phase[2], sm.ph[2]);
      atomicAdd(&a.q->phase[3], (unsigned long long)clock64() - sm.ph[4]);
    }
  }
};

// CTAs per SM the kernel is compiled for: two when two CTAs' shared memory fits an SM (the
// register budget per thread halves accordingly), else one.
template <class C>
constexpr int min_blocks_per_sm() {
  return sizeof(Smem<C>) <= 110u * 1024u ? 2 : 1;
}

template <class C>
__global__ void __launch_bounds__(C::NT, min_blocks_per_sm<C>()) persistent_kernel(SortArgs<typename C::T> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem<C>& sm = *reinterpret_cast<Smem<C>*>(smem_raw);
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int i = 0; i < C::STAGES; ++i) {
      mbar_init(&sm.full[i], 1);
      mbar_init(&sm.empty[i], 1);
    }
    mbar_init(&sm.lfull, 1);
    mbar_init(&sm.lempty, 1);
    sm.cq_head = 0;
    sm.cq_tail = 0;
    sm.term = 0;
    sm.rq_tail = 0;
    for (int i = 0; i < C::RQ; ++i) sm.rs_done[i] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  pdl_wait();  // the seed kernel's jobs and tickets are visible from here on
#ifdef GQS_PROFILE
  if (tid == 0) atomicCAS(&a.q->lvl_start, 0ull, (unsigned long long)global_timer_ns());
#endif
  const int warp = tid >> 5;
  if (warp < C::NCW) {
    Persistent<C>::consumers(a, sm);
  } else if (warp == C::NCW) {
    Persistent<C>::producer(a, sm);
  } else if (warp == C::NCW + 1) {
    Persistent<C>::completer(a, sm);
  } else {
    Persistent<C>::reserver(a, sm);
  }
}

}  // namespace gqs
