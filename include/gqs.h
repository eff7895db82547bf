/*
 * gqs -- GPU-Quicksort for NVIDIA GB300 (sm_103a): the C ABI.
 *
 * This is the drop-in boundary for the reference's single-array sort,
 * rioffe/gpu-quicksort `template <class T> void GPUQSort(OCLResources*, size_t size, T* d, T* dn)`
 * (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:835-906; uint-only form at
 * GPU-Quicksort_OpenCL_1.2/QuicksortMain.cpp:297-384), which its benchmark driver calls as
 * GPUQSort(&myOCL, arraySize, pArray, pArrayCopy) (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:1114).
 * The reference is C++ templates only; these plain-C entry points are what an FFI
 * (ctypes, cgo, JNI) binds, and include/gqs/Quicksort.h restores the template.
 *
 * Conventions
 *   - Every call returns a gqs_status. Nothing here calls exit(), abort() or traps; device-side
 *     failures (a bounded wait that ran out, a full job queue) come back as a status.
 *   - Keys: uint32_t, float, double. Output is ascending and identical to std::sort for inputs
 *     without NaN; -0.0 sorts before +0.0 (both are kept bit for bit).
 *   - A gqs_ctx is bound to one device. Calls on one context are serialised (internally
 *     locked, and device work of consecutive calls is ordered even across streams). Use one
 *     context per concurrent stream for overlap.
 *   - Nothing is allocated on the device-pointer path once the context's pools have grown to
 *     the largest size seen (first call at a new size allocates; gqs_reserve pre-grows).
 */
#ifndef GQS_H
#define GQS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gqs_ctx gqs_ctx;

typedef enum gqs_status {
  GQS_OK = 0,
  GQS_ERR_INVALID = 1,   /* null / misaligned pointer, size out of range, bad segment table */
  GQS_ERR_CUDA = 2,      /* a CUDA runtime call failed */
  GQS_ERR_NOMEM = 3,     /* device or pinned allocation failed */
  GQS_ERR_TIMEOUT = 4,   /* a bounded device-side wait ran out (the sort made no progress) */
  GQS_ERR_CAPACITY = 5,  /* the device job queue overflowed (pathological pivot sequence) */
  GQS_ERR_NO_DEVICE = 6, /* no usable CUDA device, or not an sm_103 GPU */
  GQS_ERR_INTERNAL = 7,  /* an internal invariant failed on the device */
  GQS_ERR_CANCELLED = 8, /* a server request was cancelled before it ran */
  GQS_ERR_BOUNDS = 9     /* a -DGQS_CHECK build found a job record, range or write index outside
                            the sort's bounds (and skipped the access) */
} gqs_status;

typedef enum gqs_dtype { GQS_U32 = 0, GQS_F32 = 1, GQS_F64 = 2 } gqs_dtype;

typedef struct gqs_config {
  int32_t variant;     /* -1: per sort, the tuned variant for its key type and size; else fixed */
  uint32_t timeout_ms; /* device-side no-progress limit for bounded waits; 0 means 4000 */
  uint32_t sync;       /* 1 (default): *_dev calls wait for the stream and return the device status */
  uint32_t timing;     /* 1: time the persistent kernel with CUDA events (gqs_stats.kernel_ms) */
  uint32_t reserved[4];
} gqs_config;

typedef struct gqs_stats {
  uint64_t keys;       /* keys in the last sort */
  uint64_t part_keys;  /* keys read by partition chunks, summed over all levels */
  uint64_t local_keys; /* keys sorted on chip by local jobs */
  uint64_t tiny_keys;  /* keys sorted in registers by a single warp */
  uint64_t fill_keys;  /* pivot-run keys written by the completer warp */
  uint64_t chunks;     /* partition chunks processed */
  uint64_t algo_bytes; /* key bytes * 2 * (part_keys + local_keys + tiny_keys) */
  uint32_t part_jobs, local_jobs, fill_chunks, max_depth;
  uint32_t status, variant, grid, threads;
  double kernel_ms; /* persistent-kernel time from CUDA events, or -1 when timing is off */
} gqs_stats;

typedef struct gqs_variant_desc {
  int32_t threads, tile, chunk, kpt, stages, tiny;
  uint64_t smem_bytes;
  char name[64];
} gqs_variant_desc;

/* Fills *cfg with the defaults (variant -1, timeout 4000 ms, sync 1, timing 0). */
void gqs_config_default(gqs_config* cfg);

/* Creates a context on `device` (cfg may be NULL for the defaults). */
gqs_status gqs_create(gqs_ctx** out, int device, const gqs_config* cfg);
void gqs_destroy(gqs_ctx* ctx);

/* Pre-grows the context's pools for n keys of `dtype` in up to `nseg` segments, so later
 * calls of that size allocate nothing. with_buffers also sizes the key/scratch pools that the
 * host-pointer calls stage through. */
gqs_status gqs_reserve(gqs_ctx* ctx, int dtype, size_t n, size_t nseg, int with_buffers);

/* Host-pointer sorts, the reference's semantics: `d` (host memory, n keys) is sorted in place.
 * `dn` is the reference's scratch array; it is not touched and may be NULL (device scratch
 * comes from the context pool). Keys travel over one host->device and one device->host copy
 * (fastest from pinned memory). Replaces GPUQSort<T>(OCLResources*, size, d, dn),
 * GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:835-836. */
gqs_status gqs_sort_u32(gqs_ctx* ctx, uint32_t* d, uint32_t* dn, size_t n);
gqs_status gqs_sort_f32(gqs_ctx* ctx, float* d, float* dn, size_t n);
gqs_status gqs_sort_f64(gqs_ctx* ctx, double* d, double* dn, size_t n);

/* Device-pointer sorts: `d` (device memory, n keys) is sorted in place; `scratch` is n keys of
 * device memory clobbered by the sort (the reference's dn), or NULL to use the context pool.
 * Work is ordered on `stream` (a cudaStream_t; NULL = legacy default stream). With
 * cfg.sync = 1 the call waits and returns the device status; with sync = 0 it returns after
 * enqueueing and gqs_sync() reports the device status. Same replacement as above, with the
 * buffers already resident in HBM. */
gqs_status gqs_sort_u32_dev(gqs_ctx* ctx, uint32_t* d, uint32_t* scratch, size_t n, void* stream);
gqs_status gqs_sort_f32_dev(gqs_ctx* ctx, float* d, float* scratch, size_t n, void* stream);
gqs_status gqs_sort_f64_dev(gqs_ctx* ctx, double* d, double* scratch, size_t n, void* stream);

/* Segmented sorts: keys[offsets[i], offsets[i+1]) is sorted independently for each of the
 * nseg segments, all in one persistent launch. offsets holds nseg + 1 non-decreasing entries
 * (device memory for *_dev, host memory otherwise) with offsets[nseg] <= n, where n is the
 * length of keys (and of scratch). No reference counterpart: the reference sorts one array per
 * call; this is the batched form of the same GPUQSort<T> path. */
gqs_status gqs_sort_segments_u32_dev(gqs_ctx* ctx, uint32_t* keys, uint32_t* scratch, size_t n,
                                     const uint64_t* offsets, size_t nseg, void* stream);
gqs_status gqs_sort_segments_f32_dev(gqs_ctx* ctx, float* keys, float* scratch, size_t n,
                                     const uint64_t* offsets, size_t nseg, void* stream);
gqs_status gqs_sort_segments_f64_dev(gqs_ctx* ctx, double* keys, double* scratch, size_t n,
                                     const uint64_t* offsets, size_t nseg, void* stream);
gqs_status gqs_sort_segments_u32(gqs_ctx* ctx, uint32_t* keys, size_t n, const uint64_t* offsets, size_t nseg);
gqs_status gqs_sort_segments_f32(gqs_ctx* ctx, float* keys, size_t n, const uint64_t* offsets, size_t nseg);
gqs_status gqs_sort_segments_f64(gqs_ctx* ctx, double* keys, size_t n, const uint64_t* offsets, size_t nseg);

/* Key-value sorts: n (key, value) pairs, keys uint32 or float, values uint32, sorted by key with
 * every value travelling with its key. Pairs with equal keys come out in ascending value order,
 * so values 0..n-1 give a stable argsort (the sorting permutation). Host-pointer forms sort both
 * host arrays in place; *_dev forms take device arrays and a stream (cfg.sync as above). Each
 * pair is packed into one 64-bit word (the key's order-preserving map above the value) and
 * the words are sorted by the same persistent kernel. No reference counterpart: the reference
 * sorts keys only; this is the key-value variant of its GPUQSort<T> path. */
gqs_status gqs_sort_pairs_u32(gqs_ctx* ctx, uint32_t* keys, uint32_t* values, size_t n);
gqs_status gqs_sort_pairs_f32(gqs_ctx* ctx, float* keys, uint32_t* values, size_t n);
gqs_status gqs_sort_pairs_u32_dev(gqs_ctx* ctx, uint32_t* keys, uint32_t* values, size_t n, void* stream);
gqs_status gqs_sort_pairs_f32_dev(gqs_ctx* ctx, float* keys, uint32_t* values, size_t n, void* stream);

/* Largest n accepted by gqs_sort_u32_noalloc. */
#define GQS_NOALLOC_MAX_KEYS (1u << 20)

/* Sort that allocates nothing, for callers that must not allocate device memory when they sort:
 * hosts that give all device memory to their own pool at start-up and forbid allocations later,
 * and latency-critical code that cannot take cudaMalloc's implicit device synchronisation.
 * Such callers cannot create a gqs_ctx (its pools are cudaMalloc'd), so this call takes none.
 * Sorts d (device memory, n <= GQS_NOALLOC_MAX_KEYS uint32 keys) in place on the current
 * device and `stream`, waits, and returns the device status; larger n returns GQS_ERR_INVALID
 * before any work. All of its scratch is one static device array inside the library (about
 * 6 MB, held by every GPU that loads the library until the process exits) shared by every call:
 * calls that overlap on the GPU race, so the caller serialises them. The first call on a device
 * looks up that array's address and prepares the kernel. Every call blocks: it reads the
 * status block back and synchronises `stream` before it returns, so it must never be made on a
 * stream that is being captured into a CUDA graph. The device-side no-progress limit is fixed
 * at 4 s (there is no context to configure it): a sort that stalls returns GQS_ERR_TIMEOUT after
 * about 4 s, and the static array then still holds that call's partial state, which the next
 * call clears before it starts. No counterpart in the reference, which allocates its buffers
 * per call. */
gqs_status gqs_sort_u32_noalloc(uint32_t* d, size_t n, void* stream);

/* ---- Batched sort, captured once as a CUDA graph ------------------------------------------
 * A batch sorts up to max_segments independent arrays (segments) of one key type, holding up to
 * max_keys keys in total, in one persistent launch. It owns its device memory: a key arena of
 * max_keys keys that the caller fills (gqs_batch_keys), its scratch, the job records, ticket
 * ring and status block. The work of one batch (copy of the segment table from pinned host
 * memory, clearing of the status block and ring, the seed kernel, the persistent kernel, the
 * read-back of the status block) is captured once per kernel variant as a CUDA graph;
 * gqs_batch_launch replays it with a single cudaGraphLaunch. The segment table is data, so
 * batches of any shape up to the maxima replay the same graph.
 * No reference counterpart: the reference sorts one array per call
 * (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:835-906); this is the batched form of that path. */
typedef struct gqs_batch gqs_batch;

/* cfg may be NULL; cfg->variant (>= 0) picks the initial kernel variant, cfg->timeout_ms the
 * device-side no-progress limit. */
gqs_status gqs_batch_create(int device, int dtype, size_t max_keys, size_t max_segments, const gqs_config* cfg,
                            gqs_batch** out);
void gqs_batch_destroy(gqs_batch* b);
/* The device key arena (max_keys keys of the batch's type); segments index into it. */
void* gqs_batch_keys(gqs_batch* b);
/* The pinned host segment table: max_segments + 1 non-decreasing boundaries; segment i is
 * keys[offsets[i], offsets[i+1]). Write the first nseg + 1 entries before gqs_batch_launch. */
uint64_t* gqs_batch_offsets(gqs_batch* b);
/* Sorts the nseg segments of the table: waits for the batch's previous replay (which reads the
 * table), checks the table on the host, then enqueues one graph replay on `stream`. */
gqs_status gqs_batch_launch(gqs_batch* b, size_t nseg, void* stream);
/* Waits for the last replay; returns its device status and fills *stats (may be NULL);
 * stats->kernel_ms is the replay's time from CUDA events. */
gqs_status gqs_batch_wait(gqs_batch* b, gqs_stats* stats);
/* Synchronous copies between host memory and keys [first, first + n) of the arena, for callers
 * without CUDA bindings of their own. */
gqs_status gqs_batch_copy_in(gqs_batch* b, const void* host, size_t first, size_t n);
gqs_status gqs_batch_copy_out(gqs_batch* b, void* host, size_t first, size_t n);
gqs_status gqs_batch_set_variant(gqs_batch* b, int variant);
int gqs_batch_get_variant(gqs_batch* b);
/* The autotuner. Times every kernel variant of the batch's key type on the batch as it stands
 * (the first nseg segments of the table, keys restored from a copy before every replay): one
 * warm-up replay, then `reps` timed replays, median kept. Variants differ in the partition ->
 * on-chip sort switch (tile keys), CTA size (consumer warps) and keys per thread of a partition
 * chunk (gqs_variant_describe). Writes each variant's median ms to ms[v] (-1: cannot run; ms may
 * be NULL), selects the fastest for later launches and returns it in *best. On return the keys
 * are sorted, by the chosen variant. Allocates a temporary copy of the keys. */
gqs_status gqs_batch_autotune(gqs_batch* b, size_t nseg, int reps, double* ms, int* best);

/* ---- Sort server: continuous batching of mixed requests ------------------------------------
 * A server owns a device arena (the memory budget) and a dispatcher thread. Submitted requests
 * (key type, host input, host output, n) are admitted in arrival order as soon as their keys
 * and scratch fit in the free part of the arena; their keys are then copied to the device and
 * wait there. Whenever one of `lanes` batches-in-flight is free, every resident request of one
 * key type (oldest type first, up to batch_segments requests and batch_keys keys) is sorted as
 * one segment of one graph-captured batch launch, and results are copied back to each
 * request's output. Requests that arrive while others run are admitted and launched as memory
 * and lanes free up, so copies and sorts of different batches overlap on the device. A
 * request's result does not depend on what it was batched with. Output buffers in page-locked
 * memory (cudaHostAlloc / cudaHostRegister) are filled asynchronously; pageable ones are filled
 * by a synchronous copy when the batch retires. No reference counterpart. */
typedef struct gqs_server gqs_server;

typedef struct gqs_server_config {
  uint64_t budget_bytes;   /* device memory for the server: records + keys + scratch; 0 = 64 GiB */
  uint64_t batch_keys;     /* most keys in one batch, and in one request; 0 = 2^27 */
  uint32_t batch_segments; /* most requests in one batch; 0 = 4096 */
  uint32_t lanes;          /* batches in flight; 0 = 3 */
  uint32_t timeout_ms;     /* device-side no-progress limit; 0 = 4000 */
  uint32_t per_request;    /* 1: no batching. One request at a time through the plain sort (copy
                              in, gqs_sort_<type>_dev, copy out, wait): the comparison baseline */
  int32_t variant[3];      /* kernel variant per key type (GQS_U32, GQS_F32, GQS_F64); -1 = 0 */
  uint32_t reserved[4];
} gqs_server_config;

typedef struct gqs_request_info {
  uint32_t status;         /* gqs_status of the request */
  uint32_t dtype;
  uint64_t n;
  uint64_t t_submit_ns;    /* gqs_srv_now_ns() clock */
  uint64_t t_admit_ns;     /* keys resident on the device (copy enqueued) */
  uint64_t t_launch_ns;    /* its batch launched */
  uint64_t t_done_ns;      /* result in the output buffer */
  uint32_t batch_requests; /* requests in its batch */
  uint32_t lane;
} gqs_request_info;

typedef struct gqs_server_stats {
  uint64_t submitted, completed, failed, cancelled, completed_keys;
  uint64_t batches, max_batch_requests;
  uint64_t arena_bytes, arena_used, arena_peak;
  uint64_t pending, outstanding;
} gqs_server_stats;

void gqs_srv_config_default(gqs_server_config* cfg);
gqs_status gqs_srv_create(int device, const gqs_server_config* cfg, gqs_server** out);
/* Finishes every submitted request, then stops the dispatcher and frees everything. */
void gqs_srv_destroy(gqs_server* s);
/* Queues a request: sort n keys of `dtype` read from `in` into `out` (host memory; may be the
 * same buffer). Both stay owned by the caller and must stay valid until the request completes.
 * n must be at most batch_keys. Returns at once with the request id. */
gqs_status gqs_srv_submit(gqs_server* s, int dtype, const void* in, void* out, size_t n, uint64_t* id);
/* Blocks until request `id` completes; returns its status, fills *info (may be NULL) and
 * forgets the id. */
gqs_status gqs_srv_wait(gqs_server* s, uint64_t id, gqs_request_info* info);
/* Returns the next completed request not yet collected (completion order), or GQS_ERR_TIMEOUT
 * when none completes within timeout_ms. */
gqs_status gqs_srv_wait_any(gqs_server* s, uint64_t* id, gqs_request_info* info, uint32_t timeout_ms);
/* Cancels a request that has not started: it completes at once with GQS_ERR_CANCELLED and its
 * device memory is released. Returns GQS_OK if it was cancelled, GQS_ERR_INVALID if the id is
 * unknown or the request is already running or finished. */
gqs_status gqs_srv_cancel(gqs_server* s, uint64_t id);
/* Blocks until every submitted request has completed. */
gqs_status gqs_srv_drain(gqs_server* s);
gqs_status gqs_srv_stats(gqs_server* s, gqs_server_stats* out);
/* The server's clock (steady, nanoseconds). */
uint64_t gqs_srv_now_ns(void);

/* Self-test of the bounded device waits. Runs the persistent kernel (key type `dtype`) on a job
 * queue that claims one unsorted key but holds no work, so every role of the kernel waits for
 * progress that never comes. Returns the status the kernel reports: GQS_ERR_TIMEOUT after about
 * timeout_ms (0 means the context's timeout) when the waits end as designed. No GPU fault, trap
 * or hang is involved; the context stays usable. No reference counterpart (the reference waits
 * on the host with blocking reads). */
gqs_status gqs_selftest_stalled_queue(gqs_ctx* ctx, int dtype, uint32_t timeout_ms);

/* Self-test of the bounds checks of a -DGQS_CHECK build (libgqs_check.so): sorts 2^16 keys of
 * type `dtype` in the context's pool while telling the kernel that key indices end at 2^15, so
 * the first job already lies outside the bound. A check build reports GQS_ERR_BOUNDS without
 * touching anything past the bound; the product build, whose checks are compiled out, sorts the
 * keys and returns GQS_OK. Every access stays inside the 2^16-key buffers either way. */
gqs_status gqs_selftest_bounds(gqs_ctx* ctx, int dtype);

/* Waits for the context's last enqueued sort and returns its device status. */
gqs_status gqs_sync(gqs_ctx* ctx);

/* Statistics of the last completed sort (waits for it if it is still running). */
gqs_status gqs_last_stats(gqs_ctx* ctx, gqs_stats* out);

/* Per-role cycle counters of the last sort, filled only by a library built with -DGQS_PROFILE
 * (zeros otherwise). Writes up to n values and returns the number written. */
int gqs_last_profile(gqs_ctx* ctx, uint64_t* out, size_t n);

/* Where the last sort's persistent kernel spent its time, on the clock of each CTA's consumer
 * leader thread (SM cycles, summed over CTAs): on-chip sorts of ranges of at most one tile (the
 * lqsort_kernel counterpart: tile wait, sort, write-out), writes of queued pivot runs, and the
 * whole consumer loop; partition_cycles is the rest of the loop: partition chunk iterations (the
 * gqsort_kernel counterpart), pipeline drains and waits for work (chunks are not timed one by
 * one, which would put a clock read on every chunk's critical path). Recorded by every build. */
typedef struct gqs_phases {
  uint64_t partition_cycles;
  uint64_t onchip_cycles;
  uint64_t fill_cycles;
  uint64_t total_cycles;
} gqs_phases;

/* The phase split of the context's last sort (waits for it if it is still running). */
gqs_status gqs_last_phases(gqs_ctx* ctx, gqs_phases* out);

/* One partition level (job depth; the root job is depth 0) of the last sort. */
typedef struct gqs_level {
  uint32_t depth;
  uint32_t part_jobs;  /* partition jobs that finished at this depth */
  uint64_t part_keys;  /* the keys they partitioned */
  uint32_t local_jobs; /* on-chip sorts of ranges at this depth */
  uint32_t reserved;
  uint64_t local_keys; /* the keys they sorted */
  double first_ms;     /* a first and the last job completion at this depth, ms after the */
  double last_ms;      /* persistent kernel started */
} gqs_level;

/* Per-level statistics of the context's last sort, the counterpart of the reference's optional
 * per-level timing (GET_DETAILED_PERFORMANCE, GPU-Quicksort_OpenCL_1.2/QuicksortMain.cpp:148,
 * 226-252): fills up to `max` rows, one per depth with any work (depths beyond 47 share the
 * last row), and returns how many. Only the profiling flavour of the library
 * (libgqs_prof.so) records them; the product library returns 0. */
int gqs_last_levels(gqs_ctx* ctx, gqs_level* out, int max);

/* Kernel variants available for a key type (gqs_variant_describe: tile, chunk, CTA size). A
 * context created with cfg.variant = -1 picks, for every sort, the variant a tuning run on the
 * GPU found fastest for that key type and size class (ceil(log2 n)) on a GPU with the nearest
 * SM count: the counterpart of the reference's size-dependent launch parameters (optp,
 * GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:831-833). gqs_set_variant fixes one variant for a key
 * type instead; gqs_get_variant returns it, or -1 while the context picks per sort (the variant a
 * sort ran with is in gqs_stats.variant). */
int gqs_variant_count(int dtype);
gqs_status gqs_variant_describe(int dtype, int variant, gqs_variant_desc* out);
gqs_status gqs_set_variant(gqs_ctx* ctx, int dtype, int variant);
int gqs_get_variant(gqs_ctx* ctx, int dtype);

const char* gqs_strerror(gqs_status s);
int gqs_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GQS_H */
