// Internal launch interface between the C ABI (gqs_capi.cu, gqs_batch.cu) and the
// translation units that instantiate the kernels (gqs_variant_tu.cu, one per variant).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace gqs {

struct Job;
struct Queue;

// DT_U64 is internal: the packed words of the pair sort (gqs_sort_pairs_*).
enum DType : int { DT_U32 = 0, DT_F32 = 1, DT_F64 = 2, DT_U64 = 3 };

struct VariantInfo {
  int ncw;         // consumer warps per CTA
  int threads;     // threads per CTA (consumers + producer + completer)
  int tile;        // keys sorted on chip by one local job (the gqsort -> lqsort switch)
  int chunk;       // keys per staged partition chunk
  int kpt;         // keys per consumer thread per chunk
  int stages;      // chunks in flight per CTA
  int tiny;        // keys sorted in registers by one warp
  size_t smem;     // dynamic shared memory per CTA
  const char* name;
};

struct LaunchParams {
  void* d;
  void* dn;
  Job* jobs;
  Queue* q;
  unsigned long long* tmap;  // ticket ring, zeroed before the sort
  uint32_t capacity;
  uint32_t tmask;
  unsigned long long timeout_ns;
  const unsigned long long* offsets;  // nseg + 1 device offsets, or null for one segment [0, n)
  unsigned long long n;               // keys when offsets is null; else the bound of every offset
  uint32_t nseg;                      // segments (with nseg_dev: the most the launch may see)
  const unsigned long long* nseg_dev; // optional: segment count read on the device (replayable graphs)
  uint32_t pairs;                     // 1: offsets holds (start, end) per segment, 2 * nseg entries
  uint32_t from_dn;                   // 1: the segments' keys are in dn (buckets of a top split)
  int variant;
  int grid;
  cudaStream_t stream;
  cudaEvent_t ev_begin;  // optional: recorded around the persistent kernel
  cudaEvent_t ev_end;
  unsigned long long check_n;  // 0, or a tighter bound on key indices for -DGQS_CHECK builds' tests
};

// Launches `kernel`; with `early`, as a programmatic dependent launch: the grid may start while
// the kernel before it in the stream finishes, and must call pdl_wait() before it reads anything
// that kernel wrote. Only for a kernel whose predecessor in the stream is a kernel.
template <class... KArgs, class... Args>
inline cudaError_t launch_kernel(bool early, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                 cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute at[1];
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  if (early) {
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Per key type (defined in gqs_sort_dispatch.cu).
#define GQS_DECLARE_TYPE(S)                         \
  int variant_count_##S();                          \
  VariantInfo variant_info_##S(int v);              \
  int variant_prepare_##S(int v);                   \
  cudaError_t launch_##S(const LaunchParams& p);
GQS_DECLARE_TYPE(u32)
GQS_DECLARE_TYPE(f32)
GQS_DECLARE_TYPE(f64)
GQS_DECLARE_TYPE(u64)
#undef GQS_DECLARE_TYPE

// Dispatch by key type (defined in gqs_capi.cu).
int variant_count(int dtype);
VariantInfo variant_info(int dtype, int v);
// Sets the shared-memory attribute and returns the resident CTAs per SM (0 if it cannot run).
int variant_prepare(int dtype, int v);
cudaError_t launch_sort(int dtype, const LaunchParams& p);
// Merges sorted runs a[0, na) and b[0, nb) of key type dtype into out (defined in gqs_merge.cu);
// `splits` is device scratch of merge_split_words(na + nb) words. The output is made in tiles
// of merge_tile_keys() keys: merge_plan finds where every tile starts in a and b, then
// merge_tiles writes tiles [t0, t1) (several launches may cover the tiles in turn, so that
// the first part of the output can leave while the rest is merged); merge_runs does both.
size_t merge_split_words(size_t total);
size_t merge_tile_keys();
cudaError_t merge_plan(int dtype, const void* a, size_t na, const void* b, size_t nb, unsigned long long* splits,
                       cudaStream_t s);
cudaError_t merge_tiles(int dtype, const void* a, size_t na, const void* b, size_t nb, void* out,
                        const unsigned long long* splits, size_t t0, size_t t1, cudaStream_t s);
cudaError_t merge_runs(int dtype, const void* a, size_t na, const void* b, size_t nb, void* out,
                       unsigned long long* splits, cudaStream_t s);

// Top split of a plain sort of n keys (defined in gqs_split.cu): picks K - 1 splitters from
// sorted samples of d, counts every key's bucket per CTA, scans the counts into bucket offsets
// (segs, K + 1 entries) and scatters the keys into dn bucket by bucket. The buckets are then
// sorted as segments whose keys are in dn. `scratch` holds split_scratch_bytes(dtype, n) bytes.
struct SplitPlan {
  uint32_t k;      // buckets (a power of two, 2 .. 1024)
  uint32_t lg;     // log2 k
  uint32_t ctas;   // CTAs of the count and scatter kernels
  uint32_t samples;
};
bool split_plan(int dtype, size_t n, int tile, int sms, SplitPlan* plan);
size_t split_scratch_bytes(const SplitPlan& plan);
cudaError_t split_launch(int dtype, const SplitPlan& plan, const void* d, void* dn, size_t n, void* scratch,
                         unsigned long long** segs, Queue* q, cudaStream_t s);

}  // namespace gqs
