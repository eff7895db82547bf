// gqs_sort_u32_noalloc: the uint32 device-pointer sort for callers that cannot allocate
// device memory when they sort.
//
// Some callers must not call cudaMalloc at sort time: hosts that hand all device memory to
// their own pool at start-up and forbid allocations afterwards, and latency-critical code
// that cannot afford cudaMalloc's implicit device synchronisation or the risk of it failing
// mid-run. They also cannot create a gqs_ctx, whose pools are cudaMalloc'd. This entry point
// runs the same seed + persistent sort kernels as gqs_sort_u32_dev, but every byte of scratch
// (the second key buffer, job records, ticket ring and status block) lives in one file-scope
// static __device__ array below, which every GPU that loads the library holds until exit.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "gqs.h"
#include "gqs_device.cuh"
#include "gqs_launch.h"

namespace {

// Geometry of kernel variant 0 for uint32 keys, which this entry point always runs.
constexpr size_t kTile = 12288, kTiny = 256, kChunk = 8192;

constexpr size_t kMaxKeys = GQS_NOALLOC_MAX_KEYS;
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
// Same bounds as the context pools: one record per disjoint range longer than kTiny or kTile
// keys (with room for uneven pivots), fill jobs, one root, and slack.
constexpr size_t kJobs = kMaxKeys / kTiny + 16 * (kMaxKeys / kTile) + kMaxKeys / 32768 + 2 + 4096;
constexpr size_t pow2_at_least(size_t x) {
  size_t r = 1;
  while (r < x) r <<= 1;
  return r;
}
constexpr size_t kRing = pow2_at_least(2 * (kMaxKeys / kChunk) + kMaxKeys / kTiny + kMaxKeys / 32768 + 2 + 65536);

constexpr size_t kOffKeys = 0;
constexpr size_t kOffJobs = align256(kOffKeys + kMaxKeys * sizeof(uint32_t));
constexpr size_t kOffRing = align256(kOffJobs + kJobs * sizeof(gqs::Job));
constexpr size_t kOffQueue = align256(kOffRing + kRing * sizeof(unsigned long long));
constexpr size_t kScratchBytes = align256(kOffQueue + sizeof(gqs::Queue));

// The scratch. In host code this name is only a stand-in for the symbol, never a device
// address: the address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;

struct DeviceSetup {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  int grid = 0;
};

std::mutex g_mu;
DeviceSetup g_setup[kMaxDevices];

// First call on a device (with that device current): resolve the scratch address, set the
// kernel's shared-memory attribute and size the grid. None of these allocate.
gqs_status setup_device(int dev, DeviceSetup** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceSetup& s = g_setup[dev];
  if (!s.ready) {
    int major = 0, minor = 0, sms = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      (void)cudaGetLastError();
      return GQS_ERR_CUDA;
    }
    if (major != 10 || minor != 3) return GQS_ERR_NO_DEVICE;
    const gqs::VariantInfo vi = gqs::variant_info(gqs::DT_U32, 0);
    if ((size_t)vi.tile != kTile || (size_t)vi.tiny != kTiny || (size_t)vi.chunk != kChunk) return GQS_ERR_INTERNAL;
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
      (void)cudaGetLastError();
      return GQS_ERR_CUDA;
    }
    const int per_sm = gqs::variant_prepare(gqs::DT_U32, 0);
    if (per_sm <= 0) return GQS_ERR_NO_DEVICE;
    s.scratch = static_cast<unsigned char*>(p);
    s.grid = sms * per_sm;
    s.ready = true;
  }
  *out = &s;
  return GQS_OK;
}

}  // namespace

extern "C" gqs_status gqs_sort_u32_noalloc(uint32_t* d, size_t n, void* stream) {
  if (n > kMaxKeys) return GQS_ERR_INVALID;  // larger than the static scratch
  if (n <= 1) return (d || n == 0) ? GQS_OK : GQS_ERR_INVALID;
  if (!d || (reinterpret_cast<uintptr_t>(d) & 3u) != 0) return GQS_ERR_INVALID;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    (void)cudaGetLastError();
    return GQS_ERR_NO_DEVICE;
  }
  DeviceSetup* s = nullptr;
  gqs_status st = setup_device(dev, &s);
  if (st != GQS_OK) return st;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  gqs::Queue* q = reinterpret_cast<gqs::Queue*>(s->scratch + kOffQueue);
  unsigned long long* ring = reinterpret_cast<unsigned long long*>(s->scratch + kOffRing);
  // The array keeps the previous call's contents: the status block and the ticket ring must
  // start at zero (job records are only read through published tickets).
  if (cudaMemsetAsync(q, 0, sizeof(gqs::Queue), cs) != cudaSuccess ||
      cudaMemsetAsync(ring, 0, kRing * sizeof(unsigned long long), cs) != cudaSuccess) {
    (void)cudaGetLastError();
    return GQS_ERR_CUDA;
  }
  gqs::LaunchParams p{};
  p.d = d;
  p.dn = s->scratch + kOffKeys;
  p.jobs = reinterpret_cast<gqs::Job*>(s->scratch + kOffJobs);
  p.q = q;
  p.tmap = ring;
  p.capacity = (uint32_t)kJobs;
  p.tmask = (uint32_t)(kRing - 1);
  p.timeout_ns = 4000ull * 1000000ull;
  p.offsets = nullptr;
  p.n = n;
  p.nseg = 1;
  p.variant = 0;
  p.grid = s->grid;
  p.stream = cs;
  if (gqs::launch_sort(gqs::DT_U32, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return GQS_ERR_CUDA;
  }
  uint32_t dev_status = 0;
  unsigned long long done = 0, total = 0;
  if (cudaMemcpyAsync(&dev_status, &q->error, sizeof(dev_status), cudaMemcpyDeviceToHost, cs) != cudaSuccess ||
      cudaMemcpyAsync(&done, &q->done, sizeof(done), cudaMemcpyDeviceToHost, cs) != cudaSuccess ||
      cudaMemcpyAsync(&total, &q->total, sizeof(total), cudaMemcpyDeviceToHost, cs) != cudaSuccess ||
      cudaStreamSynchronize(cs) != cudaSuccess) {
    (void)cudaGetLastError();
    return GQS_ERR_CUDA;
  }
  if (dev_status != 0) return (gqs_status)dev_status;
  return done == total ? GQS_OK : GQS_ERR_INTERNAL;
}
