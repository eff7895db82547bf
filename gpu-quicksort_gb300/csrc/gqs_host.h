// Host-side helpers shared by the context API (gqs_capi.cu), the graph-captured batch
// (gqs_batch.cu) and the server (gqs_serve.cu): pool sizing, status mapping, statistics.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "gqs.h"
#include "gqs_device.cuh"
#include "gqs_launch.h"

namespace gqs {

constexpr size_t kElemSize[4] = {4, 4, 8, 8};  // u32, f32, f64, and the internal u64

inline gqs_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return GQS_OK;
  (void)cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return GQS_ERR_NOMEM;
  return GQS_ERR_CUDA;
}

// Job records one sort can need: local jobs are disjoint ranges longer than `tiny` keys,
// partition jobs ranges longer than `tile` keys (with generous room for uneven pivots), plus
// one root per segment and the fill jobs of long pivot runs.
inline size_t job_capacity(const VariantInfo& vi, size_t n, size_t nseg) {
  return n / (size_t)vi.tiny + 16 * (n / (size_t)vi.tile) + n / 32768 + 2 * nseg + 4096;
}

// Ticket-ring entries: tickets not yet taken belong to live jobs, whose ranges are disjoint,
// so they number at most the chunks of n keys (plus one partial chunk per job) plus one per
// local job and fill chunk.
inline size_t ticket_ring(const VariantInfo& vi, size_t n, size_t nseg) {
  size_t need = 2 * (n / (size_t)vi.chunk) + n / (size_t)vi.tiny + n / 32768 + 2 * nseg + 65536;
  size_t r = 1;
  while (r < need) r <<= 1;
  return r;
}

// Statistics of a finished sort from its status block; status is GQS_ERR_INTERNAL when the
// device reported no error but did not place every key.
inline gqs_stats stats_from_queue(const Queue& q, int dtype, int variant, int grid) {
  gqs_stats s{};
  s.keys = q.total;
  s.part_keys = q.part_keys;
  s.local_keys = q.local_keys;
  s.tiny_keys = q.tiny_keys;
  s.fill_keys = q.fill_keys;
  s.chunks = q.chunks;
  s.algo_bytes = kElemSize[dtype] * 2 * (q.part_keys + q.local_keys + q.tiny_keys);
  s.part_jobs = q.part_jobs;
  s.local_jobs = q.local_jobs;
  s.fill_chunks = q.fill_jobs;
  s.max_depth = q.max_depth;
  s.status = q.error;
  s.variant = (uint32_t)variant;
  s.grid = (uint32_t)grid;
  s.threads = (uint32_t)variant_info(dtype, variant).threads;
  s.kernel_ms = -1.0;
  if (q.error == 0 && q.done != q.total) s.status = GQS_ERR_INTERNAL;
  return s;
}

// Makes `dev` current for the guard's lifetime.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// True when `device` exists and is an sm_103 GPU; fills its SM count.
inline gqs_status check_device(int device, int* num_sms) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    (void)cudaGetLastError();
    return GQS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) return GQS_ERR_INVALID;
  int major = 0, minor = 0, sms = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    (void)cudaGetLastError();
    return GQS_ERR_NO_DEVICE;
  }
  if (major != 10 || minor != 3) return GQS_ERR_NO_DEVICE;  // built for sm_103a only
  *num_sms = sms;
  return GQS_OK;
}

}  // namespace gqs
