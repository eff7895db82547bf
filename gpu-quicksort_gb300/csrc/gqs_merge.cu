// Merge of two sorted runs (merge path), used by the host-pointer sort to sort an array in
// pieces while later pieces are still being copied in, then merge the sorted pieces.
//
// Each CTA produces kTile consecutive outputs. Where its output range starts and ends in the
// two runs comes from a binary search along the merge path (the split (i, j), i + j = diagonal,
// with a[i-1] <= b[j] and b[j-1] < a[i]: on equal keys the element of `a` comes first), done for
// every tile boundary at once by a first kernel (one thread each, so the dependent global loads
// of the searches overlap instead of delaying every CTA of the merge). The merge CTA stages
// both input slices in shared memory, and every thread merges kPer consecutive outputs from the
// staged slices into shared memory; the tile then leaves with coalesced stores. Keys are
// compared through the sort's order-preserving map, so float runs merge in the same order the
// sort produces (-0.0 before +0.0).
#include <cuda_runtime.h>

#include <cstdint>

#include "gqs_device.cuh"
#include "gqs_launch.h"

namespace gqs {
namespace {

constexpr int kThreads = 256;
constexpr int kPer = 8;
constexpr int kTile = kThreads * kPer;

template <class T>
__device__ __forceinline__ size_t merge_path(const typename KeyOps<T>::B* a, size_t na,
                                             const typename KeyOps<T>::B* b, size_t nb, size_t diag) {
  using Ops = KeyOps<T>;
  size_t lo = diag > nb ? diag - nb : 0, hi = diag < na ? diag : na;
  while (lo < hi) {
    const size_t mid = (lo + hi) >> 1;
    if (Ops::key(a[mid]) <= Ops::key(b[diag - 1 - mid])) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <class T>
__global__ void __launch_bounds__(256) merge_splits(const typename KeyOps<T>::B* __restrict__ a, size_t na,
                                                    const typename KeyOps<T>::B* __restrict__ b, size_t nb,
                                                    unsigned long long* __restrict__ splits, size_t nsplits) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nsplits) return;
  const size_t total = na + nb;
  const size_t diag = k * kTile < total ? k * kTile : total;
  splits[k] = merge_path<T>(a, na, b, nb, diag);
}

template <class T>
__global__ void __launch_bounds__(kThreads) merge_kernel(const typename KeyOps<T>::B* __restrict__ a, size_t na,
                                                         const typename KeyOps<T>::B* __restrict__ b, size_t nb,
                                                         const unsigned long long* __restrict__ splits,
                                                         typename KeyOps<T>::B* __restrict__ out, size_t tile0) {
  using B = typename KeyOps<T>::B;
  using Ops = KeyOps<T>;
  __shared__ B sa[kTile];  // a slice, then b slice, packed: [0, la) and [la, la + lb)
  __shared__ B so[kTile];
  const size_t total = na + nb;
  const size_t tile = tile0 + blockIdx.x;
  const size_t d0 = tile * kTile;
  if (d0 >= total) return;
  const size_t d1 = d0 + kTile < total ? d0 + kTile : total;
  const size_t a0 = splits[tile], a1 = splits[tile + 1];
  const size_t b0 = d0 - a0, b1 = d1 - a1;
  const uint32_t la = (uint32_t)(a1 - a0), lb = (uint32_t)(b1 - b0), n = la + lb;
  {
    // element i of the staged tile is a[a0 + i] for i < la, else b[b0 + i - la]; every thread
    // issues all its loads before its first shared store, so they are in flight together
    B v[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const uint32_t i = threadIdx.x + (uint32_t)u * kThreads;
      v[u] = i < la ? a[a0 + i] : (i < n ? b[b0 + (i - la)] : B(0));
    }
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const uint32_t i = threadIdx.x + (uint32_t)u * kThreads;
      if (i < n) sa[i] = v[u];
    }
  }
  __syncthreads();
  // this thread's outputs [o0, o1) of the tile: split the staged slices along the same path
  const uint32_t o0 = threadIdx.x * kPer < n ? threadIdx.x * kPer : n;
  const uint32_t o1 = o0 + kPer < n ? o0 + kPer : n;
  uint32_t lo = o0 > lb ? o0 - lb : 0, hi = o0 < la ? o0 : la;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (Ops::key(sa[mid]) <= Ops::key(sa[la + o0 - 1 - mid])) lo = mid + 1;
    else hi = mid;
  }
  uint32_t i = lo, j = o0 - lo;
  for (uint32_t o = o0; o < o1; ++o) {
    const bool take_a = j >= lb || (i < la && Ops::key(sa[i]) <= Ops::key(sa[la + j]));
    so[o] = take_a ? sa[i++] : sa[la + j++];
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < kPer; ++u) {
    const uint32_t k = threadIdx.x + (uint32_t)u * kThreads;
    if (k < n) out[d0 + k] = so[k];
  }
}

template <class T>
cudaError_t launch_plan(const void* a, size_t na, const void* b, size_t nb, unsigned long long* splits,
                        cudaStream_t s) {
  using B = typename KeyOps<T>::B;
  const size_t total = na + nb;
  if (total == 0) return cudaSuccess;
  const size_t words = (total + kTile - 1) / kTile + 1;
  merge_splits<T><<<(unsigned)((words + 255) / 256), 256, 0, s>>>(static_cast<const B*>(a), na,
                                                                  static_cast<const B*>(b), nb, splits, words);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_tiles(const void* a, size_t na, const void* b, size_t nb, void* out,
                         const unsigned long long* splits, size_t t0, size_t t1, cudaStream_t s) {
  using B = typename KeyOps<T>::B;
  const size_t tiles = (na + nb + kTile - 1) / kTile;
  if (t1 > tiles) t1 = tiles;
  if (t0 >= t1) return cudaSuccess;
  merge_kernel<T><<<(unsigned)(t1 - t0), kThreads, 0, s>>>(static_cast<const B*>(a), na, static_cast<const B*>(b), nb,
                                                          splits, static_cast<B*>(out), t0);
  return cudaGetLastError();
}

}  // namespace

size_t merge_split_words(size_t total) { return (total + kTile - 1) / kTile + 1; }
size_t merge_tile_keys() { return kTile; }

cudaError_t merge_plan(int dtype, const void* a, size_t na, const void* b, size_t nb, unsigned long long* splits,
                       cudaStream_t s) {
  switch (dtype) {
    case DT_U32: return launch_plan<uint32_t>(a, na, b, nb, splits, s);
    case DT_F32: return launch_plan<float>(a, na, b, nb, splits, s);
    case DT_F64: return launch_plan<double>(a, na, b, nb, splits, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t merge_tiles(int dtype, const void* a, size_t na, const void* b, size_t nb, void* out,
                        const unsigned long long* splits, size_t t0, size_t t1, cudaStream_t s) {
  switch (dtype) {
    case DT_U32: return launch_tiles<uint32_t>(a, na, b, nb, out, splits, t0, t1, s);
    case DT_F32: return launch_tiles<float>(a, na, b, nb, out, splits, t0, t1, s);
    case DT_F64: return launch_tiles<double>(a, na, b, nb, out, splits, t0, t1, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t merge_runs(int dtype, const void* a, size_t na, const void* b, size_t nb, void* out,
                       unsigned long long* splits, cudaStream_t s) {
  cudaError_t e = merge_plan(dtype, a, na, b, nb, splits, s);
  if (e == cudaSuccess) e = merge_tiles(dtype, a, na, b, nb, out, splits, 0, merge_split_words(na + nb), s);
  return e;
}

}  // namespace gqs
