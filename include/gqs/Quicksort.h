// C++ mirror of the reference's templated sort entry over the gqs C ABI.
//
// The reference declares `template <class T> void GPUQSort(OCLResources* pOCL, size_t size, T* d, T* dn)`
// for T in {uint, float, double} (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:835-836, kernel handles
// per type at QuicksortMain.cpp:712-724) and calls it as GPUQSort(&myOCL, arraySize, pArray, pArrayCopy)
// (QuicksortMain.cpp:1114). Here the OCLResources handle becomes a gqs_ctx, the result still lands
// in `d`, and the function returns a status instead of void (the reference reports errors through
// assert/exit, GPU-Quicksort_OpenCL_1.2/OpenCLUtils.h:41-61).
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>

#include "../gqs.h"

namespace gqs {

template <class T>
gqs_status GPUQSort(gqs_ctx* ctx, size_t size, T* d, T* dn);

template <>
inline gqs_status GPUQSort<uint32_t>(gqs_ctx* ctx, size_t size, uint32_t* d, uint32_t* dn) {
  return gqs_sort_u32(ctx, d, dn, size);
}
template <>
inline gqs_status GPUQSort<float>(gqs_ctx* ctx, size_t size, float* d, float* dn) {
  return gqs_sort_f32(ctx, d, dn, size);
}
template <>
inline gqs_status GPUQSort<double>(gqs_ctx* ctx, size_t size, double* d, double* dn) {
  return gqs_sort_f64(ctx, d, dn, size);
}

// Same sort on buffers already in device memory (dn: device scratch of `size` keys, or nullptr).
template <class T>
gqs_status GPUQSortDevice(gqs_ctx* ctx, size_t size, T* d, T* dn, void* stream = nullptr);

template <>
inline gqs_status GPUQSortDevice<uint32_t>(gqs_ctx* ctx, size_t size, uint32_t* d, uint32_t* dn, void* stream) {
  return gqs_sort_u32_dev(ctx, d, dn, size, stream);
}
template <>
inline gqs_status GPUQSortDevice<float>(gqs_ctx* ctx, size_t size, float* d, float* dn, void* stream) {
  return gqs_sort_f32_dev(ctx, d, dn, size, stream);
}
template <>
inline gqs_status GPUQSortDevice<double>(gqs_ctx* ctx, size_t size, double* d, double* dn, void* stream) {
  return gqs_sort_f64_dev(ctx, d, dn, size, stream);
}

// Owning handle for a context (the role of the reference's OCLResources).
class Context {
 public:
  explicit Context(int device = 0, const gqs_config* cfg = nullptr) {
    gqs_status st = gqs_create(&ctx_, device, cfg);
    if (st != GQS_OK) throw std::runtime_error(gqs_strerror(st));
  }
  ~Context() { gqs_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  gqs_ctx* get() const { return ctx_; }

 private:
  gqs_ctx* ctx_ = nullptr;
};

}  // namespace gqs
