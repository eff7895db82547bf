// Reference-compatible benchmark command line for the gqs sort.
//
//   quicksort <iterations> <gpu|cpu> <vendor> <width> <height> <show_cl|no_show_cl>
//
// Same argument meaning as the reference's driver (GPU-Quicksort_OpenCL_1.2/QuicksortMain.cpp:
// 112-136, Full SYCL form GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:140-164): the array has
// width * height keys, the input is the shuffled sequence 1..N, every iteration sorts a fresh
// copy with GPUQSort<T> through host pointers and checks it against std::sort, and the same
// statistics are printed (QuicksortMain.cpp:518-540): time per iteration, failures, average,
// standard deviation, 3-sigma error, min, max, and the speedup over a single-core std::sort.
// As in the Full SYCL driver (QuicksortMain.cpp:1192-1194) the test runs for uint, float and
// double in turn. Only the gpu device type exists in this build (there is no CPU fallback);
// the vendor argument is accepted for compatibility and must name the GPU maker, nvidia.
// The input comes from the seeded workload generator (shuffled 1..N, identical on every
// platform) rather than std::random_shuffle, whose order is implementation-defined.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "gqs.h"
#include "gqs/Quicksort.h"
#include "gqs_workload.h"

namespace {

const char* kUsage =
    "Usage: quicksort [num test iterations] [cpu|gpu] [intel|amd|nvidia] [SurfWidth(^2 only)] "
    "[SurfHeight(^2 only)] [show_CL | no_show_CL]";

double seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void print_device_info(int dev) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
    std::printf("device %d: properties unavailable\n", dev);
    return;
  }
  std::printf("\nUsing device %d: %s (compute capability %d.%d)\n", dev, p.name, p.major, p.minor);
  std::printf("Device info:\n");
  std::printf("  multiprocessors              : %8d\n", p.multiProcessorCount);
  std::printf("  global memory                : %8.1f GiB\n", p.totalGlobalMem / 1073741824.0);
  std::printf("  L2 cache                     : %8.1f MiB\n", p.l2CacheSize / 1048576.0);
  std::printf("  shared memory per block (max): %8zu bytes\n", p.sharedMemPerBlockOptin);
  std::printf("  max threads per block        : %8d\n", p.maxThreadsPerBlock);
  std::printf("  warp size                    : %8d\n", p.warpSize);
}

template <class T>
void generate_kat(uint64_t seed, size_t n, T* out);
template <>
void generate_kat<uint32_t>(uint64_t seed, size_t n, uint32_t* out) {
  gqs_workload_u32(GQS_DIST_KAT, seed, n, out);
}
template <>
void generate_kat<float>(uint64_t seed, size_t n, float* out) {
  gqs_workload_f32(GQS_DIST_KAT, seed, n, out);
}
template <>
void generate_kat<double>(uint64_t seed, size_t n, double* out) {
  gqs_workload_f64(GQS_DIST_KAT, seed, n, out);
}

// One key type: the reference's big_test<T> (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:958-1165).
template <class T>
int big_test(gqs::Context& ctx, size_t n, unsigned iterations, const char* type_name) {
  std::printf("\n\n\n--------------------------------------------------------------------\n");
  std::printf("Allocating array size of %zu (%s)\n", n, type_name);
  std::vector<T> original(n), array(n), copy(n);
  generate_kat<T>(20260301ull, n, original.data());

  std::cout << "Sorting the regular way..." << std::endl;
  copy = original;
  double t0 = seconds();
  std::sort(copy.begin(), copy.end());
  const double std_sort_time = seconds() - t0;
  std::cout << "Time to sort: " << std_sort_time * 1000 << " ms" << std::endl;
  const std::vector<T>& verify = copy;  // the reference's verifier: std::sort of the input

  std::cout << "Sorting with GPUQSort on the gpu: " << std::endl;
  std::vector<double> times(iterations, 0.0);
  double average = 0.0;
  unsigned failures = 0;
  for (unsigned k = 0; k < iterations; ++k) {
    array = original;
    t0 = seconds();
    const gqs_status st = gqs::GPUQSort<T>(ctx.get(), n, array.data(), nullptr);
    const double t = seconds() - t0;
    if (st != GQS_OK) {
      std::cout << "GPUQSort failed: " << gqs_strerror(st) << std::endl;
      ++failures;
      continue;
    }
    std::cout << "Time to sort: " << t * 1000 << " ms" << std::endl;
    times[k] = t;
    average += t;
    std::cout << "verifying: ";
    const bool correct = std::equal(verify.begin(), verify.end(), array.begin(),
                                    [](T x, T y) { return std::memcmp(&x, &y, sizeof(T)) == 0; });
    std::cout << std::boolalpha << correct << std::endl;
    if (!correct) {
      size_t discrepancies = 0;
      for (size_t i = 0; i < n; ++i)
        if (std::memcmp(&verify[i], &array[i], sizeof(T)) != 0) ++discrepancies;
      std::cout << "num_discrepancies: " << discrepancies << std::endl;
      ++failures;
    }
  }
  std::cout << " Number of failures: " << failures << " out of " << iterations << std::endl;
  average /= iterations;
  std::cout << "Average Time: " << average * 1000 << " ms" << std::endl;
  if (iterations > 1) {
    double var = 0.0, tmin = 1e30, tmax = 0.0;
    for (double t : times) {
      var += (average - t) * (average - t);
      tmin = std::min(tmin, t);
      tmax = std::max(tmax, t);
    }
    const double sd = std::sqrt(var / (iterations - 1));
    std::cout << "Standard Deviation: " << sd * 1000 << std::endl;
    std::cout << "%error (3*stdDev)/Average: " << 3 * sd / average * 100 << "%" << std::endl;
    std::cout << "min time: " << tmin * 1000 << " ms" << std::endl;
    std::cout << "max time: " << tmax * 1000 << " ms" << std::endl;
  }
  std::cout << "Average speedup over CPU std::sort: " << std_sort_time / average << std::endl;
  std::printf("-------done--------------------------------------------------------\n");
  return failures ? 1 : 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 7) {
    std::printf("%s\n", kUsage);
    return 2;
  }
  const int iterations = std::atoi(argv[1]);
  const std::string device = argv[2], vendor = argv[3];
  const long long width = std::atoll(argv[4]), height = std::atoll(argv[5]);
  const bool show = argv[6][0] == 's';
  if (iterations <= 0 || width <= 0 || height <= 0) {
    std::printf("%s\n", kUsage);
    return 2;
  }
  if (device != "gpu") {
    std::printf("device type '%s' is not available: this build sorts on the GB300 GPU only\n", device.c_str());
    return 2;
  }
  if (vendor != "nvidia") {
    std::printf("vendor '%s' is not available: this build runs on NVIDIA GB300 (sm_103a)\n", vendor.c_str());
    return 2;
  }
  const size_t n = (size_t)width * (size_t)height;
  try {
    gqs::Context ctx(0);
    if (show) print_device_info(0);
    int rc = 0;
    rc |= big_test<uint32_t>(ctx, n, (unsigned)iterations, "uint");
    rc |= big_test<float>(ctx, n, (unsigned)iterations, "float");
    rc |= big_test<double>(ctx, n, (unsigned)iterations, "double");
    return rc;
  } catch (const std::exception& e) {
    std::printf("cannot create a gqs context: %s\n", e.what());
    return 3;
  }
}
