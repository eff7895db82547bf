// A C++ caller of the drop-in entry, written the way the reference's driver calls its sort:
// big_test<T> fills an array with the shuffled sequence 1..N, sorts it with GPUQSort<T>(ctx,
// size, d, dn) and checks it against std::sort (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:
// 1114-1138, 1192-1194), for uint32, float and double in turn. Built with plain g++ against
// include/gqs/Quicksort.h and libgqs.so by tests/test_cxx_dropin.py.
//
// Exit status: 0 when every sort matches std::sort; 3 when no GB300 is present (the context
// cannot be created, as on the CPU-only container); 1 on a mismatch or a failed call.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

#include "gqs/Quicksort.h"

namespace {

template <class T>
bool big_test(gqs_ctx* ctx, size_t n, const char* name) {
  std::vector<T> d(n), dn(n);
  for (size_t i = 0; i < n; ++i) d[i] = (T)(i + 1);
  uint64_t s = 0x9E3779B97F4A7C15ull ^ n;  // a fixed shuffle (Fisher-Yates with splitmix64)
  for (size_t i = n - 1; i > 0; --i) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    std::swap(d[i], d[z % (i + 1)]);
  }
  std::vector<T> ref(d);
  std::sort(ref.begin(), ref.end());
  const gqs_status st = gqs::GPUQSort<T>(ctx, n, d.data(), dn.data());
  if (st != GQS_OK) {
    std::printf("%s: GPUQSort failed: %s\n", name, gqs_strerror(st));
    return false;
  }
  const bool ok = d == ref;
  std::printf("%s: %zu keys, verifying: %s\n", name, n, ok ? "true" : "false");
  return ok;
}

}  // namespace

int main(int argc, char** argv) {
  const size_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : (size_t)1 << 22;
  try {
    gqs::Context ctx(0);
    bool ok = big_test<uint32_t>(ctx.get(), n, "uint") && big_test<float>(ctx.get(), n, "float") &&
              big_test<double>(ctx.get(), n, "double");
    return ok ? 0 : 1;
  } catch (const std::runtime_error& e) {
    std::printf("no usable device: %s\n", e.what());
    return 3;
  }
}
