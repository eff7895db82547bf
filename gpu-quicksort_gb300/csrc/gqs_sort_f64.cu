// Kernel instantiations for double keys.
#include "gqs_variants.cuh"

namespace gqs {

// Cfg<T, consumer warps, tile keys, chunk keys, stages, keys per lane in the register sort, warp-phase max>
using f64_v0 = Cfg<double, 16, 6144, 4096, 3, 4, 2048>;

int variant_count_f64() { return 1; }

VariantInfo variant_info_f64(int v) {
  switch (v) {
    default:
      return VariantOps<f64_v0>::info("f64_ncw16_tile6144_chunk4096");
  }
}

int variant_prepare_f64(int v) {
  switch (v) {
    default:
      return VariantOps<f64_v0>::prepare();
  }
}

cudaError_t launch_f64(const LaunchParams& p) {
  switch (p.variant) {
    default:
      return VariantOps<f64_v0>::launch(p);
  }
}

}  // namespace gqs
