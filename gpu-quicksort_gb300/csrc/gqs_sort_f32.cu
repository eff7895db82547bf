// Kernel instantiations for float keys.
#include "gqs_variants.cuh"

namespace gqs {

// Cfg<T, consumer warps, tile keys, chunk keys, stages, keys per lane in the register sort, warp-phase max>
using f32_v0 = Cfg<float, 16, 12288, 8192, 3, 8, 4096>;

int variant_count_f32() { return 1; }

VariantInfo variant_info_f32(int v) {
  switch (v) {
    default:
      return VariantOps<f32_v0>::info("f32_ncw16_tile12288_chunk8192");
  }
}

int variant_prepare_f32(int v) {
  switch (v) {
    default:
      return VariantOps<f32_v0>::prepare();
  }
}

cudaError_t launch_f32(const LaunchParams& p) {
  switch (p.variant) {
    default:
      return VariantOps<f32_v0>::launch(p);
  }
}

}  // namespace gqs
