// Kernel instantiations for uint32_t keys.
#include "gqs_variants.cuh"

namespace gqs {

// Cfg<T, consumer warps, tile keys, chunk keys, stages, keys per lane in the register sort, warp-phase max>
using u32_v0 = Cfg<uint32_t, 16, 12288, 8192, 3, 8, 4096>;

int variant_count_u32() { return 1; }

VariantInfo variant_info_u32(int v) {
  switch (v) {
    default:
      return VariantOps<u32_v0>::info("u32_ncw16_tile12288_chunk8192");
  }
}

int variant_prepare_u32(int v) {
  switch (v) {
    default:
      return VariantOps<u32_v0>::prepare();
  }
}

cudaError_t launch_u32(const LaunchParams& p) {
  switch (p.variant) {
    default:
      return VariantOps<u32_v0>::launch(p);
  }
}

}  // namespace gqs
