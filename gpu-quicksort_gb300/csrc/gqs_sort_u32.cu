// Kernel instantiations for uint32_t keys.
#include "gqs_variants.cuh"

namespace gqs {

// Cfg<T, consumer warps, tile keys, chunk keys, stages, keys per lane in the register sort, warp-phase max>
using u32_v0 = Cfg<uint32_t, 16, 16384, 4096, 4, 8, 1024>;

int variant_count_u32() { return 1; }

VariantInfo variant_info_u32(int v) {
  switch (v) {
    default:
      return VariantOps<u32_v0>::info("u32_ncw16_tile16384_chunk4096");
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
