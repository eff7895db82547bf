// Per-key-type variant tables: name, shared memory and launch of each compiled variant.
#include "gqs_variant_table.h"
#include "gqs_variants.cuh"

namespace gqs {

#define GQS_DECL(S, V, T, NCW, TILE, CHUNK, STAGES, R) \
  VariantInfo info_##S##_##V();                            \
  int prepare_##S##_##V();                                 \
  cudaError_t launch_##S##_##V(const LaunchParams& p);
GQS_VARIANTS_U32(GQS_DECL)
GQS_VARIANTS_F32(GQS_DECL)
GQS_VARIANTS_F64(GQS_DECL)
GQS_VARIANTS_U64(GQS_DECL)
#undef GQS_DECL

#define GQS_CASE_INFO(S, V, ...) \
  case V:                        \
    return info_##S##_##V();
#define GQS_CASE_PREP(S, V, ...) \
  case V:                        \
    return prepare_##S##_##V();
#define GQS_CASE_LAUNCH(S, V, ...) \
  case V:                          \
    return launch_##S##_##V(p);

#define GQS_TYPE_TABLE(S, LIST)                                        \
  int variant_count_##S() { return GQS_VARIANT_COUNT; }                \
  VariantInfo variant_info_##S(int v) {                                \
    switch (v) {                                                       \
      LIST(GQS_CASE_INFO)                                              \
      default:                                                         \
        return info_##S##_0();                                         \
    }                                                                  \
  }                                                                    \
  int variant_prepare_##S(int v) {                                     \
    switch (v) {                                                       \
      LIST(GQS_CASE_PREP)                                              \
      default:                                                         \
        return 0;                                                      \
    }                                                                  \
  }                                                                    \
  cudaError_t launch_##S(const LaunchParams& p) {                      \
    switch (p.variant) {                                               \
      LIST(GQS_CASE_LAUNCH)                                            \
      default:                                                         \
        return cudaErrorInvalidValue;                                  \
    }                                                                  \
  }

GQS_TYPE_TABLE(u32, GQS_VARIANTS_U32)
GQS_TYPE_TABLE(f32, GQS_VARIANTS_F32)
GQS_TYPE_TABLE(f64, GQS_VARIANTS_F64)
GQS_TYPE_TABLE(u64, GQS_VARIANTS_U64)

}  // namespace gqs
