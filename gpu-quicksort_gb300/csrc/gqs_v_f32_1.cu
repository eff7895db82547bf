// One kernel variant, compiled on its own so variants build in parallel.
#include "gqs_variant_table.h"
#include "gqs_variants.cuh"

namespace gqs {
#define GQS_PICK(S, V, T, NCW, TILE, CHUNK, STAGES, R, WM) \
  GQS_DEFINE_VARIANT_IF(S, V, 1, T, NCW, TILE, CHUNK, STAGES, R, WM)
GQS_VARIANTS_F32(GQS_PICK)
#undef GQS_PICK
}  // namespace gqs
