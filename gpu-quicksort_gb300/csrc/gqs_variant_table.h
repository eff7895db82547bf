// Kernel variants per key type: Cfg<T, consumer warps, tile keys (the partition -> on-chip
// sort switch), chunk keys (keys per consumer thread = chunk / (32 * consumer warps)),
// stages, keys per lane of the largest register sort>.
// The build compiles gqs_variant_tu.cu once per entry; a context picks one per call from the
// tuning table (gqs_tuning.h) by key type and size, and the batch autotuner times them all.
// Variant 6 halves variant 0's chunk, so that small sorts spread each level over more CTAs.
#pragma once
#define GQS_VARIANTS_U32(X)                                  \
  X(u32, 0, uint32_t, 16, 12288, 8192, 3, 8)           \
  X(u32, 1, uint32_t, 24, 12288, 6144, 3, 8)           \
  X(u32, 2, uint32_t, 16, 8192, 8192, 4, 8)            \
  X(u32, 3, uint32_t, 16, 16384, 4096, 3, 8)           \
  X(u32, 4, uint32_t, 8, 12288, 4096, 3, 8)            \
  X(u32, 5, uint32_t, 8, 4096, 2048, 4, 8)            \
  X(u32, 6, uint32_t, 16, 12288, 4096, 4, 8)
#define GQS_VARIANTS_F32(X)                                  \
  X(f32, 0, float, 16, 12288, 8192, 3, 8)              \
  X(f32, 1, float, 24, 12288, 6144, 3, 8)              \
  X(f32, 2, float, 16, 8192, 8192, 4, 8)               \
  X(f32, 3, float, 16, 16384, 4096, 3, 8)              \
  X(f32, 4, float, 8, 12288, 4096, 3, 8)               \
  X(f32, 5, float, 8, 4096, 2048, 4, 8)               \
  X(f32, 6, float, 16, 12288, 4096, 4, 8)
#define GQS_VARIANTS_F64(X)                                  \
  X(f64, 0, double, 16, 6144, 4096, 3, 4)              \
  X(f64, 1, double, 24, 6144, 3072, 3, 4)              \
  X(f64, 2, double, 16, 4096, 4096, 4, 4)              \
  X(f64, 3, double, 16, 8192, 2048, 3, 4)              \
  X(f64, 4, double, 8, 6144, 2048, 3, 4)               \
  X(f64, 5, double, 8, 2048, 1024, 4, 4)              \
  X(f64, 6, double, 16, 6144, 2048, 4, 4)
// Packed (key, value) words of the pair sort: the f64 geometry with an identity key map.
#define GQS_VARIANTS_U64(X)                                  \
  X(u64, 0, uint64_t, 16, 6144, 4096, 3, 4)            \
  X(u64, 1, uint64_t, 24, 6144, 3072, 3, 4)            \
  X(u64, 2, uint64_t, 16, 4096, 4096, 4, 4)            \
  X(u64, 3, uint64_t, 16, 8192, 2048, 3, 4)            \
  X(u64, 4, uint64_t, 8, 6144, 2048, 3, 4)             \
  X(u64, 5, uint64_t, 8, 2048, 1024, 4, 4)            \
  X(u64, 6, uint64_t, 16, 6144, 2048, 4, 4)
#define GQS_VARIANT_COUNT 7
