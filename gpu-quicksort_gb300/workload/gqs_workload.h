/* Seeded synthetic sort workloads (host-side, deterministic across platforms). */
#ifndef GQS_WORKLOAD_H
#define GQS_WORKLOAD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum gqs_dist {
  GQS_DIST_UNIFORM = 0,    /* u32: [0, 2^32); f32/f64: U[-1e9, 1e9] */
  GQS_DIST_SORTED = 1,     /* monotone non-decreasing */
  GQS_DIST_REVERSE = 2,    /* monotone non-increasing */
  GQS_DIST_DISTINCT16 = 3, /* 16 distinct values, picked uniformly */
  GQS_DIST_ZIPF = 4,       /* u32 only: Zipf(1.1) over 2^20 ranks, rank r -> (r+1)*2654435761 */
  GQS_DIST_GAUSSIAN = 5,   /* u32: N(2^31, 2^28) rounded and clamped; f32/f64: N(0, 1e3) */
  GQS_DIST_KAT = 6,        /* shuffled 1..n (the reference's known-answer input) */
  GQS_DIST_ALLEQUAL = 7    /* every key the same */
};

int gqs_workload_u32(int dist, uint64_t seed, size_t n, uint32_t* out);
int gqs_workload_f32(int dist, uint64_t seed, size_t n, float* out);
int gqs_workload_f64(int dist, uint64_t seed, size_t n, double* out);
uint64_t gqs_workload_segments(uint64_t seed, size_t nseg, uint64_t minlen, uint64_t maxlen,
                               uint64_t* offsets);

#ifdef __cplusplus
}
#endif
#endif
