// The fastest kernel variant per (SM count, key type, size class), the counterpart of the
// reference's size-dependent launch parameters (optp, GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:
// 831-833). A context created with variant -1 looks up every sort here by the device's SM count
// and ceil(log2 n); rows are written by gpu-quicksort_gb300/tune_variants.py from timed sorts.
// Rows below: NVIDIA GB300, 152 SMs, median of 7 sorts per variant and size.
#pragma once

namespace gqs {

struct TuneRow {
  int sms;      // SMs of the GPU the row was measured on
  int dtype;    // DT_U32, DT_F32, DT_F64, DT_U64 (the packed pairs)
  int log2n;    // size class: n in (2^(log2n - 1), 2^log2n]
  int variant;  // fastest variant
};

constexpr TuneRow kTuneRows[] = {
    {152, 0, 10, 6},
    {152, 0, 11, 3},
    {152, 0, 12, 2},
    {152, 0, 13, 1},
    {152, 0, 14, 1},
    {152, 0, 15, 3},
    {152, 0, 16, 0},
    {152, 0, 17, 3},
    {152, 0, 18, 3},
    {152, 0, 19, 0},
    {152, 0, 20, 6},
    {152, 0, 21, 0},
    {152, 0, 22, 0},
    {152, 0, 23, 0},
    {152, 0, 24, 0},
    {152, 0, 25, 0},
    {152, 0, 26, 0},
    {152, 0, 27, 0},
    {152, 0, 28, 0},
    {152, 0, 29, 0},
    {152, 1, 10, 3},
    {152, 1, 11, 2},
    {152, 1, 12, 1},
    {152, 1, 13, 1},
    {152, 1, 14, 6},
    {152, 1, 15, 6},
    {152, 1, 16, 0},
    {152, 1, 17, 6},
    {152, 1, 18, 1},
    {152, 1, 19, 6},
    {152, 1, 20, 3},
    {152, 1, 21, 6},
    {152, 1, 22, 0},
    {152, 1, 23, 0},
    {152, 1, 24, 0},
    {152, 1, 25, 0},
    {152, 1, 26, 0},
    {152, 1, 27, 0},
    {152, 1, 28, 0},
    {152, 1, 29, 0},
    {152, 2, 10, 1},
    {152, 2, 11, 1},
    {152, 2, 12, 1},
    {152, 2, 13, 6},
    {152, 2, 14, 1},
    {152, 2, 15, 5},
    {152, 2, 16, 2},
    {152, 2, 17, 0},
    {152, 2, 18, 0},
    {152, 2, 19, 3},
    {152, 2, 20, 0},
    {152, 2, 21, 3},
    {152, 2, 22, 0},
    {152, 2, 23, 0},
    {152, 2, 24, 0},
    {152, 2, 25, 0},
    {152, 2, 26, 0},
    {152, 2, 27, 0},
    {152, 2, 28, 0},
    {152, 3, 10, 0},
    {152, 3, 11, 1},
    {152, 3, 12, 1},
    {152, 3, 13, 1},
    {152, 3, 14, 6},
    {152, 3, 15, 5},
    {152, 3, 16, 2},
    {152, 3, 17, 1},
    {152, 3, 18, 0},
    {152, 3, 19, 1},
    {152, 3, 20, 6},
    {152, 3, 21, 3},
    {152, 3, 22, 3},
    {152, 3, 23, 0},
    {152, 3, 24, 0},
    {152, 3, 25, 0},
    {152, 3, 26, 0},
    {152, 3, 27, 0},
    {152, 3, 28, 0},
};

}  // namespace gqs
