// GraphSort: one replayable sort of many segments, captured once per (key type, variant) as a
// CUDA graph. Used by the batch API (gqs_batch.cu) and by every lane of the server
// (gqs_serve.cu).
//
// The graph holds the whole sort: copy of the segment table from pinned host memory, clearing
// of the status block and ticket ring, the seed kernel, the persistent kernel, and the copy of
// the status block back to pinned host memory. The segment count is the table's first word,
// so one graph replays batches of any shape up to the capacities it was built for; replay is
// one cudaGraphLaunch.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "gqs.h"
#include "gqs_device.cuh"
#include "gqs_launch.h"

namespace gqs {

constexpr int kMaxVariantsPerType = 16;

class GraphSort {
 public:
  GraphSort() = default;
  ~GraphSort();
  GraphSort(const GraphSort&) = delete;
  GraphSort& operator=(const GraphSort&) = delete;

  // Sizes the job records and ticket ring for batches of up to max_keys keys in up to max_segs
  // segments, for every key type and variant. `pairs`: the table holds (start, end) per segment
  // instead of nseg + 1 boundaries. The current device must be `device`.
  gqs_status init(int device, int num_sms, size_t max_keys, size_t max_segs, bool pairs, uint32_t timeout_ms);

  // The key arena and its scratch (same length, `arena_bytes` each); segment bounds are element
  // indices into them. Changing the arena drops the captured graphs.
  void set_arena(void* keys, void* scratch, size_t arena_bytes);

  // Pinned host segment table after the count word: nseg + 1 boundaries, or 2 * nseg bounds.
  unsigned long long* table() const { return hdr_host_ + 1; }
  size_t max_segments() const { return max_segs_; }
  size_t max_keys() const { return max_keys_; }

  // Checks the table on the host: every segment inside the arena, at most max_keys keys.
  gqs_status validate(int dtype, size_t nseg, unsigned long long* keys_out) const;

  // Enqueues one replay of the (dtype, variant) graph for the first nseg table entries on
  // `stream`; the table must not change until the replay has finished (wait on end_event()).
  gqs_status launch(int dtype, int variant, size_t nseg, cudaStream_t stream);
  cudaEvent_t begin_event() const { return ev_begin_; }
  cudaEvent_t end_event() const { return ev_end_; }

  // Status and statistics of the last replay; call after end_event() has completed.
  gqs_stats result() const;

  // Resident CTAs per SM for a variant (0: it cannot run).
  int blocks_per_sm(int dtype, int variant);

 private:
  gqs_status capture(int dtype, int variant);
  void drop_graphs();

  int device_ = 0, num_sms_ = 0;
  size_t max_keys_ = 0, max_segs_ = 0, table_words_ = 0;
  bool pairs_ = false;
  uint32_t timeout_ms_ = 4000;
  void* keys_ = nullptr;
  void* scratch_ = nullptr;
  size_t arena_bytes_ = 0;
  Job* jobs_ = nullptr;
  size_t job_cap_ = 0;
  unsigned long long* ring_ = nullptr;
  size_t ring_len_ = 0;
  Queue* q_ = nullptr;
  Queue* q_host_ = nullptr;
  unsigned long long* hdr_dev_ = nullptr;
  unsigned long long* hdr_host_ = nullptr;
  cudaStream_t cap_stream_ = nullptr;
  cudaEvent_t ev_begin_ = nullptr, ev_end_ = nullptr;
  cudaGraph_t graph_[3][kMaxVariantsPerType] = {};
  cudaGraphExec_t exec_[3][kMaxVariantsPerType] = {};
  int bps_[3][kMaxVariantsPerType] = {};
  int last_dtype_ = 0, last_variant_ = 0;
};

}  // namespace gqs
