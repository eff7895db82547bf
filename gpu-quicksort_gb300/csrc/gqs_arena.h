// The server's device-arena allocator: first fit over byte offsets [0, size), in grains of
// kArenaGrain bytes, with frees that merge with both neighbours. Host-only C++ (no CUDA), so
// that the CPU tests can exercise it directly (tests/arena_check.cpp).
#pragma once
#include <cstddef>
#include <iterator>
#include <map>

namespace gqs {

constexpr size_t kArenaGrain = 256;  // allocation granularity (bytes)

class ArenaAlloc {
 public:
  void reset(size_t size) {
    free_.clear();
    if (size) free_[0] = size;
    used_ = 0;
  }
  // The lowest free block that holds `bytes` (rounded up to the grain); false if none does.
  bool alloc(size_t bytes, size_t* off) {
    bytes = round(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const size_t rest = it->second - bytes, at = it->first + bytes;
      free_.erase(it);
      if (rest) free_[at] = rest;
      used_ += bytes;
      return true;
    }
    return false;
  }
  // Returns a block obtained from alloc with the same byte count.
  void release(size_t off, size_t bytes) {
    bytes = round(bytes);
    used_ -= bytes;
    auto next = free_.lower_bound(off);
    if (next != free_.end() && off + bytes == next->first) {
      bytes += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += bytes;
        return;
      }
    }
    free_[off] = bytes;
  }
  size_t used() const { return used_; }
  // The free blocks, offset -> length, in address order.
  const std::map<size_t, size_t>& free_blocks() const { return free_; }
  static size_t round(size_t bytes) { return (bytes + kArenaGrain - 1) / kArenaGrain * kArenaGrain; }

 private:
  std::map<size_t, size_t> free_;
  size_t used_ = 0;
};

}  // namespace gqs
