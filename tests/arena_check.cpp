// Randomized check of the server's arena allocator (gpu-quicksort_gb300/csrc/gqs_arena.h),
// compiled and run by tests/test_arena.py on the CPU.
//
//   arena_check <seed> <operations>
//
// Keeps every live block, and after every operation checks: live blocks never overlap and lie
// inside the arena; used() is the sum of the live blocks; live and free bytes add up to the
// arena; free blocks are disjoint, ordered and never adjacent (frees merge); an allocation fails
// only when no free block holds the request, and otherwise returns the lowest such block (first
// fit). Freeing everything leaves one free block, the whole arena. Prints "ok" and exits 0, or
// prints the first violation and exits 1.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <vector>

#include "gqs_arena.h"

namespace {

uint64_t next(uint64_t& s) {  // splitmix64
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int fail(const char* what, long op) {
  std::printf("violation at operation %ld: %s\n", op, what);
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  uint64_t seed = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1;
  const long ops = argc > 2 ? std::strtol(argv[2], nullptr, 10) : 100000;
  const size_t arena = (size_t)64 << 20;
  gqs::ArenaAlloc a;
  a.reset(arena);
  std::map<size_t, size_t> live;  // offset -> rounded length
  for (long op = 0; op < ops; ++op) {
    const uint64_t r = next(seed);
    if (live.empty() || r % 100 < 55) {
      // sizes from a byte to a few MB, log-uniform-ish
      const size_t want = (size_t)1 << (next(seed) % 23);
      const size_t bytes = 1 + next(seed) % want;
      const size_t need = gqs::ArenaAlloc::round(bytes);
      size_t first_fit = SIZE_MAX;
      for (const auto& f : a.free_blocks())
        if (f.second >= need) {
          first_fit = f.first;
          break;
        }
      size_t off = 0;
      const bool ok = a.alloc(bytes, &off);
      if (ok != (first_fit != SIZE_MAX)) return fail("allocation result differs from the free list", op);
      if (ok) {
        if (off != first_fit) return fail("not the first fitting block", op);
        live[off] = need;
      }
    } else {
      auto it = live.begin();
      std::advance(it, (long)(next(seed) % live.size()));
      a.release(it->first, it->second);
      live.erase(it);
    }
    // invariants
    size_t used = 0, end = 0;
    for (const auto& l : live) {
      if (l.first < end) return fail("live blocks overlap", op);
      end = l.first + l.second;
      if (end > arena) return fail("live block outside the arena", op);
      used += l.second;
    }
    if (used != a.used()) return fail("used() differs from the live blocks", op);
    size_t freeb = 0, fend = 0;
    bool first = true;
    for (const auto& f : a.free_blocks()) {
      if (f.second == 0) return fail("empty free block", op);
      if (!first && f.first <= fend) return fail("free blocks overlap or touch (not merged)", op);
      first = false;
      fend = f.first + f.second;
      freeb += f.second;
      auto l = live.upper_bound(f.first);
      if (l != live.begin() && std::prev(l)->first + std::prev(l)->second > f.first)
        return fail("a free block starts inside a live block", op);
      if (l != live.end() && l->first < fend) return fail("a live block starts inside a free block", op);
    }
    if (used + freeb != arena) return fail("live and free bytes do not add up to the arena", op);
  }
  for (const auto& l : live) a.release(l.first, l.second);
  if (a.used() != 0 || a.free_blocks().size() != 1 || a.free_blocks().begin()->second != arena)
    return fail("freeing everything does not restore one whole block", ops);
  std::printf("ok\n");
  return 0;
}
