// Randomised check of the serving arena's allocator (pps_arena.h) against a
// plain model: no two live blocks overlap, every block lies inside the arena
// and keeps the 256-byte alignment of the request sizes, used() and peak()
// track the live bytes, a request fails only when no free gap can take it,
// and once every block is released the arena is one free block again.
// Exit status 0 on success; the first violation is printed.
#include <cstdint>
#include <cstdio>
#include <map>
#include <random>
#include <vector>

#include "pps_arena.h"

namespace {

struct Live {
  size_t off, bytes;
};

int fail(const char* what, long step) {
  std::fprintf(stderr, "arena check failed at step %ld: %s\n", step, what);
  return 1;
}

// largest gap between live blocks (the model's view of the free space)
size_t largest_gap(const std::map<size_t, size_t>& live, size_t cap) {
  size_t at = 0, best = 0;
  for (const auto& kv : live) {
    best = std::max(best, kv.first - at);
    at = kv.first + kv.second;
  }
  return std::max(best, cap - at);
}

int run(uint64_t seed, size_t cap, int steps) {
  std::mt19937_64 rng(seed);
  pps::Arena a;
  a.reset(cap);
  std::map<size_t, size_t> live;  // offset -> bytes
  size_t used = 0, peak = 0;
  for (long step = 0; step < steps; ++step) {
    const bool do_alloc = live.empty() || (rng() % 100) < 55;
    if (do_alloc) {
      const size_t bytes = 256 * (1 + rng() % (cap / 256 / 8));
      size_t off = 0;
      const bool ok = a.alloc(bytes, &off);
      if (!ok) {
        if (largest_gap(live, cap) >= bytes) return fail("refused a request a free gap could take", step);
        continue;
      }
      if (off % 256) return fail("misaligned block", step);
      if (off + bytes > cap) return fail("block outside the arena", step);
      auto nx = live.lower_bound(off);
      if (nx != live.end() && off + bytes > nx->first) return fail("overlaps the next live block", step);
      if (nx != live.begin()) {
        auto pv = std::prev(nx);
        if (pv->first + pv->second > off) return fail("overlaps the previous live block", step);
      }
      live[off] = bytes;
      used += bytes;
      peak = std::max(peak, used);
    } else {
      auto it = live.begin();
      std::advance(it, (long)(rng() % live.size()));
      a.release(it->first, it->second);
      used -= it->second;
      live.erase(it);
    }
    if (a.used() != used) return fail("used() differs from the live bytes", step);
    if (a.peak() != peak) return fail("peak() differs from the largest live total", step);
  }
  for (const auto& kv : live) a.release(kv.first, kv.second);
  if (a.used() != 0) return fail("used() not zero after releasing everything", steps);
  size_t off = 1;
  if (!a.alloc(cap, &off) || off != 0) return fail("free blocks did not coalesce into the whole arena", steps);
  return 0;
}

}  // namespace

int main() {
  const size_t caps[] = {256 * 64, 256 * 1000, (size_t)1 << 30};
  for (uint64_t seed = 1; seed <= 20; ++seed)
    for (size_t cap : caps)
      if (run(seed, cap, 5000)) return 1;
  std::puts("arena ok");
  return 0;
}
