// pps_arena.h -- the serving arena's allocator (host only, no CUDA): first
// fit over the free blocks of one device allocation, kept in offset order,
// with neighbouring free blocks merged on release.  The server sizes every
// request's block in multiples of 256 bytes, so every block it hands out
// stays 256-byte aligned.
#pragma once

#include <algorithm>
#include <cstddef>
#include <iterator>
#include <map>

namespace pps {

class Arena {
 public:
  void reset(size_t cap) {
    free_.clear();
    free_[0] = cap;
    used_ = 0;
    peak_ = 0;
  }
  bool alloc(size_t bytes, size_t* off) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes;
        const size_t at = it->first + bytes;
        free_.erase(it);
        if (rest) free_[at] = rest;
        used_ += bytes;
        peak_ = std::max(peak_, used_);
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t used() const { return used_; }
  size_t peak() const { return peak_; }

 private:
  std::map<size_t, size_t> free_;
  size_t used_ = 0, peak_ = 0;
};

}  // namespace pps
