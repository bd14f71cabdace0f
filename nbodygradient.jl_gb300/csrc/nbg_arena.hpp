// nbg_arena.hpp -- the request server's output arena allocator (host only).
//
// The server keeps every admitted request's tt / dtdq0 / dtdelements block
// in one device allocation; this first-fit allocator hands out offsets into
// it.  Units are doubles; blocks are rounded up to 32 doubles (256 bytes),
// free neighbours are merged on release, and `used` counts the rounded
// lengths handed out.
#pragma once
#include <algorithm>
#include <cstddef>
#include <iterator>
#include <map>

namespace nbg {

struct Arena {
  size_t size = 0;
  std::map<size_t, size_t> free_;  // offset -> length
  size_t used = 0;

  void init(size_t n) {
    size = n;
    free_.clear();
    if (n) free_[0] = n;
    used = 0;
  }
  // The length a request of n doubles occupies.
  static size_t round(size_t n) { return (std::max<size_t>(n, 1) + 31) / 32 * 32; }
  // Lowest-offset free block that holds n doubles; false when none does.
  bool alloc(size_t n, size_t* off) {
    n = round(n);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        *off = it->first;
        const size_t rest = it->second - n, at = it->first + n;
        free_.erase(it);
        if (rest) free_[at] = rest;
        used += n;
        return true;
      }
    }
    return false;
  }
  // Returns a block from alloc(n) (the same n).
  void release(size_t off, size_t n) {
    n = round(n);
    used -= n;
    auto it = free_.emplace(off, n).first;
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
};

}  // namespace nbg
