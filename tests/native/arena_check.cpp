// Randomised check of the server's output arena allocator (nbg_arena.hpp)
// against a brute-force model: one owner word per double of the arena.
// Prints "ok" and exits 0, or prints the first failure and exits 1.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "nbg_arena.hpp"

static int fail(const char* what, long long a, long long b) {
  std::printf("FAIL %s (%lld, %lld)\n", what, a, b);
  return 1;
}

int main() {
  for (int trial = 0; trial < 20; trial++) {
    std::mt19937_64 rng(1000 + trial);
    const size_t size = 32 * (1 + rng() % 4096);
    nbg::Arena a;
    a.init(size);
    std::vector<int> owner(size, -1);  // -1: free
    struct Block { size_t off, n; };
    std::vector<Block> live;
    for (int op = 0; op < 4000; op++) {
      if (live.empty() || rng() % 3) {
        const size_t n = 1 + rng() % (size / 8 + 1);
        const size_t len = nbg::Arena::round(n);
        // the model's first fit: lowest offset starting a free run of len
        long long first = -1;
        for (size_t o = 0, run = 0; o < size; o++) {
          run = owner[o] < 0 ? run + 1 : 0;
          if (run == len) { first = (long long)(o + 1 - len); break; }
        }
        size_t off = 0;
        const bool ok = a.alloc(n, &off);
        if (ok != (first >= 0)) return fail("alloc success differs from the model", ok, first);
        if (!ok) continue;
        if ((long long)off != first) return fail("not first fit", (long long)off, first);
        if (off % 32) return fail("unaligned block", (long long)off, 0);
        for (size_t q = off; q < off + len; q++) {
          if (owner[q] >= 0) return fail("overlap", (long long)q, owner[q]);
          owner[q] = op;
        }
        live.push_back({off, n});
      } else {
        const size_t k = rng() % live.size();
        const Block b = live[k];
        live[k] = live.back();
        live.pop_back();
        for (size_t q = b.off; q < b.off + nbg::Arena::round(b.n); q++) owner[q] = -1;
        a.release(b.off, b.n);
      }
      size_t used = 0;
      for (int w : owner) used += w >= 0;
      if (used != a.used) return fail("used count", (long long)a.used, (long long)used);
      // free list: sorted, disjoint, merged (no two adjacent runs), exactly the model's free words
      size_t prev_end = 0, nfree = 0;
      bool first_run = true;
      for (auto& kv : a.free_) {
        if (!first_run && kv.first <= prev_end) return fail("free runs not merged or overlapping", kv.first, prev_end);
        for (size_t q = kv.first; q < kv.first + kv.second; q++)
          if (owner[q] >= 0) return fail("free run covers a live block", (long long)q, owner[q]);
        nfree += kv.second;
        prev_end = kv.first + kv.second;
        first_run = false;
      }
      if (nfree + used != size) return fail("free + used != size", (long long)nfree, (long long)used);
    }
    for (const Block& b : live) a.release(b.off, b.n);
    if (a.used != 0 || a.free_.size() != 1 || a.free_.begin()->first != 0 || a.free_.begin()->second != size)
      return fail("arena not whole after releasing everything", (long long)a.free_.size(), (long long)a.used);
  }
  std::printf("ok\n");
  return 0;
}
