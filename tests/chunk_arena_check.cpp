// Randomised check of ChunkArena (the server's slab sub-allocator): ranges are
// granule-aligned, inside their chunk and disjoint; free lists plus live ranges
// tile every chunk with no two free ranges adjacent; a chunk leaves the arena
// exactly when its last range is given back.  Chunk memory is host memory here.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <vector>

#include "arena.h"

using fpcc::ChunkArena;

static int fail(const char* what, long a = 0, long b = 0) {
  std::printf("FAIL %s %ld %ld\n", what, a, b);
  return 1;
}

int main(int argc, char** argv) {
  const unsigned seed = argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u;
  const size_t G = 256, CH = 1 << 20;
  std::mt19937 rng(seed);
  ChunkArena ar(G);
  std::map<char*, size_t> live;          // start -> rounded length
  std::vector<char*> owned;              // chunk memory handed to the arena
  long returned = 0;
  for (int step = 0; step < 4000; step++) {
    const bool alloc = live.empty() || (rng() % 100) < 55;
    if (alloc) {
      const size_t bytes = 1 + rng() % (CH / 4);
      void* p = ar.take(bytes);
      if (!p) {
        char* base = static_cast<char*>(std::malloc(CH));
        owned.push_back(base);
        p = ar.add_chunk(base, CH, bytes);
        if (p != base) return fail("add_chunk did not return its base");
      }
      live[static_cast<char*>(p)] = ar.round(bytes);
    } else {
      auto it = live.begin();
      std::advance(it, rng() % live.size());
      bool found = false;
      void* empty = ar.give(it->first, it->second, &found);
      if (!found) return fail("range not found in any chunk");
      live.erase(it);
      if (empty) {
        returned++;
        for (auto& kv : live)
          if (kv.first >= static_cast<char*>(empty) && kv.first < static_cast<char*>(empty) + CH)
            return fail("chunk returned while a range is live");
      }
    }
    // invariants over every chunk still held (every few steps)
    if (step % 8) continue;
    for (const auto& c : ar.chunks()) {
      size_t used = 0, freeb = 0, prev_end = 0;
      std::map<size_t, size_t> all(c.free.begin(), c.free.end());
      for (auto& kv : live)
        if (kv.first >= c.base && kv.first < c.base + c.size) {
          const size_t off = (size_t)(kv.first - c.base);
          if (off % G) return fail("unaligned range", (long)off);
          if (off + kv.second > c.size) return fail("range beyond its chunk", (long)off, (long)kv.second);
          used += kv.second;
          if (all.count(off)) return fail("live range starts a free range", (long)off);
          all[off] = kv.second;
        }
      for (auto& kv : c.free) freeb += kv.second;
      if (used != c.used) return fail("used bytes", (long)used, (long)c.used);
      if (used + freeb != c.size) return fail("chunk not tiled", (long)(used + freeb), (long)c.size);
      for (auto& kv : all) {
        if (kv.first != prev_end) return fail("gap or overlap at", (long)kv.first, (long)prev_end);
        prev_end = kv.first + kv.second;
      }
      for (auto it = c.free.begin(); it != c.free.end(); ++it) {
        auto nx = std::next(it);
        if (nx != c.free.end() && it->first + it->second == nx->first) return fail("free ranges not merged");
      }
    }
  }
  while (!live.empty()) {
    bool found = false;
    void* empty = ar.give(live.begin()->first, live.begin()->second, &found);
    if (!found) return fail("range not found at the end");
    live.erase(live.begin());
    if (empty) returned++;
  }
  if (!ar.chunks().empty()) return fail("chunks left after every range was given back", (long)ar.chunks().size());
  if (returned != (long)owned.size()) return fail("chunks returned", returned, (long)owned.size());
  for (char* p : owned) std::free(p);
  std::printf("ok chunks=%zu\n", owned.size());
  return 0;
}
