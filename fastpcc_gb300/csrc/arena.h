// First-fit sub-allocation of byte ranges inside chunks of device memory
// (host-side bookkeeping only: the arena keeps offsets, the caller owns the
// chunks' memory and the stream order of its use).
//
// Ranges are rounded up to a granule and carved first-fit from the chunks'
// free lists; a freed range merges with its free neighbours, and a chunk whose
// ranges are all free leaves the arena (its base is handed back to the caller
// to release).
#pragma once

#include <cstddef>
#include <iterator>
#include <map>
#include <vector>

namespace fpcc {

class ChunkArena {
 public:
  struct Chunk {
    char* base;
    size_t size, used;
    std::map<size_t, size_t> free;   // offset -> length of each free range
  };

  explicit ChunkArena(size_t granule = 256) : g_(granule) {}

  size_t round(size_t bytes) const { return (bytes + g_ - 1) / g_ * g_; }

  // A range of `bytes` (rounded) from the chunks already held, or nullptr.
  void* take(size_t bytes) {
    const size_t b = round(bytes);
    for (auto& c : chunks_)
      for (auto it = c.free.begin(); it != c.free.end(); ++it)
        if (it->second >= b) {
          const size_t off = it->first, len = it->second;
          c.free.erase(it);
          if (len > b) c.free[off + b] = len - b;
          c.used += b;
          return c.base + off;
        }
    return nullptr;
  }

  // Adds the chunk [base, base + size) and takes its first `bytes` (rounded,
  // at most size).
  void* add_chunk(void* base, size_t size, size_t bytes) {
    const size_t b = round(bytes);
    Chunk c{static_cast<char*>(base), size, b, {}};
    if (size > b) c.free[b] = size - b;
    chunks_.push_back(std::move(c));
    return base;
  }

  // Gives back [p, p + bytes).  *found tells whether p lies in a chunk of the
  // arena; the return value is the chunk's base when that chunk became empty
  // (it has left the arena), else nullptr.
  void* give(void* p, size_t bytes, bool* found) {
    const size_t b = round(bytes);
    char* q = static_cast<char*>(p);
    for (size_t i = 0; i < chunks_.size(); i++) {
      Chunk& c = chunks_[i];
      if (q < c.base || q >= c.base + c.size) continue;
      *found = true;
      size_t off = (size_t)(q - c.base), len = b;
      auto nx = c.free.lower_bound(off);
      if (nx != c.free.end() && nx->first == off + len) {   // merge with the next free range
        len += nx->second;
        nx = c.free.erase(nx);
      }
      if (nx != c.free.begin()) {                            // and with the previous one
        auto pv = std::prev(nx);
        if (pv->first + pv->second == off) {
          off = pv->first;
          len += pv->second;
          c.free.erase(pv);
        }
      }
      c.free[off] = len;
      c.used -= b;
      if (c.used == 0) {
        char* base = c.base;
        chunks_.erase(chunks_.begin() + (std::ptrdiff_t)i);
        return base;
      }
      return nullptr;
    }
    *found = false;
    return nullptr;
  }

  const std::vector<Chunk>& chunks() const { return chunks_; }

 private:
  size_t g_;
  std::vector<Chunk> chunks_;
};

}  // namespace fpcc
