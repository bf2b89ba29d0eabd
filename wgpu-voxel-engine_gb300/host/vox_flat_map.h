// vox_flat_map.h — the streaming engine's bookkeeping maps: chunk coordinates and request
// ids to entries, built for a request rate of millions of chunks per second.
#pragma once

#include <cstddef>
#include <cstdint>
#include <utility>
#include <vector>

#include "voxgpu.h"

namespace vox {

inline uint64_t mix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}
struct CoordHash {
  uint64_t operator()(const vox_chunk_coord& c) const {
    return mix64(((uint64_t)(uint32_t)c.x | ((uint64_t)(uint32_t)c.y << 32)) ^
                 mix64((uint64_t)(uint32_t)c.z + 0x9E3779B97F4A7C15ull));
  }
};
struct CoordEq {
  bool operator()(const vox_chunk_coord& a, const vox_chunk_coord& b) const {
    return a.x == b.x && a.y == b.y && a.z == b.z;
  }
};
struct IdHash {
  uint64_t operator()(uint64_t id) const { return mix64(id); }
};
struct IdEq {
  bool operator()(uint64_t a, uint64_t b) const { return a == b; }
};

// Open-addressing hash map of the engine's bookkeeping: a power-of-two table at most half
// full, linear probing with backward-shift deletion (no tombstones), each table slot
// holding an item's 64-bit hash and its index in a dense item array (a hash match is
// confirmed on the key). Erasure moves the last item into the hole. Insertion and erasure
// invalidate iterators and references to items, as std::vector's do.
template <typename K, typename V, typename Hash, typename Eq>
class FlatMap {
 public:
  struct Item {
    K first;
    V second;
  };
  using iterator = Item*;
  iterator begin() { return items_.data(); }
  iterator end() { return items_.data() + items_.size(); }
  size_t size() const { return items_.size(); }
  void reserve(size_t n) {
    size_t cap = 16;
    while (cap < 2 * n) cap <<= 1;
    if (cap > slot_.size()) rehash(cap);
    items_.reserve(n);
  }
  iterator find(const K& k) {
    if (items_.empty()) return end();
    const uint64_t hk = Hash()(k);
    for (size_t h = hk & mask_;; h = (h + 1) & mask_) {
      if (slot_[h] == kNone) return end();
      if (hash_[h] == hk && Eq()(items_[slot_[h]].first, k)) return items_.data() + slot_[h];
    }
  }
  // k must not be present
  iterator emplace(const K& k, V v) {
    if (2 * (items_.size() + 1) > slot_.size()) rehash(slot_.empty() ? 16 : 2 * slot_.size());
    const uint64_t hk = Hash()(k);
    size_t h = hk & mask_;
    while (slot_[h] != kNone) h = (h + 1) & mask_;
    hash_[h] = hk;
    slot_[h] = (uint32_t)items_.size();
    items_.push_back(Item{k, std::move(v)});
    return &items_.back();
  }
  void erase(iterator it) {
    const uint32_t idx = (uint32_t)(it - items_.data());
    size_t hole = locate(idx);
    // pull every later member of the probe run whose home is not after the hole into it
    for (size_t j = (hole + 1) & mask_; slot_[j] != kNone; j = (j + 1) & mask_) {
      if (((j - (hash_[j] & mask_)) & mask_) >= ((j - hole) & mask_)) {
        hash_[hole] = hash_[j];
        slot_[hole] = slot_[j];
        hole = j;
      }
    }
    slot_[hole] = kNone;
    const uint32_t last = (uint32_t)items_.size() - 1;
    if (idx != last) {
      slot_[locate(last)] = idx;
      items_[idx] = std::move(items_[last]);
    }
    items_.pop_back();
  }

 private:
  static constexpr uint32_t kNone = ~0u;
  // the table slot of item idx
  size_t locate(uint32_t idx) const {
    size_t h = Hash()(items_[idx].first) & mask_;
    while (slot_[h] != idx) h = (h + 1) & mask_;
    return h;
  }
  void rehash(size_t cap) {
    hash_.assign(cap, 0);
    slot_.assign(cap, kNone);
    mask_ = cap - 1;
    for (uint32_t i = 0; i < (uint32_t)items_.size(); ++i) {
      const uint64_t hk = Hash()(items_[i].first);
      size_t h = hk & mask_;
      while (slot_[h] != kNone) h = (h + 1) & mask_;
      hash_[h] = hk;
      slot_[h] = i;
    }
  }
  std::vector<uint64_t> hash_;
  std::vector<uint32_t> slot_;
  std::vector<Item> items_;
  size_t mask_ = 0;
};

}  // namespace vox
