// Randomized check of vox::FlatMap (the streaming engine's bookkeeping maps) against
// std::unordered_map: inserts, finds, in-place updates and erasures over a small key space
// (long probe runs and frequent backward shifts), coordinates beyond 21 bits per axis,
// iteration and reserve. Prints "ok" and exits 0 when every operation agrees.
#include <cstdint>
#include <cstdio>
#include <random>
#include <unordered_map>

#include "vox_flat_map.h"

int main() {
  std::mt19937_64 rng(7);
  vox::FlatMap<vox_chunk_coord, int, vox::CoordHash, vox::CoordEq> fm;
  vox::FlatMap<uint64_t, int, vox::IdHash, vox::IdEq> ids;
  std::unordered_map<uint64_t, int> ref, ref_ids;
  auto key = [](const vox_chunk_coord& c) {
    return ((uint64_t)(uint32_t)c.x << 40) ^ ((uint64_t)(uint32_t)c.y << 20) ^ (uint64_t)(uint32_t)c.z;
  };
  long ops = 0;
  for (int round = 0; round < 200; ++round) {
    for (int k = 0; k < 5000; ++k, ++ops) {
      vox_chunk_coord c{(int)(rng() % 64) - 32, (int)(rng() % 3) - 1, (int)(rng() % 64) - 32};
      if (rng() % 7 == 0) c.x += (rng() % 2) ? (1 << 22) : -(1 << 22);
      const int op = (int)(rng() % 3);
      auto it = fm.find(c);
      auto r = ref.find(key(c));
      if ((it == fm.end()) != (r == ref.end())) return std::printf("find mismatch\n"), 1;
      if (it != fm.end() && it->second != r->second) return std::printf("value mismatch\n"), 1;
      if (op == 0 && it == fm.end()) {
        const int v = (int)(rng() % 1000000);
        fm.emplace(c, v);
        ref[key(c)] = v;
      } else if (op == 1 && it != fm.end()) {
        fm.erase(it);
        ref.erase(r);
      } else if (op == 2 && it != fm.end()) {
        it->second += 1;
        r->second += 1;
      }
      const uint64_t id = rng() % 4096;
      auto ii = ids.find(id);
      auto ri = ref_ids.find(id);
      if ((ii == ids.end()) != (ri == ref_ids.end())) return std::printf("id find mismatch\n"), 1;
      if (ii == ids.end()) {
        ids.emplace(id, (int)id);
        ref_ids[id] = (int)id;
      } else if (rng() % 2) {
        ids.erase(ii);
        ref_ids.erase(ri);
      }
    }
    if (fm.size() != ref.size() || ids.size() != ref_ids.size()) return std::printf("size mismatch\n"), 1;
    size_t seen = 0;
    for (auto& kv : fm) {
      auto r = ref.find(key(kv.first));
      if (r == ref.end() || r->second != kv.second) return std::printf("iteration mismatch\n"), 1;
      ++seen;
    }
    if (seen != ref.size()) return std::printf("iteration count mismatch\n"), 1;
    if (round % 50 == 0) fm.reserve(fm.size() + 3000);
  }
  std::printf("ok %ld operations\n", ops);
  return 0;
}
