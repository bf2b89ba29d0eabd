// vox_order.h — the streaming engine's admit order: chunk requests sorted by their squared
// distance from the eye, nearest first, as a stable least-significant-digit radix sort on
// the bits of the distances.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

namespace vox {

// Fills order with 0..n-1 sorted by keys[i] ascending, equal keys in index order (a stable
// sort). The keys are squared distances: non-negative and never -0 (+inf and NaN sort
// last). A non-negative float's bit pattern orders like the float, so four counting passes
// over its bytes, lowest first, give the order.
inline void radix_order(const float* keys, size_t n, std::vector<uint32_t>& order) {
  std::vector<uint32_t> key(n), key2(n), idx2(n);
  order.resize(n);
  for (size_t i = 0; i < n; ++i) {
    std::memcpy(&key[i], &keys[i], sizeof(float));
    order[i] = (uint32_t)i;
  }
  for (int shift = 0; shift < 32; shift += 8) {
    size_t count[257] = {0};
    for (size_t i = 0; i < n; ++i) ++count[((key[i] >> shift) & 255u) + 1];
    for (int b = 0; b < 256; ++b) count[b + 1] += count[b];
    for (size_t i = 0; i < n; ++i) {
      const size_t at = count[(key[i] >> shift) & 255u]++;
      key2[at] = key[i];
      idx2[at] = order[i];
    }
    key.swap(key2);
    order.swap(idx2);
  }
}

}  // namespace vox
