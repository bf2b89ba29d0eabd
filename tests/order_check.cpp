// Randomized check of vox::radix_order (the streaming engine's admit order) against
// std::stable_sort of the same keys: squared distances of chunk centres from random eyes
// (many ties), uniform and log-uniform floats, zeros, subnormals and +inf, at sizes from 0
// to 200,000. Prints "ok" and exits 0 when every order agrees.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <random>
#include <vector>

#include "vox_order.h"

static bool agrees(const std::vector<float>& keys) {
  std::vector<uint32_t> got;
  vox::radix_order(keys.data(), keys.size(), got);
  std::vector<uint32_t> want(keys.size());
  for (size_t i = 0; i < want.size(); ++i) want[i] = (uint32_t)i;
  std::stable_sort(want.begin(), want.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  return got == want;
}

int main() {
  std::mt19937_64 rng(11);
  std::uniform_real_distribution<float> unit(0.0f, 1.0f);
  const size_t sizes[] = {0, 1, 2, 3, 255, 256, 257, 1000, 4096, 65537, 200000};
  long cases = 0;
  for (size_t n : sizes) {
    for (int kind = 0; kind < 4; ++kind, ++cases) {
      std::vector<float> keys(n);
      const float ex = (float)(rng() % 4096) - 2048.0f + unit(rng);
      const float ez = (float)(rng() % 4096) - 2048.0f + unit(rng);
      for (size_t i = 0; i < n; ++i) {
        switch (kind) {
          case 0: {  // chunk centres of a disk of 16^3 chunks around an eye (ties)
            const float dx = (float)((int)(rng() % 49) - 24) * 16.0f + 8.0f - ex;
            const float dy = (float)((int)(rng() % 5) - 2) * 16.0f + 8.0f - 40.0f;
            const float dz = (float)((int)(rng() % 49) - 24) * 16.0f + 8.0f - ez;
            keys[i] = dx * dx + dy * dy + dz * dz;
            break;
          }
          case 1:
            keys[i] = unit(rng) * 1.0e6f;
            break;
          case 2:
            keys[i] = std::ldexp(1.0f + unit(rng), (int)(rng() % 300) - 160);  // subnormals to 1e42
            break;
          default: {
            const uint64_t r = rng() % 8;
            keys[i] = r == 0 ? 0.0f : r == 1 ? std::numeric_limits<float>::infinity()
                    : r == 2 ? std::numeric_limits<float>::denorm_min() : (float)(rng() % 16);
          }
        }
      }
      if (!agrees(keys)) return std::printf("order mismatch: n %zu kind %d\n", n, kind), 1;
    }
  }
  std::printf("ok %ld cases\n", cases);
  return 0;
}
