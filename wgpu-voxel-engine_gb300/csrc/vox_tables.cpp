// vox_tables.cpp — per-context constant tables, computed once on the host.
//
// The reference builds one Rotation3::from_euler_angles per emitted face
// (src/quad.rs:14-46) and one T*R matrix product per face (src/quad.rs:47-54). Every
// face of a direction shares the same rotation, so the six rotations, the parts of
// T*R that do not depend on the translation, and the four rotated quad corners are
// evaluated here once, with the same f32 operations, and the kernels only add the
// translation. Built with -ffp-contract=off (no FMA contraction on any host).
#include "vox_tables.h"

#include <cmath>
#include <cstring>

namespace vox {

namespace {

// splitmix64 (Steele, Lea, Flood 2014).
uint64_t splitmix_next(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// f32::to_radians: deg * (PI / 180), PI and the quotient rounded to f32.
float to_radians(float deg) {
  const float pi = 3.14159265358979323846f;
  const float rad_per_deg = pi / 180.0f;
  return deg * rad_per_deg;
}

// Quad::new angles (roll, pitch, yaw) by emission direction L R Bk F D U.
void face_angles(int dir, float& roll, float& pitch, float& yaw) {
  roll = pitch = yaw = 0.0f;
  switch (dir) {
    case 0: pitch = to_radians(-90.0f); break;
    case 1: pitch = to_radians(90.0f); break;
    case 2: pitch = to_radians(180.0f); break;
    case 3: break;
    case 4: roll = to_radians(90.0f); break;
    default: roll = to_radians(-90.0f); break;
  }
}

}  // namespace

void face_rotation(int dir, float R[3][3]) {
  float roll, pitch, yaw;
  face_angles(dir, roll, pitch, yaw);
  const float sr = std::sin(roll), cr = std::cos(roll);
  const float sp = std::sin(pitch), cp = std::cos(pitch);
  const float sy = std::sin(yaw), cy = std::cos(yaw);
  // Rz(yaw) * Ry(pitch) * Rx(roll) multiplied out.
  R[0][0] = cy * cp;
  R[0][1] = cy * sp * sr - sy * cr;
  R[0][2] = cy * sp * cr + sy * sr;
  R[1][0] = sy * cp;
  R[1][1] = sy * sp * sr + cy * cr;
  R[1][2] = sy * sp * cr - cy * sr;
  R[2][0] = -sp;
  R[2][1] = cp * sr;
  R[2][2] = cp * cr;
}

void build_tables(const vox_config& cfg, TablesDev& t) {
  std::memset(&t, 0, sizeof t);
  static const int kSlot[6] = {VOX_FACE_LEFT, VOX_FACE_RIGHT, VOX_FACE_BACK,
                               VOX_FACE_FRONT, VOX_FACE_DOWN, VOX_FACE_UP};
  static const float kPos[4][3] = {
      {-0.5f, 0.5f, 0.5f}, {0.5f, 0.5f, 0.5f}, {-0.5f, -0.5f, 0.5f}, {0.5f, -0.5f, 0.5f}};
  static const float kUV[4][2] = {{0.0f, 0.0f}, {1.0f, 0.0f}, {0.0f, 1.0f}, {1.0f, 1.0f}};
  for (int d = 0; d < 6; ++d) {
    float R[3][3];
    face_rotation(d, R);
    // T*R with T = translation(0) for the parts that do not involve t: entry (i, j) is
    // sum_k T[i][k] * Rh[k][j] accumulated k = 0, 1, 2 (the k = 3 term is t_i * Rh[3][j]).
    const float T3[4][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f},
                            {0.0f, 0.0f, 0.0f}};
    float M0[3][3];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 3; ++j) {
        float s = T3[i][0] * R[0][j];
        s = s + T3[i][1] * R[1][j];
        s = s + T3[i][2] * R[2][j];
        if (i < 3) {
          t.part[d][i][j] = s;
          M0[i][j] = s + 0.0f * 0.0f;  // the t_i * Rh[3][j] term at t_i = 0
        } else {
          t.row3[d][j] = s + 1.0f * 0.0f;  // T[3][3] * Rh[3][j]
        }
      }
    // Rotated quad corners: (M * (p, 1))[r] without the final + t_r.
    for (int v = 0; v < 4; ++v)
      for (int r = 0; r < 3; ++r) {
        float s = M0[r][0] * kPos[v][0];
        s = s + M0[r][1] * kPos[v][1];
        s = s + M0[r][2] * kPos[v][2];
        t.corner[d][v][r] = s;
      }
    t.slot[d] = (uint32_t)kSlot[d];
    t.tex[d] = cfg.texture_index[kSlot[d]];
  }
  for (int v = 0; v < 4; ++v) {
    t.uv[v][0] = kUV[v][0];
    t.uv[v][1] = kUV[v][1];
  }
  // Noise permutation: Fisher-Yates over 0..255 driven by splitmix64(seed), doubled.
  uint8_t perm[256];
  for (int i = 0; i < 256; ++i) perm[i] = (uint8_t)i;
  uint64_t s = cfg.gen.seed;
  for (int i = 255; i > 0; --i) {
    const uint64_t r = splitmix_next(s);
    const int j = (int)(r % (uint64_t)(i + 1));
    const uint8_t tmp = perm[i];
    perm[i] = perm[j];
    perm[j] = tmp;
  }
  for (int i = 0; i < 512; ++i) t.perm[i] = perm[i & 255];
  // Gradient of hash h (Perlin 2002): u = x if h < 8 else y, v = y if h < 4, x if h is
  // 12 or 14, z otherwise; bit 0 negates u, bit 1 negates v. u and v are different axes.
  for (int h = 0; h < 16; ++h) {
    float g[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    g[h < 8 ? 0 : 1] = (h & 1) ? -1.0f : 1.0f;
    g[h < 4 ? 1 : ((h == 12 || h == 14) ? 0 : 2)] = (h & 2) ? -1.0f : 1.0f;
    for (int k = 0; k < 4; ++k) t.grad[h][k] = g[k];
  }
}

}  // namespace vox
