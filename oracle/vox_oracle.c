/*
 * vox_oracle.c — CPU oracle (test infrastructure only; see vox_oracle.h for the
 * parity status). Each function cites the reference file:line it restates.
 *
 * Build: cc -O2 -ffp-contract=off -fPIC -shared vox_oracle.c -lm -lpthread
 */
#include "vox_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define OR_AIR 2u
#define OR_GRASS 0u

/* ------------------------------------------------------------------------------------ */
/* splitmix64 and the seeded permutation                                                 */
/* ------------------------------------------------------------------------------------ */

uint64_t or_splitmix64_next(uint64_t* state) {
  uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

void or_perm_init(uint64_t seed, uint8_t p[512]) {
  uint8_t perm[256];
  for (int i = 0; i < 256; ++i) perm[i] = (uint8_t)i;
  uint64_t s = seed;
  for (int i = 255; i > 0; --i) {
    uint64_t r = or_splitmix64_next(&s);
    int j = (int)(r % (uint64_t)(i + 1));
    uint8_t t = perm[i];
    perm[i] = perm[j];
    perm[j] = t;
  }
  for (int i = 0; i < 512; ++i) p[i] = perm[i & 255];
}

/* ------------------------------------------------------------------------------------ */
/* Improved noise (K. Perlin, "Improving Noise", SIGGRAPH 2002)                          */
/* ------------------------------------------------------------------------------------ */

static float fade_f(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
static float lerp_f(float t, float a, float b) { return a + t * (b - a); }

/* Gradient of hash h as coefficients (gx, gy, gz) in {-1, 0, 1}. Perlin's 2002 gradient
 * picks u = (h < 8 ? x : y) and v = (h < 4 ? y : h == 12 || h == 14 ? x : z) with the
 * signs of bits 0 and 1; u and v are always different axes, so the gradient is the dot
 * product with this coefficient vector. The project's noise spec evaluates it as
 * ((gx*x + gy*y) + gz*z), which equals u' + v' except for the sign of an exact zero. */
void or_grad_coef(int h, float g[3]) {
  h &= 15;
  const float su = (h & 1) ? -1.0f : 1.0f, sv = (h & 2) ? -1.0f : 1.0f;
  g[0] = g[1] = g[2] = 0.0f;
  g[h < 8 ? 0 : 1] = su;
  g[h < 4 ? 1 : ((h == 12 || h == 14) ? 0 : 2)] = sv;
}
static float grad3_f(int h, float x, float y, float z) {
  float g[3];
  or_grad_coef(h, g);
  return (g[0] * x + g[1] * y) + g[2] * z;
}
static float grad2_f(int h, float x, float y) {
  float g[3];
  or_grad_coef(h, g);
  return g[0] * x + g[1] * y;
}

static double fade_d(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
static double lerp_d(double t, double a, double b) { return a + t * (b - a); }
static double grad3_d(int h, double x, double y, double z) {
  float g[3];
  or_grad_coef(h, g);
  return ((double)g[0] * x + (double)g[1] * y) + (double)g[2] * z;
}
static double grad2_d(int h, double x, double y) {
  float g[3];
  or_grad_coef(h, g);
  return (double)g[0] * x + (double)g[1] * y;
}

float or_noise3_f32(const uint8_t* p, float x, float y, float z) {
  float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  float u = fade_f(x), v = fade_f(y), w = fade_f(z);
  int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
  int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
  float x1 = x - 1.0f, y1 = y - 1.0f, z1 = z - 1.0f;
  float l00 = lerp_f(u, grad3_f(p[AA], x, y, z), grad3_f(p[BA], x1, y, z));
  float l10 = lerp_f(u, grad3_f(p[AB], x, y1, z), grad3_f(p[BB], x1, y1, z));
  float l01 = lerp_f(u, grad3_f(p[AA + 1], x, y, z1), grad3_f(p[BA + 1], x1, y, z1));
  float l11 = lerp_f(u, grad3_f(p[AB + 1], x, y1, z1), grad3_f(p[BB + 1], x1, y1, z1));
  return lerp_f(w, lerp_f(v, l00, l10), lerp_f(v, l01, l11));
}

float or_noise2_f32(const uint8_t* p, float x, float y) {
  float fx = floorf(x), fy = floorf(y);
  int X = (int)fx & 255, Y = (int)fy & 255;
  x = x - fx;
  y = y - fy;
  float u = fade_f(x), v = fade_f(y);
  int A = p[X] + Y, B = p[X + 1] + Y;
  float x1 = x - 1.0f, y1 = y - 1.0f;
  float l0 = lerp_f(u, grad2_f(p[p[A]], x, y), grad2_f(p[p[B]], x1, y));
  float l1 = lerp_f(u, grad2_f(p[p[A + 1]], x, y1), grad2_f(p[p[B + 1]], x1, y1));
  return lerp_f(v, l0, l1);
}

double or_noise3_f64(const uint8_t* p, double x, double y, double z) {
  double fx = floor(x), fy = floor(y), fz = floor(z);
  int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  double u = fade_d(x), v = fade_d(y), w = fade_d(z);
  int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
  int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
  double x1 = x - 1.0, y1 = y - 1.0, z1 = z - 1.0;
  double l00 = lerp_d(u, grad3_d(p[AA], x, y, z), grad3_d(p[BA], x1, y, z));
  double l10 = lerp_d(u, grad3_d(p[AB], x, y1, z), grad3_d(p[BB], x1, y1, z));
  double l01 = lerp_d(u, grad3_d(p[AA + 1], x, y, z1), grad3_d(p[BA + 1], x1, y, z1));
  double l11 = lerp_d(u, grad3_d(p[AB + 1], x, y1, z1), grad3_d(p[BB + 1], x1, y1, z1));
  return lerp_d(w, lerp_d(v, l00, l10), lerp_d(v, l01, l11));
}

double or_noise2_f64(const uint8_t* p, double x, double y) {
  double fx = floor(x), fy = floor(y);
  int X = (int)fx & 255, Y = (int)fy & 255;
  x = x - fx;
  y = y - fy;
  double u = fade_d(x), v = fade_d(y);
  int A = p[X] + Y, B = p[X + 1] + Y;
  double x1 = x - 1.0, y1 = y - 1.0;
  double l0 = lerp_d(u, grad2_d(p[p[A]], x, y), grad2_d(p[p[B]], x1, y));
  double l1 = lerp_d(u, grad2_d(p[p[A + 1]], x, y1), grad2_d(p[p[B + 1]], x1, y1));
  return lerp_d(v, l0, l1);
}

float or_fbm2_f32(const uint8_t* p, float x, float y, int octaves, float freq, float lac,
                  float gain) {
  float sum = 0.0f, amp = 1.0f, f = freq;
  for (int o = 0; o < octaves; ++o) {
    sum = sum + amp * or_noise2_f32(p, x * f, y * f);
    f = f * lac;
    amp = amp * gain;
  }
  return sum;
}

float or_fbm3_f32(const uint8_t* p, float x, float y, float z, int octaves, float freq, float lac,
                  float gain) {
  float sum = 0.0f, amp = 1.0f, f = freq;
  for (int o = 0; o < octaves; ++o) {
    sum = sum + amp * or_noise3_f32(p, x * f, y * f, z * f);
    f = f * lac;
    amp = amp * gain;
  }
  return sum;
}

double or_fbm2_f64(const uint8_t* p, double x, double y, int octaves, double freq, double lac,
                   double gain) {
  double sum = 0.0, amp = 1.0, f = freq;
  for (int o = 0; o < octaves; ++o) {
    sum = sum + amp * or_noise2_f64(p, x * f, y * f);
    f = f * lac;
    amp = amp * gain;
  }
  return sum;
}

double or_fbm3_f64(const uint8_t* p, double x, double y, double z, int octaves, double freq,
                   double lac, double gain) {
  double sum = 0.0, amp = 1.0, f = freq;
  for (int o = 0; o < octaves; ++o) {
    sum = sum + amp * or_noise3_f64(p, x * f, y * f, z * f);
    f = f * lac;
    amp = amp * gain;
  }
  return sum;
}

/* ------------------------------------------------------------------------------------ */
/* Chunk::new / generate_terrain (src/chunk.rs:21-46)                                    */
/* ------------------------------------------------------------------------------------ */

static int valid_size(int n) { return n == 8 || n == 16 || n == 32 || n == 64; }

/* Heightmap column height at world (wx, wz). */
static float height_f32(const vox_generator* g, const uint8_t* p, int32_t wx, int32_t wz) {
  float f = or_fbm2_f32(p, (float)wx, (float)wz, g->octaves, g->frequency, g->lacunarity, g->gain);
  return g->base_height + g->amplitude * f;
}

/* Density value at world (wx, wy, wz). */
static float density_f32(const vox_generator* g, const uint8_t* p, int32_t wx, int32_t wy,
                         int32_t wz) {
  float f = or_fbm3_f32(p, (float)wx, (float)wy, (float)wz, g->octaves, g->frequency,
                        g->lacunarity, g->gain);
  return f - ((float)wy - g->y_ref) * g->y_scale;
}

static int density_solid(const vox_generator* g, float d) {
  return g->solid_below_zero ? (d < 0.0f) : (d > 0.0f);
}

int or_generate_cubes(const vox_config* cfg, vox_chunk_coord c, int64_t chunk_index,
                      uint8_t* cubes) {
  const int N = cfg->chunk_size;
  if (!valid_size(N)) return VOX_ERR_INVALID;
  const vox_generator* g = &cfg->gen;
  const int32_t ox = c.x * N, oy = c.y * N, oz = c.z * N;
  uint8_t p[512];
  if (g->kind == VOX_GEN_HEIGHTMAP) {
    or_perm_init(g->seed, p);
    float* h = (float*)malloc(sizeof(float) * (size_t)N * (size_t)N);
    if (!h) return VOX_ERR_OOM;
    for (int z = 0; z < N; ++z)
      for (int x = 0; x < N; ++x) h[z * N + x] = height_f32(g, p, ox + x, oz + z);
    for (int y = 0; y < N; ++y)
      for (int z = 0; z < N; ++z)
        for (int x = 0; x < N; ++x)
          cubes[x + N * z + N * N * y] =
              ((float)(oy + y) < h[z * N + x]) ? OR_GRASS : OR_AIR;
    free(h);
  } else if (g->kind == VOX_GEN_DENSITY) {
    or_perm_init(g->seed, p);
    for (int y = 0; y < N; ++y)
      for (int z = 0; z < N; ++z)
        for (int x = 0; x < N; ++x)
          cubes[x + N * z + N * N * y] =
              density_solid(g, density_f32(g, p, ox + x, oy + y, oz + z)) ? OR_GRASS : OR_AIR;
  } else if (g->kind == VOX_GEN_BERNOULLI) {
    /* One draw per voxel in (y, z, x) order, x fastest; solid iff the draw's low bit. */
    uint64_t s = g->seed ^ (uint64_t)chunk_index;
    for (int y = 0; y < N; ++y)
      for (int z = 0; z < N; ++z)
        for (int x = 0; x < N; ++x)
          cubes[x + N * z + N * N * y] = (or_splitmix64_next(&s) & 1u) ? OR_GRASS : OR_AIR;
  } else {
    return VOX_ERR_INVALID;
  }
  return VOX_OK;
}

static int words_per_row(int N) { return N > 32 ? N / 32 : 1; }

void or_cubes_to_occ(int N, const uint8_t* cubes, uint32_t* occ) {
  const int W = words_per_row(N);
  memset(occ, 0, sizeof(uint32_t) * (size_t)N * (size_t)N * (size_t)W);
  for (int y = 0; y < N; ++y)
    for (int z = 0; z < N; ++z)
      for (int x = 0; x < N; ++x)
        if (cubes[x + N * z + N * N * y] != OR_AIR)
          occ[(size_t)(y * N + z) * W + (x >> 5)] |= 1u << (x & 31);
}

void or_occ_to_cubes(int N, const uint32_t* occ, uint8_t* cubes) {
  const int W = words_per_row(N);
  for (int y = 0; y < N; ++y)
    for (int z = 0; z < N; ++z)
      for (int x = 0; x < N; ++x)
        cubes[x + N * z + N * N * y] =
            ((occ[(size_t)(y * N + z) * W + (x >> 5)] >> (x & 31)) & 1u) ? OR_GRASS : OR_AIR;
}

/* ------------------------------------------------------------------------------------ */
/* cull_unseen_triangles (src/chunk.rs:59-245)                                           */
/* ------------------------------------------------------------------------------------ */

static int is_air(const uint8_t* cubes, int N, int x, int y, int z) {
  return cubes[x + N * z + N * N * y] == OR_AIR;
}

int64_t or_cull_faces(int N, int cull_mode, const uint8_t* cubes, const uint8_t* const adj[6],
                      or_face* faces, int64_t cap) {
  int64_t n = 0;
  const uint8_t* none[6] = {0, 0, 0, 0, 0, 0};
  if (!adj) adj = none;
  const int full6 = cull_mode == VOX_CULL_FULL6;
#define OR_EMIT(d)                                                     \
  do {                                                                 \
    if (faces && n < cap) {                                            \
      faces[n].x = (uint8_t)x;                                         \
      faces[n].y = (uint8_t)y;                                         \
      faces[n].z = (uint8_t)z;                                         \
      faces[n].dir = (uint8_t)(d);                                     \
    }                                                                  \
    ++n;                                                               \
  } while (0)
  for (int y = 0; y < N; ++y) {
    for (int z = 0; z < N; ++z) {
      for (int x = 0; x < N; ++x) {
        if (is_air(cubes, N, x, y, z)) continue; /* chunk.rs:71-73 */
        /* LEFT, chunk.rs:77-109: inside, else the -x neighbour's x = N-1, else emit. */
        if (x > 0) {
          if (is_air(cubes, N, x - 1, y, z)) OR_EMIT(0);
        } else if (adj[0]) {
          if (is_air(adj[0], N, N - 1, y, z)) OR_EMIT(0);
        } else {
          OR_EMIT(0);
        }
        /* RIGHT, chunk.rs:110-140 */
        if (x < N - 1) {
          if (is_air(cubes, N, x + 1, y, z)) OR_EMIT(1);
        } else if (adj[1]) {
          if (is_air(adj[1], N, 0, y, z)) OR_EMIT(1);
        } else {
          OR_EMIT(1);
        }
        /* BACK, chunk.rs:141-173 */
        if (z > 0) {
          if (is_air(cubes, N, x, y, z - 1)) OR_EMIT(2);
        } else if (adj[2]) {
          if (is_air(adj[2], N, x, y, N - 1)) OR_EMIT(2);
        } else {
          OR_EMIT(2);
        }
        /* FRONT, chunk.rs:174-204 */
        if (z < N - 1) {
          if (is_air(cubes, N, x, y, z + 1)) OR_EMIT(3);
        } else if (adj[3]) {
          if (is_air(adj[3], N, x, y, 0)) OR_EMIT(3);
        } else {
          OR_EMIT(3);
        }
        /* DOWN, chunk.rs:205-222: the y border is always emitted in the reference. */
        if (y > 0) {
          if (is_air(cubes, N, x, y - 1, z)) OR_EMIT(4);
        } else if (full6 && adj[4]) {
          if (is_air(adj[4], N, x, N - 1, z)) OR_EMIT(4);
        } else {
          OR_EMIT(4);
        }
        /* UP, chunk.rs:223-240 */
        if (y < N - 1) {
          if (is_air(cubes, N, x, y + 1, z)) OR_EMIT(5);
        } else if (full6 && adj[5]) {
          if (is_air(adj[5], N, x, 0, z)) OR_EMIT(5);
        } else {
          OR_EMIT(5);
        }
      }
    }
  }
#undef OR_EMIT
  return n;
}

/* ------------------------------------------------------------------------------------ */
/* Quad::new / Quad::to_raw (src/quad.rs:14-54) and the vertex shader (vertex.vert:22-27) */
/* ------------------------------------------------------------------------------------ */

int or_dir_slot(int dir) {
  static const int slot[6] = {VOX_FACE_LEFT, VOX_FACE_RIGHT, VOX_FACE_BACK,
                              VOX_FACE_FRONT, VOX_FACE_DOWN, VOX_FACE_UP};
  return slot[dir];
}

/* f32::to_radians: deg * (PI / 180) with PI and the quotient rounded to f32. */
static float to_radians_f(float deg) {
  const float pi = 3.14159265358979323846f;
  const float rad_per_deg = pi / 180.0f;
  return deg * rad_per_deg;
}

void or_face_rotation(int dir, float R[3][3]) {
  /* Euler angles (roll, pitch, yaw) per face, src/quad.rs:17-37. */
  float roll = 0.0f, pitch = 0.0f, yaw = 0.0f;
  switch (dir) {
    case 0: pitch = to_radians_f(-90.0f); break; /* LEFT */
    case 1: pitch = to_radians_f(90.0f); break;  /* RIGHT */
    case 2: pitch = to_radians_f(180.0f); break; /* BACK */
    case 3: break;                               /* FRONT */
    case 4: roll = to_radians_f(90.0f); break;   /* DOWN */
    case 5: roll = to_radians_f(-90.0f); break;  /* UP */
    default: break;
  }
  const float sr = sinf(roll), cr = cosf(roll);
  const float sp = sinf(pitch), cp = cosf(pitch);
  const float sy = sinf(yaw), cy = cosf(yaw);
  /* R = Rz(yaw) * Ry(pitch) * Rx(roll), multiplied out symbolically. */
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

/* M = T * R with T, R as 4x4 homogeneous matrices; each entry is the dot product of a
 * row of T and a column of R accumulated k = 0..3 in order. M is row-major M[row][col]. */
static void instance_matrix(int dir, int32_t wx, int32_t wy, int32_t wz, float M[4][4]) {
  float R[3][3];
  or_face_rotation(dir, R);
  float T[4][4] = {{1.0f, 0.0f, 0.0f, (float)wx},
                   {0.0f, 1.0f, 0.0f, (float)wy},
                   {0.0f, 0.0f, 1.0f, (float)wz},
                   {0.0f, 0.0f, 0.0f, 1.0f}};
  float Rh[4][4] = {{R[0][0], R[0][1], R[0][2], 0.0f},
                    {R[1][0], R[1][1], R[1][2], 0.0f},
                    {R[2][0], R[2][1], R[2][2], 0.0f},
                    {0.0f, 0.0f, 0.0f, 1.0f}};
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float s = T[i][0] * Rh[0][j];
      s = s + T[i][1] * Rh[1][j];
      s = s + T[i][2] * Rh[2][j];
      s = s + T[i][3] * Rh[3][j];
      M[i][j] = s;
    }
}

void or_instance_raw(int dir, int32_t wx, int32_t wy, int32_t wz, uint32_t texture_index,
                     vox_instance_raw* out) {
  float M[4][4];
  instance_matrix(dir, wx, wy, wz, M);
  /* nalgebra Matrix4 -> [[f32; 4]; 4] is column-major: t_matrix[col][row]. */
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) out->t_matrix[c][r] = M[r][c];
  out->texture_index = texture_index;
}

/* quad::VERTICES (src/quad.rs:66-87): tr, tl, br, bl. */
static const float kQuadPos[4][3] = {
    {-0.5f, 0.5f, 0.5f}, {0.5f, 0.5f, 0.5f}, {-0.5f, -0.5f, 0.5f}, {0.5f, -0.5f, 0.5f}};
static const float kQuadUV[4][2] = {{0.0f, 0.0f}, {1.0f, 0.0f}, {0.0f, 1.0f}, {1.0f, 1.0f}};
/* quad::INDICES (src/quad.rs:89). */
static const uint32_t kQuadIdx[6] = {0, 2, 1, 3, 1, 2};

void or_face_vertices(int dir, int32_t wx, int32_t wy, int32_t wz, uint32_t local_face,
                      vox_vertex out_v[4], uint32_t out_i[6]) {
  float M[4][4];
  instance_matrix(dir, wx, wy, wz, M);
  for (int v = 0; v < 4; ++v) {
    const float px = kQuadPos[v][0], py = kQuadPos[v][1], pz = kQuadPos[v][2];
    for (int r = 0; r < 3; ++r) {
      /* (instance * vec4(pos, 1))[r], summed over columns 0..3 in order. */
      float s = M[r][0] * px;
      s = s + M[r][1] * py;
      s = s + M[r][2] * pz;
      s = s + M[r][3] * 1.0f;
      out_v[v].position[r] = s;
    }
    out_v[v].tex_coords[0] = kQuadUV[v][0];
    out_v[v].tex_coords[1] = kQuadUV[v][1];
    out_v[v].face = (uint32_t)or_dir_slot(dir);
  }
  for (int k = 0; k < 6; ++k) out_i[k] = 4u * local_face + kQuadIdx[k];
}

static void emit_faces(const vox_config* cfg, vox_chunk_coord coord, const or_face* faces,
                       int64_t count, uint64_t first_local, void* out0, void* out1) {
  const int N = cfg->chunk_size;
  const int32_t ox = coord.x * N, oy = coord.y * N, oz = coord.z * N;
  for (int64_t f = 0; f < count; ++f) {
    const or_face* fc = &faces[f];
    const int32_t wx = ox + fc->x, wy = oy + fc->y, wz = oz + fc->z;
    if (cfg->layout == VOX_LAYOUT_INSTANCED) {
      vox_instance_raw* o = (vox_instance_raw*)out0 + f;
      or_instance_raw(fc->dir, wx, wy, wz, cfg->texture_index[or_dir_slot(fc->dir)], o);
    } else {
      vox_vertex* ov = (vox_vertex*)out0 + 4 * f;
      uint32_t* oi = (uint32_t*)out1 + 6 * f;
      or_face_vertices(fc->dir, wx, wy, wz, (uint32_t)(first_local + (uint64_t)f), ov, oi);
    }
  }
}

int64_t or_mesh_chunk(const vox_config* cfg, vox_chunk_coord coord, const uint8_t* cubes,
                      const uint8_t* const adj[6], void* out0, void* out1, int64_t cap) {
  const int N = cfg->chunk_size;
  int64_t total = or_cull_faces(N, cfg->cull_mode, cubes, adj, NULL, 0);
  if (!out0 || cap <= 0) return total;
  int64_t w = total < cap ? total : cap;
  or_face* faces = (or_face*)malloc(sizeof(or_face) * (size_t)(total > 0 ? total : 1));
  if (!faces) return -1;
  or_cull_faces(N, cfg->cull_mode, cubes, adj, faces, total);
  emit_faces(cfg, coord, faces, w, 0, out0, out1);
  free(faces);
  return total;
}

static vox_chunk_coord nbr_coord(vox_chunk_coord c, int d) {
  static const int dx[6] = {-1, 1, 0, 0, 0, 0};
  static const int dy[6] = {0, 0, 0, 0, -1, 1};
  static const int dz[6] = {0, 0, -1, 1, 0, 0};
  vox_chunk_coord r = {c.x + dx[d], c.y + dy[d], c.z + dz[d]};
  return r;
}

int64_t or_gen_mesh_batch(const vox_config* cfg, const vox_chunk_coord* coords,
                          const uint8_t* nbr_mask, int32_t n, int64_t index_base, void* out0,
                          void* out1, int64_t cap, uint64_t* face_offsets) {
  const int N = cfg->chunk_size;
  if (!valid_size(N) || n < 0) return -1;
  const size_t vox = (size_t)N * N * N;
  uint8_t* cubes = (uint8_t*)malloc(vox * 7);
  if (!cubes) return -1;
  uint64_t total = 0;
  int64_t per_face0 = cfg->layout == VOX_LAYOUT_INSTANCED ? (int64_t)sizeof(vox_instance_raw)
                                                           : 4 * (int64_t)sizeof(vox_vertex);
  for (int32_t i = 0; i < n; ++i) {
    or_generate_cubes(cfg, coords[i], index_base + i, cubes);
    const uint8_t* adj[6] = {0, 0, 0, 0, 0, 0};
    uint8_t m = nbr_mask ? nbr_mask[i] : 0;
    if (cfg->gen.kind == VOX_GEN_BERNOULLI) m = 0; /* Bernoulli chunks are isolated */
    for (int d = 0; d < 6; ++d) {
      if (!((m >> d) & 1)) continue;
      if (d >= 4 && cfg->cull_mode != VOX_CULL_FULL6) continue;
      uint8_t* nb = cubes + vox * (size_t)(1 + d);
      or_generate_cubes(cfg, nbr_coord(coords[i], d), 0, nb);
      adj[d] = nb;
    }
    int64_t cnt = or_cull_faces(N, cfg->cull_mode, cubes, adj, NULL, 0);
    if (face_offsets) face_offsets[i] = total;
    if (out0 && (int64_t)total < cap) {
      int64_t room = cap - (int64_t)total;
      int64_t w = cnt < room ? cnt : room;
      or_face* faces = (or_face*)malloc(sizeof(or_face) * (size_t)(cnt > 0 ? cnt : 1));
      if (!faces) {
        free(cubes);
        return -1;
      }
      or_cull_faces(N, cfg->cull_mode, cubes, adj, faces, cnt);
      void* o0 = (char*)out0 + (size_t)total * (size_t)per_face0;
      void* o1 = out1 ? (void*)((uint32_t*)out1 + 6 * total) : NULL;
      emit_faces(cfg, coords[i], faces, w, 0, o0, o1);
      free(faces);
    }
    total += (uint64_t)cnt;
  }
  if (face_offsets) face_offsets[n] = total;
  free(cubes);
  return (int64_t)total;
}

/* ------------------------------------------------------------------------------------ */
/* CPU baseline: the reference's pool work, one chunk per task                           */
/* ------------------------------------------------------------------------------------ */

typedef struct {
  const vox_config* cfg;
  const vox_chunk_coord* coords;
  const uint8_t* nbr_mask;
  int32_t n;
  int64_t index_base;
  uint8_t* cubes; /* n chunks */
  const int32_t* nbr_index; /* 6 per chunk, -1 = none */
  int phase;
  volatile int64_t next;
  int64_t total;
  pthread_mutex_t lock;
} baseline_job;

static int64_t claim(baseline_job* j) { return __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED); }

static void* baseline_worker(void* arg) {
  baseline_job* j = (baseline_job*)arg;
  const int N = j->cfg->chunk_size;
  const size_t vox = (size_t)N * N * N;
  int64_t local_total = 0;
  for (;;) {
    int64_t i = claim(j);
    if (i >= j->n) break;
    if (j->phase == 0) {
      /* Chunk::new(pos) */
      or_generate_cubes(j->cfg, j->coords[i], j->index_base + i, j->cubes + vox * (size_t)i);
    } else {
      /* create_mesh(device, adjacent_chunks): faces Vec<Quad>, then Vec<InstanceRaw>. */
      const uint8_t* adj[6] = {0, 0, 0, 0, 0, 0};
      for (int d = 0; d < 6; ++d) {
        int32_t k = j->nbr_index[6 * i + d];
        if (k >= 0) adj[d] = j->cubes + vox * (size_t)k;
      }
      const uint8_t* cubes = j->cubes + vox * (size_t)i;
      int64_t cap = 64;
      or_face* faces = (or_face*)malloc(sizeof(or_face) * (size_t)cap);
      int64_t cnt = or_cull_faces(N, j->cfg->cull_mode, cubes, adj, faces, cap);
      if (cnt > cap) { /* the Vec grew: collect again into the larger buffer */
        free(faces);
        faces = (or_face*)malloc(sizeof(or_face) * (size_t)cnt);
        or_cull_faces(N, j->cfg->cull_mode, cubes, adj, faces, cnt);
      }
      size_t per0 = j->cfg->layout == VOX_LAYOUT_INSTANCED ? sizeof(vox_instance_raw)
                                                            : 4 * sizeof(vox_vertex);
      void* o0 = malloc(per0 * (size_t)(cnt > 0 ? cnt : 1));
      void* o1 = j->cfg->layout == VOX_LAYOUT_INSTANCED
                     ? NULL
                     : malloc(6 * sizeof(uint32_t) * (size_t)(cnt > 0 ? cnt : 1));
      emit_faces(j->cfg, j->coords[i], faces, cnt, 0, o0, o1);
      /* keep the writes observable */
      if (cnt > 0) local_total += (int64_t)((const uint8_t*)o0)[0] * 0 + cnt;
      free(o0);
      free(o1);
      free(faces);
    }
  }
  pthread_mutex_lock(&j->lock);
  j->total += local_total;
  pthread_mutex_unlock(&j->lock);
  return NULL;
}

static int coord_eq(vox_chunk_coord a, vox_chunk_coord b) {
  return a.x == b.x && a.y == b.y && a.z == b.z;
}

static uint64_t coord_hash(vox_chunk_coord c) {
  uint64_t s = ((uint64_t)(uint32_t)c.x * 0x9E3779B97F4A7C15ULL) ^
               ((uint64_t)(uint32_t)c.y * 0xC2B2AE3D27D4EB4FULL) ^
               ((uint64_t)(uint32_t)c.z * 0x165667B19E3779F9ULL);
  return or_splitmix64_next(&s);
}

int64_t or_baseline_run(const vox_config* cfg, const vox_chunk_coord* coords,
                        const uint8_t* nbr_mask, int32_t n, int64_t index_base, int nthreads) {
  const int N = cfg->chunk_size;
  if (!valid_size(N) || n <= 0) return -1;
  if (nthreads < 1) nthreads = 1;
  const size_t vox = (size_t)N * N * N;
  baseline_job j;
  memset(&j, 0, sizeof j);
  j.cfg = cfg;
  j.coords = coords;
  j.nbr_mask = nbr_mask;
  j.n = n;
  j.index_base = index_base;
  j.cubes = (uint8_t*)malloc(vox * (size_t)n);
  int32_t* nbr_index = (int32_t*)malloc(sizeof(int32_t) * 6 * (size_t)n);
  /* World.chunks lookup (src/chunk_builder.rs:134-169) as an open-addressing table. */
  size_t cap = 1;
  while (cap < 2 * (size_t)n) cap <<= 1;
  int32_t* table = (int32_t*)malloc(sizeof(int32_t) * cap);
  if (!j.cubes || !nbr_index || !table) {
    free(j.cubes);
    free(nbr_index);
    free(table);
    return -1;
  }
  for (size_t k = 0; k < cap; ++k) table[k] = -1;
  for (int32_t i = 0; i < n; ++i) {
    size_t h = coord_hash(coords[i]) & (cap - 1);
    while (table[h] >= 0) h = (h + 1) & (cap - 1);
    table[h] = i;
  }
  for (int32_t i = 0; i < n; ++i) {
    uint8_t m = nbr_mask ? nbr_mask[i] : 0;
    if (cfg->gen.kind == VOX_GEN_BERNOULLI) m = 0;
    for (int d = 0; d < 6; ++d) {
      nbr_index[6 * i + d] = -1;
      if (!((m >> d) & 1)) continue;
      if (d >= 4 && cfg->cull_mode != VOX_CULL_FULL6) continue;
      vox_chunk_coord q = nbr_coord(coords[i], d);
      size_t h = coord_hash(q) & (cap - 1);
      while (table[h] >= 0) {
        if (coord_eq(coords[table[h]], q)) {
          nbr_index[6 * i + d] = table[h];
          break;
        }
        h = (h + 1) & (cap - 1);
      }
    }
  }
  free(table);
  j.nbr_index = nbr_index;
  pthread_mutex_init(&j.lock, NULL);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  for (int phase = 0; phase < 2; ++phase) {
    j.phase = phase;
    j.next = 0;
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, baseline_worker, &j);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  }
  pthread_mutex_destroy(&j.lock);
  free(th);
  free(nbr_index);
  free(j.cubes);
  return j.total;
}

/* ------------------------------------------------------------------------------------ */
/* Per-chunk digests of whole batches (parity at full workload sizes)                    */
/* ------------------------------------------------------------------------------------ */

static uint64_t or_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

uint64_t or_digest(const void* bytes, uint64_t len) {
  const uint8_t* b = (const uint8_t*)bytes;
  uint64_t h = len;
  uint64_t k = 0;
  for (uint64_t off = 0; off < len; off += 8, ++k) {
    uint64_t w = 0;
    const uint64_t m = len - off < 8 ? len - off : 8;
    for (uint64_t j = 0; j < m; ++j) w |= (uint64_t)b[off + j] << (8 * j);
    h = or_mix64(h ^ or_mix64(w + k * 0x9E3779B97F4A7C15ULL));
  }
  return h;
}

typedef struct {
  const void* out0;
  const void* out1;
  const uint64_t* offs;
  int32_t n;
  int32_t b0, b1;
  uint64_t* digests;
  volatile int64_t next;
} digest_job;

static void* digest_worker(void* arg) {
  digest_job* j = (digest_job*)arg;
  for (;;) {
    const int64_t i = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
    if (i >= j->n) break;
    const uint64_t lo = j->offs[i], hi = j->offs[i + 1];
    j->digests[2 * i] = or_digest((const uint8_t*)j->out0 + lo * (uint64_t)j->b0, (hi - lo) * (uint64_t)j->b0);
    j->digests[2 * i + 1] =
        j->b1 > 0 ? or_digest((const uint8_t*)j->out1 + lo * (uint64_t)j->b1, (hi - lo) * (uint64_t)j->b1)
                  : 0;
  }
  return NULL;
}

void or_chunk_digests(const void* out0, const void* out1, const uint64_t* offs, int32_t n,
                      int32_t b0, int32_t b1, int nthreads, uint64_t* digests) {
  digest_job j;
  memset(&j, 0, sizeof j);
  j.out0 = out0;
  j.out1 = out1;
  j.offs = offs;
  j.n = n;
  j.b0 = b0;
  j.b1 = b1;
  j.digests = digests;
  if (nthreads < 1) nthreads = 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  if (!th) {
    digest_worker(&j);
    return;
  }
  for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, digest_worker, &j);
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(th);
}

typedef struct {
  const vox_config* cfg;
  const vox_chunk_coord* coords;
  const uint8_t* nbr_mask;
  int32_t n;
  int64_t index_base;
  uint64_t* counts;
  uint64_t* digests;
  volatile int64_t next;
  volatile int failed;
} gen_digest_job;

/* One chunk of or_gen_mesh_batch (the same generation, neighbour halo and emission), its
 * faces emitted into the worker's own buffers. */
static void* gen_digest_worker(void* arg) {
  gen_digest_job* j = (gen_digest_job*)arg;
  const vox_config* cfg = j->cfg;
  const int N = cfg->chunk_size;
  const size_t vox = (size_t)N * N * N;
  uint8_t* cubes = (uint8_t*)malloc(vox * 7);
  const size_t max_faces = (size_t)3 * vox + (size_t)6 * N * N;
  or_face* faces = j->digests ? (or_face*)malloc(sizeof(or_face) * max_faces) : NULL;
  const size_t b0 = cfg->layout == VOX_LAYOUT_INSTANCED ? sizeof(vox_instance_raw) : 4 * sizeof(vox_vertex);
  const size_t b1 = cfg->layout == VOX_LAYOUT_INSTANCED ? 0 : 6 * sizeof(uint32_t);
  uint8_t* o0 = j->digests ? (uint8_t*)malloc(b0 * max_faces) : NULL;
  uint8_t* o1 = j->digests && b1 ? (uint8_t*)malloc(b1 * max_faces) : NULL;
  if (!cubes || (j->digests && (!faces || !o0 || (b1 && !o1)))) {
    j->failed = 1;
    free(cubes);
    free(faces);
    free(o0);
    free(o1);
    return NULL;
  }
  for (;;) {
    const int64_t i = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
    if (i >= j->n) break;
    or_generate_cubes(cfg, j->coords[i], j->index_base + i, cubes);
    const uint8_t* adj[6] = {0, 0, 0, 0, 0, 0};
    uint8_t m = j->nbr_mask ? j->nbr_mask[i] : 0;
    if (cfg->gen.kind == VOX_GEN_BERNOULLI) m = 0; /* Bernoulli chunks are isolated */
    for (int d = 0; d < 6; ++d) {
      if (!((m >> d) & 1)) continue;
      if (d >= 4 && cfg->cull_mode != VOX_CULL_FULL6) continue;
      uint8_t* nb = cubes + vox * (size_t)(1 + d);
      or_generate_cubes(cfg, nbr_coord(j->coords[i], d), 0, nb);
      adj[d] = nb;
    }
    const int64_t cnt = or_cull_faces(N, cfg->cull_mode, cubes, adj, faces, faces ? (int64_t)max_faces : 0);
    j->counts[i] = (uint64_t)cnt;
    if (j->digests) {
      emit_faces(cfg, j->coords[i], faces, cnt, 0, o0, o1);
      j->digests[2 * i] = or_digest(o0, (uint64_t)cnt * b0);
      j->digests[2 * i + 1] = b1 ? or_digest(o1, (uint64_t)cnt * b1) : 0;
    }
  }
  free(cubes);
  free(faces);
  free(o0);
  free(o1);
  return NULL;
}

int or_gen_mesh_digests(const vox_config* cfg, const vox_chunk_coord* coords,
                        const uint8_t* nbr_mask, int32_t n, int64_t index_base, int nthreads,
                        uint64_t* counts, uint64_t* digests) {
  if (!valid_size(cfg->chunk_size) || n < 0 || !counts) return -1;
  gen_digest_job j;
  memset(&j, 0, sizeof j);
  j.cfg = cfg;
  j.coords = coords;
  j.nbr_mask = nbr_mask;
  j.n = n;
  j.index_base = index_base;
  j.counts = counts;
  j.digests = digests;
  if (nthreads < 1) nthreads = 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  if (!th) return -1;
  for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, gen_digest_worker, &j);
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(th);
  return j.failed ? -1 : 0;
}

/* ------------------------------------------------------------------------------------ */
/* Camera::update_global_matrix (src/camera.rs:41-51)                                    */
/* ------------------------------------------------------------------------------------ */

static void or_cross(const float a[3], const float b[3], float out[3]) {
  out[0] = a[1] * b[2] - a[2] * b[1];
  out[1] = a[2] * b[0] - a[0] * b[2];
  out[2] = a[0] * b[1] - a[1] * b[0];
}

static int or_normalize(float v[3]) {
  const float len = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (!(len > 0.0f)) return -1;
  for (int k = 0; k < 3; ++k) v[k] = v[k] / len;
  return 0;
}

int or_camera_global_matrix(const float eye[3], const float dir[3], float aspect, float fovy,
                            float znear, float zfar, float out[16]) {
  /* look_at_rh(eye, target = eye + dir, up = +y); target - eye is taken as dir itself */
  const float up[3] = {0.0f, 1.0f, 0.0f};
  float zaxis[3] = {-dir[0], -dir[1], -dir[2]}, xaxis[3], yaxis[3];
  if (or_normalize(zaxis)) return -1;
  or_cross(up, zaxis, xaxis);
  if (or_normalize(xaxis)) return -1;
  or_cross(zaxis, xaxis, yaxis);
  if (or_normalize(yaxis)) return -1;
  const float* rows[3] = {xaxis, yaxis, zaxis};
  float V[4][4];
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) V[r][c] = rows[r][c];
    V[r][3] = rows[r][0] * (-eye[0]) + rows[r][1] * (-eye[1]) + rows[r][2] * (-eye[2]);
  }
  V[3][0] = V[3][1] = V[3][2] = 0.0f;
  V[3][3] = 1.0f;
  /* new_perspective(aspect, fovy, znear, zfar) */
  float P[4][4];
  memset(P, 0, sizeof P);
  P[1][1] = 1.0f / tanf(fovy / 2.0f);
  P[0][0] = P[1][1] / aspect;
  P[2][2] = (zfar + znear) / (znear - zfar);
  P[2][3] = zfar * znear * 2.0f / (znear - zfar);
  P[3][2] = -1.0f;
  /* OPENGL_TO_WGPU_MATRIX as camera.rs:18-23 writes it (Matrix4::new takes rows) */
  static const float G[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 0.5f, 0}, {0, 0, 0.5f, 1}};
  float GP[4][4], M[4][4];
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 4; ++k) {
      float a = G[i][0] * P[0][k];
      for (int q = 1; q < 4; ++q) a = a + G[i][q] * P[q][k];
      GP[i][k] = a;
    }
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 4; ++k) {
      float a = GP[i][0] * V[0][k];
      for (int q = 1; q < 4; ++q) a = a + GP[i][q] * V[q][k];
      M[i][k] = a;
    }
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) out[c * 4 + r] = M[r][c];
  return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Frustum (src/frustum_culling.rs:16-85)                                                */
/* ------------------------------------------------------------------------------------ */

void or_frustum_planes(const float m[16], float planes[24]) {
  /* data[col][row] of the column-major matrix, frustum_culling.rs:54. */
#define D(c, r) m[(c) * 4 + (r)]
  float left[4], right[4], top[4], bottom[4], near_[4], far_[4];
  for (int c = 0; c < 4; ++c) {
    left[c] = D(c, 3) + D(c, 0);
    right[c] = D(c, 3) - D(c, 0);
    top[c] = D(c, 3) - D(c, 1);
    bottom[c] = D(c, 3) + D(c, 1);
    near_[c] = D(c, 3) + D(c, 2);
    far_[c] = D(c, 3) - D(c, 2);
  }
#undef D
  const float* order[6] = {near_, far_, left, right, top, bottom}; /* frustum_culling.rs:84 */
  for (int k = 0; k < 6; ++k)
    for (int c = 0; c < 4; ++c) planes[4 * k + c] = order[k][c];
}

int or_frustum_contains(const float planes[24], vox_chunk_coord c, int E) {
  const float px = (float)(c.x * E), py = (float)(c.y * E), pz = (float)(c.z * E);
  const float e = (float)E;
  const float corners[8][3] = {{px, py, pz},         {px + e, py, pz},
                               {px, py, pz + e},     {px + e, py, pz + e},
                               {px, py + e, pz},     {px + e, py + e, pz},
                               {px, py + e, pz + e}, {px + e, py + e, pz + e}};
  for (int k = 0; k < 8; ++k) {
    int inside = 1;
    for (int i = 0; i < 6; ++i) {
      const float* pl = planes + 4 * i;
      float dist = pl[0] * corners[k][0] + pl[1] * corners[k][1] + pl[2] * corners[k][2] + pl[3];
      if (dist < 0.0f) {
        inside = 0;
        break;
      }
    }
    if (inside) return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------------------ */
/* FP32 vs FP64 noise report                                                             */
/* ------------------------------------------------------------------------------------ */

int or_noise_error_stats(const vox_config* cfg, const vox_chunk_coord* coords, int32_t n,
                         double* max_abs_err, int64_t* near_threshold, int64_t* mismatches) {
  const int N = cfg->chunk_size;
  const vox_generator* g = &cfg->gen;
  if (!valid_size(N) || (g->kind != VOX_GEN_HEIGHTMAP && g->kind != VOX_GEN_DENSITY))
    return VOX_ERR_INVALID;
  uint8_t p[512];
  or_perm_init(g->seed, p);
  const size_t per = (size_t)N * N * N;
  double* v64 = (double*)malloc(sizeof(double) * per);
  float* v32 = (float*)malloc(sizeof(float) * per);
  if (!v64 || !v32) {
    free(v64);
    free(v32);
    return VOX_ERR_OOM;
  }
  double err = 0.0;
  int64_t mism = 0;
  /* pass 1: max error and mismatches */
  for (int pass = 0; pass < 2; ++pass) {
    int64_t near = 0;
    for (int32_t i = 0; i < n; ++i) {
      const int32_t ox = coords[i].x * N, oy = coords[i].y * N, oz = coords[i].z * N;
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z)
          for (int x = 0; x < N; ++x) {
            const int32_t wx = ox + x, wy = oy + y, wz = oz + z;
            double d64, t64;
            float d32;
            int s32, s64;
            if (g->kind == VOX_GEN_HEIGHTMAP) {
              d32 = height_f32(g, p, wx, wz);
              d64 = (double)g->base_height +
                    (double)g->amplitude * or_fbm2_f64(p, (double)wx, (double)wz, g->octaves,
                                                       (double)g->frequency,
                                                       (double)g->lacunarity, (double)g->gain);
              s32 = (float)wy < d32;
              s64 = (double)wy < d64;
              t64 = d64 - (double)wy; /* distance to the threshold */
            } else {
              d32 = density_f32(g, p, wx, wy, wz);
              double f = or_fbm3_f64(p, (double)wx, (double)wy, (double)wz, g->octaves,
                                     (double)g->frequency, (double)g->lacunarity,
                                     (double)g->gain);
              d64 = f - ((double)wy - (double)g->y_ref) * (double)g->y_scale;
              s32 = density_solid(g, d32);
              s64 = g->solid_below_zero ? (d64 < 0.0) : (d64 > 0.0);
              t64 = d64;
            }
            if (pass == 0) {
              double e = fabs((double)d32 - d64);
              if (e > err) err = e;
              if (s32 != s64) ++mism;
            } else if (fabs(t64) <= err) {
              ++near;
            }
          }
    }
    if (pass == 1) *near_threshold = near;
  }
  *max_abs_err = err;
  *mismatches = mism;
  free(v64);
  free(v32);
  return VOX_OK;
}

/* ------------------------------------------------------------------------------------ */
/* Headless rasteriser (project spec; vertex stage src/shaders/vertex.vert:22-27,        */
/* pipeline state src/renderer/pipeline.rs:36-45, clear src/renderer/renderer.rs:92-105) */
/* ------------------------------------------------------------------------------------ */

typedef struct {
  float x, y, z, w, u, v;
} or_sv;

static int or_to_screen(const float* m, const uint8_t* vertices, uint64_t g, int k, int W, int H,
                        or_sv* o) {
  float vx[5];
  memcpy(vx, vertices + g * 96 + (uint64_t)k * 24, sizeof vx);
  const float px = vx[0], py = vx[1], pz = vx[2];
  const float cx = ((m[0] * px + m[4] * py) + m[8] * pz) + m[12];
  const float cy = ((m[1] * px + m[5] * py) + m[9] * pz) + m[13];
  const float cz = ((m[2] * px + m[6] * py) + m[10] * pz) + m[14];
  const float cw = ((m[3] * px + m[7] * py) + m[11] * pz) + m[15];
  if (!(cw > 0.0f)) return 0;
  const float nx = cx / cw, ny = cy / cw, nz = cz / cw;
  o->x = (nx + 1.0f) * 0.5f * (float)W;
  o->y = (1.0f - ny) * 0.5f * (float)H;
  o->z = nz;
  o->w = cw;
  o->u = vx[3];
  o->v = vx[4];
  return 1;
}

static float or_edge(const or_sv* a, const or_sv* b, float px, float py) {
  return (b->x - a->x) * (py - a->y) - (b->y - a->y) * (px - a->x);
}

static int or_top_left(const or_sv* a, const or_sv* b) {
  const float dx = b->x - a->x, dy = b->y - a->y;
  return dy < 0.0f || (dy == 0.0f && dx > 0.0f);
}

static int or_tri_setup(const float* m, const uint8_t* vertices, const uint8_t* indices,
                        uint64_t g, int t, int W, int H, or_sv* v0, or_sv* v1, or_sv* v2,
                        float* area) {
  uint32_t ix[3];
  memcpy(ix, indices + g * 24 + (uint64_t)t * 12, sizeof ix);
  if (!or_to_screen(m, vertices, g, (int)(ix[0] & 3u), W, H, v0) ||
      !or_to_screen(m, vertices, g, (int)(ix[1] & 3u), W, H, v1) ||
      !or_to_screen(m, vertices, g, (int)(ix[2] & 3u), W, H, v2))
    return 0;
  float a = or_edge(v0, v1, v2->x, v2->y);
  if (!(a < 0.0f)) return 0; /* back face (clockwise in NDC) or degenerate */
  const or_sv tmp = *v1;
  *v1 = *v2;
  *v2 = tmp;
  *area = -a;
  return 1;
}

static uint32_t or_float_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, sizeof u);
  return u;
}

static void or_shade(uint32_t tex, float u, float v, uint8_t* rgba) {
  static const float pal[4][3] = {{0.45f, 0.55f, 0.25f}, {0.45f, 0.32f, 0.20f},
                                  {0.30f, 0.70f, 0.25f}, {0.60f, 0.60f, 0.60f}};
  const float* c = pal[tex & 3u];
  const int cu = (int)floorf(u * 4.0f), cv = (int)floorf(v * 4.0f);
  const float f = ((cu + cv) & 1) ? 0.85f : 1.0f;
  for (int k = 0; k < 3; ++k) rgba[k] = (uint8_t)(c[k] * f * 255.0f + 0.5f);
  rgba[3] = 255;
}

void or_raster(const float m[16], const void* vertices_, const void* indices_, uint64_t faces,
               int W, int H, const uint32_t tex[6], uint8_t* rgba) {
  const uint8_t* vertices = (const uint8_t*)vertices_;
  const uint8_t* indices = (const uint8_t*)indices_;
  const size_t npx = (size_t)W * (size_t)H;
  uint64_t* keys = (uint64_t*)malloc(npx * sizeof(uint64_t));
  if (!keys) return;
  for (size_t i = 0; i < npx; ++i) keys[i] = ~0ull;
  for (uint64_t tri = 0; tri < 2 * faces; ++tri) {
    or_sv v0, v1, v2;
    float area;
    if (!or_tri_setup(m, vertices, indices, tri >> 1, (int)(tri & 1), W, H, &v0, &v1, &v2, &area))
      continue;
    const float fx0 = fminf(fminf(v0.x, v1.x), v2.x), fx1 = fmaxf(fmaxf(v0.x, v1.x), v2.x);
    const float fy0 = fminf(fminf(v0.y, v1.y), v2.y), fy1 = fmaxf(fmaxf(v0.y, v1.y), v2.y);
    if (fx1 < 0.0f || fy1 < 0.0f || fx0 > (float)W || fy0 > (float)H) continue;
    int x0 = (int)floorf(fx0), x1 = (int)ceilf(fx1), y0 = (int)floorf(fy0), y1 = (int)ceilf(fy1);
    if (x0 < 0) x0 = 0;
    if (y0 < 0) y0 = 0;
    if (x1 > W - 1) x1 = W - 1;
    if (y1 > H - 1) y1 = H - 1;
    const int tl0 = or_top_left(&v1, &v2), tl1 = or_top_left(&v2, &v0), tl2 = or_top_left(&v0, &v1);
    for (int py = y0; py <= y1; ++py) {
      const float sy = (float)py + 0.5f;
      for (int px = x0; px <= x1; ++px) {
        const float sx = (float)px + 0.5f;
        const float w0 = or_edge(&v1, &v2, sx, sy), w1 = or_edge(&v2, &v0, sx, sy),
                    w2 = or_edge(&v0, &v1, sx, sy);
        const int in = (w0 > 0.0f || (w0 == 0.0f && tl0)) && (w1 > 0.0f || (w1 == 0.0f && tl1)) &&
                       (w2 > 0.0f || (w2 == 0.0f && tl2));
        if (!in) continue;
        float z = ((w0 * v0.z + w1 * v1.z) + w2 * v2.z) / area;
        if (!(z >= 0.0f && z < 1.0f)) continue;
        z = z + 0.0f;
        const uint64_t key = ((uint64_t)or_float_bits(z) << 32) | (uint64_t)(uint32_t)tri;
        uint64_t* k = keys + (size_t)py * W + px;
        if (key < *k) *k = key;
      }
    }
  }
  for (size_t i = 0; i < npx; ++i) {
    uint8_t* o = rgba + 4 * i;
    if (keys[i] == ~0ull) {
      o[0] = (uint8_t)(0.1f * 255.0f + 0.5f);
      o[1] = (uint8_t)(0.2f * 255.0f + 0.5f);
      o[2] = (uint8_t)(0.3f * 255.0f + 0.5f);
      o[3] = 255;
      continue;
    }
    const uint64_t tri = keys[i] & 0xFFFFFFFFull, g = tri >> 1;
    or_sv v0, v1, v2;
    float area;
    or_tri_setup(m, vertices, indices, g, (int)(tri & 1), W, H, &v0, &v1, &v2, &area);
    const float sx = (float)(i % (size_t)W) + 0.5f, sy = (float)(i / (size_t)W) + 0.5f;
    const float w0 = or_edge(&v1, &v2, sx, sy), w1 = or_edge(&v2, &v0, sx, sy),
                w2 = or_edge(&v0, &v1, sx, sy);
    const float b0 = w0 / v0.w, b1 = w1 / v1.w, b2 = w2 / v2.w;
    const float den = (b0 + b1) + b2;
    const float u = ((b0 * v0.u + b1 * v1.u) + b2 * v2.u) / den;
    const float v = ((b0 * v0.v + b1 * v1.v) + b2 * v2.v) / den;
    uint32_t slot;
    memcpy(&slot, vertices + g * 96 + 20, sizeof slot);
    or_shade(tex[slot < 6u ? slot : 0u], u, v, o);
  }
  free(keys);
}
