/*
 * vox_oracle.h — CPU oracle for the chunk generation / meshing / frustum path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's CPU
 * algorithm (Blatko1/wgpu-voxel-engine, Rust) that the CUDA path's outputs are compared
 * against in the tests and, timed on the host cores, the CPU baseline. Nothing in the product links,
 * loads or calls it: only tests/, __graft_entry__.smoke() and bench.py's CPU legs do.
 *
 * Parity status: UNPINNED. The reference ships no tests, golden vectors or fixtures,
 * and it cannot be built in this environment (Rust, crates not vendored). Its noise
 * comes from the third-party crate simdnoise 3.1.6 (Cargo.lock:1802-1805, called at
 * src/perlin_noise.rs:5-22) and its rotation/matrix arithmetic from nalgebra 0.29.0
 * (Cargo.lock:1118-1121, called at src/quad.rs:19-38,49); neither is present here.
 * The oracle is therefore checked against known answers derived by hand from
 * src/chunk.rs:59-245 (face counts, emission order, neighbour rules) and against
 * committed golden digests it produced itself (tests/golden/).
 *
 * Compile with -O2 -ffp-contract=off and without -ffast-math: every float expression
 * is evaluated in the written order, one rounding per operation.
 */
#ifndef VOX_ORACLE_H
#define VOX_ORACLE_H

#include <stdint.h>
#include "../include/voxgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* splitmix64 (Steele, Lea, Flood 2014): state += golden gamma, then the mix. */
uint64_t or_splitmix64_next(uint64_t* state);
/* Seeded permutation: Fisher-Yates over 0..255 driven by splitmix64(seed), doubled to 512. */
void or_perm_init(uint64_t seed, uint8_t p[512]);

/* Gradient coefficients (gx, gy, gz) of hash h (Perlin 2002's 12 edge directions). */
void or_grad_coef(int h, float g[3]);
/* Perlin improved noise (SIGGRAPH 2002), FP32 and FP64, with the gradient evaluated as
 * ((gx*x + gy*y) + gz*z). noise2 is the z = 0 slice evaluated bilinearly (the z lerp with
 * w = fade(0) = 0 and the gz*z term are dropped). */
float or_noise2_f32(const uint8_t* p, float x, float y);
float or_noise3_f32(const uint8_t* p, float x, float y, float z);
double or_noise2_f64(const uint8_t* p, double x, double y);
double or_noise3_f64(const uint8_t* p, double x, double y, double z);
/* fBm: sum_o amp_o * noise(x * f_o), f_0 = frequency, f_{o+1} = f_o * lacunarity,
 * amp_0 = 1, amp_{o+1} = amp_o * gain; all products and sums in that order. */
float or_fbm2_f32(const uint8_t* p, float x, float y, int octaves, float freq, float lac, float gain);
float or_fbm3_f32(const uint8_t* p, float x, float y, float z, int octaves, float freq, float lac,
                  float gain);
double or_fbm2_f64(const uint8_t* p, double x, double y, int octaves, double freq, double lac,
                   double gain);
double or_fbm3_f64(const uint8_t* p, double x, double y, double z, int octaves, double freq,
                   double lac, double gain);

/* Chunk::new / generate_terrain (src/chunk.rs:21-46): one byte per voxel at
 * x + N*z + N*N*y, GRASS (0) when solid, AIR (2) otherwise. */
int or_generate_cubes(const vox_config* cfg, vox_chunk_coord coord, int64_t chunk_index,
                      uint8_t* cubes);
void or_cubes_to_occ(int n_size, const uint8_t* cubes, uint32_t* occ);
void or_occ_to_cubes(int n_size, const uint32_t* occ, uint8_t* cubes);

/* One emitted face: local voxel (x, y, z) and emission direction
 * 0 LEFT, 1 RIGHT, 2 BACK, 3 FRONT, 4 DOWN, 5 UP (the order of chunk.rs:76-240). */
typedef struct or_face {
  uint8_t x, y, z, dir;
} or_face;

/* cull_unseen_triangles (src/chunk.rs:59-245). adj[0..3] = -x, +x, -z, +z neighbour cubes
 * or NULL (not loaded); adj[4..5] = -y, +y, used only with VOX_CULL_FULL6. Returns the
 * face count; writes at most cap faces (faces may be NULL to count only). */
int64_t or_cull_faces(int n_size, int cull_mode, const uint8_t* cubes, const uint8_t* const adj[6],
                      or_face* faces, int64_t cap);

/* Quad::new rotation (src/quad.rs:14-46) for emission direction dir, computed the way
 * the reference computes it per face: Euler angles in degrees -> to_radians -> sinf/cosf
 * -> R = Rz(yaw) * Ry(pitch) * Rx(roll). R is row-major R[row][col]. */
void or_face_rotation(int dir, float R[3][3]);
/* Quad::to_raw (src/quad.rs:47-54): T * R as 4x4 homogeneous matrices. */
void or_instance_raw(int dir, int32_t wx, int32_t wy, int32_t wz, uint32_t texture_index,
                     vox_instance_raw* out);
/* vertex.vert:22-27 applied to quad::VERTICES, plus the 6 indices of quad::INDICES. */
void or_face_vertices(int dir, int32_t wx, int32_t wy, int32_t wz, uint32_t local_face,
                      vox_vertex out_v[4], uint32_t out_i[6]);
/* Emission-direction -> face slot (texture column): L0 R1 Bk2 F3 D5 U4. */
int or_dir_slot(int dir);

/* Chunk::create_mesh for one chunk: cull + emit in the configured layout. Returns the
 * face count; writes at most cap faces. out1 is the index array (vertex layout) or unused. */
int64_t or_mesh_chunk(const vox_config* cfg, vox_chunk_coord coord, const uint8_t* cubes,
                      const uint8_t* const adj[6], void* out0, void* out1, int64_t cap);

/* Whole batch: chunk i is generated from coords[i] (Bernoulli: index base + i); for every
 * bit d set in nbr_mask[i] (NULL = none) the neighbour chunk is generated from its
 * coordinate and used as the halo. Output like vox_gen_mesh_batch. Returns the total. */
int64_t or_gen_mesh_batch(const vox_config* cfg, const vox_chunk_coord* coords,
                          const uint8_t* nbr_mask, int32_t n, int64_t index_base, void* out0,
                          void* out1, int64_t cap, uint64_t* face_offsets);

/* CPU baseline: the reference's pool work for a batch, on nthreads threads, one chunk per
 * task (uvth pool, src/chunk_builder.rs:80-84): Chunk::new for every chunk, then
 * create_mesh with the neighbours of the batch, each mesh collected into its own buffer.
 * Returns the total face count (-1 on allocation failure). */
int64_t or_baseline_run(const vox_config* cfg, const vox_chunk_coord* coords,
                        const uint8_t* nbr_mask, int32_t n, int64_t index_base, int nthreads);

/* 64-bit digest of a byte run (test bookkeeping only): every 8-byte little-endian word w_k
 * (the tail zero-padded) is folded in as h = mix(h ^ mix(w_k + k * golden gamma)), with
 * mix = the splitmix64 finaliser and h starting at the length. */
uint64_t or_digest(const void* bytes, uint64_t len);
/* Per-chunk digests of a meshed batch already in memory: chunk i's out0 bytes
 * [offs[i] * b0, offs[i + 1] * b0) -> digests[2i], its out1 bytes (b1 per face; none when
 * b1 = 0) -> digests[2i + 1]. nthreads threads. */
void or_chunk_digests(const void* out0, const void* out1, const uint64_t* offs, int32_t n,
                      int32_t b0, int32_t b1, int nthreads, uint64_t* digests);
/* or_gen_mesh_batch chunk by chunk on nthreads threads, keeping only per-chunk results:
 * counts[i] = chunk i's face count and, when digests is not NULL, the or_chunk_digests
 * pair of its out0 and out1 bytes (chunk-local indices, so a chunk's bytes do not depend
 * on the rest of the batch). Returns 0, or -1 on a bad size or an allocation failure. */
int or_gen_mesh_digests(const vox_config* cfg, const vox_chunk_coord* coords,
                        const uint8_t* nbr_mask, int32_t n, int64_t index_base, int nthreads,
                        uint64_t* counts, uint64_t* digests);

/* Camera::update_global_matrix (src/camera.rs:41-51):
 * OPENGL_TO_WGPU_MATRIX * new_perspective(aspect, fovy, znear, zfar) * look_at_rh(eye,
 * eye + dir, +y), column-major. look_at_rh: z = normalize(eye - target), x = normalize(up x
 * z), y = normalize(z x x); view rows x, y, z with translation -(row . eye). Perspective
 * (OpenGL convention): m11 = 1 / tan(fovy / 2), m00 = m11 / aspect, m22 = (zfar + znear) /
 * (znear - zfar), m23 = zfar * znear * 2 / (znear - zfar), m32 = -1. Returns 0, or -1 for a
 * degenerate direction. */
int or_camera_global_matrix(const float eye[3], const float dir[3], float aspect, float fovy,
                            float znear, float zfar, float out_colmajor[16]);

/* Frustum (src/frustum_culling.rs:16-85). */
void or_frustum_planes(const float m_colmajor[16], float planes[24]);
int or_frustum_contains(const float planes[24], vox_chunk_coord coord, int chunk_extent);

/* Headless rasteriser (the GPU's vox_raster restated, for visual regression images):
 * vertex-layout faces through the global matrix (src/shaders/vertex.vert:22-27), back faces
 * culled with counter-clockwise fronts, depth Less against 1.0
 * (src/renderer/pipeline.rs:36-45), clear colour (0.1, 0.2, 0.3)
 * (src/renderer/renderer.rs:92-99), top-left fill rule at pixel centres, perspective-correct
 * (u, v) and a procedural palette per texture index. Writes width x height RGBA8. */
void or_raster(const float m_colmajor[16], const void* vertices, const void* indices,
               uint64_t faces, int width, int height, const uint32_t tex[6], uint8_t* rgba);

/* Noise precision report: FP32 generator values against FP64 at every voxel of the
 * chunks (density: d; heightmap: the column heights). max_abs_err = max |f32 - f64|;
 * near_threshold = voxels whose FP64 value lies within max_abs_err of the solid/air
 * threshold; mismatches = voxels whose solid bit differs between FP32 and FP64. */
int or_noise_error_stats(const vox_config* cfg, const vox_chunk_coord* coords, int32_t n,
                         double* max_abs_err, int64_t* near_threshold, int64_t* mismatches);

#ifdef __cplusplus
}
#endif

#endif /* VOX_ORACLE_H */
