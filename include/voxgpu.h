/*
 * voxgpu.h — C ABI of the GB300 chunk generation, meshing and chunk-frustum path.
 *
 * This is the drop-in boundary for the data-parallel core of the voxel engine
 * (Blatko1/wgpu-voxel-engine). The reference has no FFI of its own: the path sits
 * behind crate-internal Rust methods, and every entry point below names the
 * reference function it replaces (file:line inside that project).
 *
 *   Chunk::new / generate_terrain       src/chunk.rs:21-46        -> vox_generate, vox_generate_slots,
 *                                                                    vox_occ_to_cubes
 *   Chunk::create_mesh / cull_unseen... src/chunk.rs:48-245       -> vox_mesh, vox_mesh_batch
 *   Quad::new / Quad::to_raw            src/quad.rs:14-54         -> emitted records (vox_instance_raw)
 *   vertex.vert instance expansion      src/shaders/vertex.vert:22-27 -> vox_vertex layout
 *   ChunkGenerator (pool closure)       src/chunk_builder.rs:80-84 -> vox_gen_mesh_batch
 *   Frustum::matrix_to_planes           src/frustum_culling.rs:47-85 -> vox_frustum_planes
 *   Frustum::contains                   src/frustum_culling.rs:16-40 -> vox_frustum_cull
 *   World::render (draw loop)           src/world.rs:24-40        -> vox_draw_list
 *   ChunkGenerator per-tick dispatch    src/chunk_builder.rs:69-132 -> vox_graph_capture/launch
 *   vertex.vert + pipeline (render)     src/renderer/pipeline.rs:36-45 -> vox_raster (headless)
 *
 * Conventions
 *  - Every call returns an int status (VOX_OK = 0, see vox_status).
 *  - Pointers named d_* are device pointers, h_* are host pointers.
 *  - Calls taking device pointers are asynchronous on the context's stream. Errors
 *    found on the device (a bounded wait that gave up, an output that did not fit)
 *    are latched in the context and returned by vox_ctx_sync().
 *  - One context serialises its own calls with a mutex; give each host thread its
 *    own context (and stream) for concurrent work.
 *  - No call aborts the process: a failed CUDA call becomes VOX_ERR_CUDA and the
 *    message is kept for vox_ctx_last_error().
 */
#ifndef VOXGPU_H
#define VOXGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VOX_ABI_VERSION 1

/* Status codes. The reference panics (unwrap) where these are returned. */
enum vox_status {
  VOX_OK = 0,
  VOX_ERR_INVALID = 1,   /* bad argument or unsupported configuration */
  VOX_ERR_OOM = 2,       /* device or pinned host allocation failed */
  VOX_ERR_CUDA = 3,      /* a CUDA runtime call or kernel launch failed */
  VOX_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up (no hang, no trap) */
  VOX_ERR_CAPACITY = 5,  /* output capacity too small; the required size is still returned */
  VOX_ERR_NO_DEVICE = 6  /* no CUDA device visible */
};

/* ChunkCoord3D (src/coordinate.rs:146-151). World origin of a chunk = coord * chunk_size. */
typedef struct vox_chunk_coord {
  int32_t x, y, z;
} vox_chunk_coord;

/* Generator kinds. The reference's own noise (simdnoise fbm_3d, src/perlin_noise.rs:5-22)
 * is a third-party crate that is not available; these are project-defined terrain
 * specs built on Perlin's improved noise (2002). */
enum vox_gen_kind {
  VOX_GEN_HEIGHTMAP = 0, /* solid iff world_y < base_height + amplitude * fbm2(x*f, z*f) */
  VOX_GEN_DENSITY = 1,   /* d = fbm3(x*f, y*f, z*f) - (world_y - y_ref) * y_scale; solid iff d > 0
                            (or d < 0 with solid_below_zero = 1, the chunk.rs:38 rule) */
  VOX_GEN_BERNOULLI = 2  /* solid iff low bit of draw i of splitmix64(seed ^ chunk_index),
                            i = x + N*z + N*N*y; chunks have no neighbours */
};

/* Face culling modes. */
enum vox_cull_mode {
  VOX_CULL_REFERENCE = 0, /* chunk.rs:59-245: lateral (+-x, +-z) neighbour halo only;
                             faces on the y borders are always emitted */
  VOX_CULL_FULL6 = 1      /* also consult the +-y neighbours (not a reference behaviour) */
};

/* Output layouts. */
enum vox_layout {
  VOX_LAYOUT_VERTEX = 0,   /* 4 vox_vertex + 6 u32 indices per face (120 B/face) */
  VOX_LAYOUT_INSTANCED = 1 /* 1 vox_instance_raw per face (68 B/face), the reference's ChunkMesh data */
};

/* Face slots, in the reference's TEXTURE_INDEX_LIST column order (src/texture.rs:240-243;
 * chunk.rs passes texture_index[0..5] for LEFT, RIGHT, BACK, FRONT, UP, DOWN). */
enum vox_face_slot {
  VOX_FACE_LEFT = 0,  /* -x */
  VOX_FACE_RIGHT = 1, /* +x */
  VOX_FACE_BACK = 2,  /* -z */
  VOX_FACE_FRONT = 3, /* +z */
  VOX_FACE_UP = 4,    /* +y */
  VOX_FACE_DOWN = 5   /* -y */
};

typedef struct vox_generator {
  int32_t kind;            /* vox_gen_kind */
  int32_t octaves;         /* fBm octaves (>= 1) */
  uint64_t seed;           /* permutation seed (noise) or stream seed (Bernoulli) */
  float frequency;         /* base frequency, cycles per voxel */
  float lacunarity;        /* frequency multiplier per octave */
  float gain;              /* amplitude multiplier per octave */
  float amplitude;         /* heightmap amplitude */
  float base_height;       /* heightmap base height */
  float y_ref;             /* density: reference height */
  float y_scale;           /* density: height gradient */
  int32_t solid_below_zero;/* density: 1 -> solid iff d < 0 */
} vox_generator;

typedef struct vox_config {
  int32_t chunk_size;         /* N: 8, 16, 32 (reference) or 64 */
  int32_t cull_mode;          /* vox_cull_mode */
  int32_t layout;             /* vox_layout */
  uint32_t texture_index[6];  /* per face slot; the reference's GRASS row is {0,0,0,0,2,1} */
  vox_generator gen;
} vox_config;

/* De-instanced vertex: position = instance * vec4(quad_vertex, 1) (vertex.vert:22-27),
 * tex_coords from quad::VERTICES (src/quad.rs:66-87), face = vox_face_slot. 24 bytes. */
typedef struct vox_vertex {
  float position[3];
  float tex_coords[2];
  uint32_t face;
} vox_vertex;

/* InstanceRaw (src/renderer/instance.rs:1-6): column-major T*R and the texture index. 68 bytes. */
typedef struct vox_instance_raw {
  float t_matrix[4][4];
  uint32_t texture_index;
} vox_instance_raw;

typedef struct vox_ctx vox_ctx;

/* Sizes a caller needs to allocate buffers. */
typedef struct vox_sizes {
  uint32_t occ_words_per_chunk;   /* u32 words of the occupancy bitmask of one chunk */
  uint32_t bytes_per_face_out0;   /* 96 (4 vertices) or 68 (instance) */
  uint32_t bytes_per_face_out1;   /* 24 (6 indices) or 0 */
  uint32_t max_faces_per_chunk;   /* upper bound of faces one chunk can emit */
} vox_sizes;

/* ---- context ------------------------------------------------------------------------ */

/* Validates cfg and creates a context on the current CUDA device. `stream` is a
 * cudaStream_t to run on (NULL: the context creates its own non-blocking stream). */
int vox_ctx_create(const vox_config* cfg, void* stream, vox_ctx** out);
int vox_ctx_destroy(vox_ctx* ctx);
/* Waits for the context's stream and returns the first latched device-side status. */
int vox_ctx_sync(vox_ctx* ctx);
/* The context's stream (cudaStream_t). */
void* vox_ctx_stream(vox_ctx* ctx);
/* Last error message of this context (empty string if none). */
const char* vox_ctx_last_error(vox_ctx* ctx);
const char* vox_status_string(int status);
int vox_abi_version(void);
int vox_query_sizes(const vox_config* cfg, vox_sizes* out);

/* ---- Chunk::new ---------------------------------------------------------------------- */

/* Fills occupancy bitmasks for n chunks (src/chunk.rs:27-46). Layout per chunk: rows
 * indexed r = y*N + z, each row max(1, N/32) u32 words, bit x of the row = voxel
 * (x, y, z) solid. `chunk_index_base` numbers the chunks for VOX_GEN_BERNOULLI
 * (chunk i uses seed ^ (chunk_index_base + i)); other generators ignore it. */
int vox_generate(vox_ctx* ctx, const vox_chunk_coord* d_coords, int32_t n,
                 int64_t chunk_index_base, uint32_t* d_occ);

/* vox_generate into a resident pool (the chunks that World.chunks keeps, src/world.rs:14-22,
 * for later neighbour rebuilds): chunk i's occupancy goes to slot d_slots[i] of d_occ_pool
 * (pool_slots slots of occ_words_per_chunk words). A slot outside the pool writes nothing
 * and makes vox_ctx_sync() return VOX_ERR_INVALID. */
int vox_generate_slots(vox_ctx* ctx, const vox_chunk_coord* d_coords, int32_t n,
                       int64_t chunk_index_base, uint32_t* d_occ_pool, int32_t pool_slots,
                       const int32_t* d_slots);

/* Expands occupancy bitmasks to the reference's Vec<Cube> bytes (src/chunk.rs:35-45):
 * one byte per voxel at x + N*z + N*N*y, GRASS = 0 when solid, AIR = 2 otherwise. */
int vox_occ_to_cubes(vox_ctx* ctx, const uint32_t* d_occ, int32_t n, uint8_t* d_cubes);
/* Packs reference Vec<Cube> bytes into occupancy bitmasks (solid iff byte != AIR). */
int vox_cubes_to_occ(vox_ctx* ctx, const uint8_t* d_cubes, int32_t n, uint32_t* d_occ);

/* ---- Chunk::create_mesh ---------------------------------------------------------------- */

/* Plain per-chunk mesher: one chunk, one launch (src/chunk.rs:48-245 + quad.rs:47-54).
 * d_nbr[d] is the occupancy of the neighbour in direction d (0 -x, 1 +x, 2 -z, 3 +z,
 * 4 -y, 5 +y; the order of chunk_builder.rs:134-169 then -y, +y) or NULL if it is not
 * loaded. Faces beyond cap_faces are not written; *d_face_count gets the full count
 * and vox_ctx_sync() returns VOX_ERR_CAPACITY. */
int vox_mesh(vox_ctx* ctx, const uint32_t* d_occ, const uint32_t* const d_nbr[6],
             vox_chunk_coord coord, void* d_out0, void* d_out1, uint64_t cap_faces,
             uint64_t* d_face_count);

/* Batched mesher over resident occupancy (the neighbour-rebuild path,
 * src/chunk_builder.rs:89-112): chunk i reads slot d_slots[i] of d_occ_pool (pool_slots
 * slots of occ_words_per_chunk words) and neighbour slots d_nbr_slots[6*i + d]
 * (-1 = not loaded; d_nbr_slots may be NULL). Output of chunk i starts at face
 * d_face_offsets[i]; d_face_offsets[n] is the total. Indices are chunk-local. A slot
 * outside the pool makes vox_ctx_sync() return VOX_ERR_INVALID. */
int vox_mesh_batch(vox_ctx* ctx, const uint32_t* d_occ_pool, int32_t pool_slots,
                   const int32_t* d_slots, const int32_t* d_nbr_slots,
                   const vox_chunk_coord* d_coords, int32_t n, void* d_out0, void* d_out1,
                   uint64_t cap_faces, uint64_t* d_face_offsets);

/* Fused generation + meshing of n chunks in one persistent launch (the pool closure of
 * src/chunk_builder.rs:80-84 for a whole batch). d_nbr_mask[i] bit d says that the
 * neighbour of chunk i in direction d is loaded (its halo is regenerated from the
 * generator); NULL means no neighbour is loaded. Output as in vox_mesh_batch. */
int vox_gen_mesh_batch(vox_ctx* ctx, const vox_chunk_coord* d_coords, const uint8_t* d_nbr_mask,
                       int32_t n, int64_t chunk_index_base, void* d_out0, void* d_out1,
                       uint64_t cap_faces, uint64_t* d_face_offsets);

/* No counterpart in the reference. vox_gen_mesh_batch for callers that cannot allocate
 * device memory: hosts that own all device memory through their own pool, or code that
 * must not allocate once it runs. No context is needed and nothing is allocated (no
 * cudaMalloc, cudaFree or allocating library routine): the caller passes the inputs and
 * outputs as for vox_gen_mesh_batch, the per-config tables travel as a kernel parameter,
 * and the kernel's scratch is a static array inside the library (about 129 KiB, held by
 * every GPU that loads the library until the process exits). At most 16384 chunks per
 * call; larger n returns VOX_ERR_INVALID. Runs on `stream` (a cudaStream_t, NULL = the
 * default stream) and waits for it; returns the device-side status (VOX_ERR_CAPACITY,
 * VOX_ERR_TIMEOUT). Every call is synchronous, so it must never be made on a stream that is
 * being captured (it returns VOX_ERR_INVALID there without queueing work). The first call
 * on a device looks up the scratch array's address (cudaGetSymbolAddress) and keeps it for
 * the life of the process: do not use the call across cudaDeviceReset. All calls share the
 * scratch: calls whose work overlaps on the GPU race. */
int vox_gen_mesh_batch_noalloc(const vox_config* cfg, void* stream,
                               const vox_chunk_coord* d_coords, const uint8_t* d_nbr_mask,
                               int32_t n, int64_t chunk_index_base, void* d_out0, void* d_out1,
                               uint64_t cap_faces, uint64_t* d_face_offsets);

/* Same as vox_gen_mesh_batch with host buffers. Synchronous. When h_out0 (h_out1) and
 * h_face_offsets are page-locked (vox_host_alloc, cudaMallocHost, cudaHostRegister) and
 * 16-byte aligned, the kernel writes the faces and offsets straight into them (over
 * NVLink-C2C on Grace systems) and page-locked inputs are read in place; otherwise the
 * inputs are copied in and exactly the emitted faces and the offsets are copied back. */
int vox_gen_mesh_host(vox_ctx* ctx, const vox_chunk_coord* h_coords, const uint8_t* h_nbr_mask,
                      int32_t n, int64_t chunk_index_base, void* h_out0, void* h_out1,
                      uint64_t cap_faces, uint64_t* h_face_offsets);

/* ---- Tuning ------------------------------------------------------------------------------ */

/* Launch shape of the meshing kernels. */
typedef struct vox_tuning {
  int32_t threads;     /* CTA size; each chunk size has two (8: 32/64, 16: 128/256,
                          32: 256/512, 64: 512/1024) */
  int32_t stage_faces; /* 0: every lane stores its face records straight to global memory;
                          32: each warp stages 32 faces at a time in one shared-memory
                          buffer and sends them with a TMA bulk copy; 64: the same with
                          two buffers per warp (one fills while the other is sent) */
  int32_t ctas_per_sm; /* resident CTAs per SM of the persistent grid; 0 = as many as fit */
  int32_t schedule;    /* VOX_SCHEDULE_LOOKBACK, VOX_SCHEDULE_PHASED or VOX_SCHEDULE_OVERLAP */
  int32_t slab_chunks; /* output slab: chunks per launch. A larger batch is meshed in
                          consecutive launches of this many chunks, each writing its slab of
                          the output right after the previous one's (same bytes and offsets
                          as one launch); 0 = the whole batch in one launch */
  int32_t halo_staging;/* 0: each chunk's lateral halo is regenerated in shared memory by the
                          fused launch; 1: every chunk of the batch is generated once into an
                          occupancy pool (and, for every loaded neighbour outside the batch,
                          the one plane its batch neighbour reads), and the chunks are meshed
                          from the pool with each halo plane read from the neighbour's
                          occupancy, the neighbours being found by a hash lookup of the
                          batch's coordinates. Same bytes either way; mode 1
                          needs chunk coordinates within [-2^20, 2^20) (otherwise
                          VOX_ERR_INVALID from vox_ctx_sync) and applies to outputs in device
                          memory: vox_gen_mesh_host with page-locked outputs keeps mode 0,
                          whose emission overlaps generation behind the host link */
} vox_tuning;

/* Schedules of the fused batch kernel (all write the same bytes):
 * LOOKBACK: one pass; each chunk's output offset comes from a decoupled look-back over
 *   its predecessors' face counts.
 * PHASED: a cooperative launch in three phases: generate and count every chunk (the
 *   occupancy is kept in a context-owned scratch), scan the counts once, then emit every
 *   chunk at its known offset. No chunk waits for another inside a phase.
 * OVERLAP: the phases of PHASED without the grid barrier: each chunk's total is published
 *   as soon as it is counted, and emission takes a chunk's offset from a decoupled
 *   look-back over the published totals, so emission overlaps the end of generation. */
enum { VOX_SCHEDULE_LOOKBACK = 0, VOX_SCHEDULE_PHASED = 1, VOX_SCHEDULE_OVERLAP = 2 };

int vox_ctx_get_tuning(vox_ctx* ctx, vox_tuning* out);
int vox_ctx_set_tuning(vox_ctx* ctx, const vox_tuning* tuning);

/* Autotuner: times every candidate launch shape (schedule x CTA size x staging window x
 * CTAs per SM) on the given batch with vox_gen_mesh_batch (same arguments; iters launches each),
 * then, for the fastest shape, the output slab (the whole batch, or halves, quarters and
 * eighths of it while a launch keeps at least two waves of the grid), then the halo staging
 * (regenerated or staged from a pool); keeps the fastest in the context and returns it in
 * *out. The outputs of every candidate are identical; the buffers hold the last run's
 * result. */
int vox_autotune(vox_ctx* ctx, const vox_chunk_coord* d_coords, const uint8_t* d_nbr_mask,
                 int32_t n, int64_t chunk_index_base, void* d_out0, void* d_out1,
                 uint64_t cap_faces, uint64_t* d_face_offsets, int32_t iters, vox_tuning* out);

/* Self-test of the bounded device-side wait: runs one look-back whose predecessor never
 * publishes. Returns VOX_ERR_TIMEOUT after spin_limit polls (no hang, no trap) and leaves
 * the context usable. */
int vox_selftest_lookback_timeout(vox_ctx* ctx, int32_t spin_limit);

/* ---- Headless rasteriser ---------------------------------------------------------------- */

/* Renders vertex-layout faces (d_vertices: 96 B per face, d_indices: 6 u32 per face) into
 * an RGBA8 image of width x height, for visual regression: gl_Position = view_proj *
 * vertex (src/shaders/vertex.vert:22-27), counter-clockwise front faces with back faces
 * culled and depth test Less against a clear depth of 1.0
 * (src/renderer/pipeline.rs:36-45), clear colour (0.1, 0.2, 0.3)
 * (src/renderer/renderer.rs:92-99), pixel centres at +0.5 with the top-left fill rule,
 * perspective-correct texture coordinates. The texture images are replaced by a
 * procedural palette per texture index with a 4x4 checker in (u, v). Triangles with a
 * vertex behind the camera (clip w <= 0) are dropped (no near-plane clipping).
 * d_depth_keys is width x height u64 of scratch. Requires the vertex layout and
 * faces < 2^31. Equal inputs give equal bytes in any execution order. */
int vox_raster(vox_ctx* ctx, const float view_proj_colmajor[16], const void* d_vertices,
               const void* d_indices, uint64_t faces, int32_t width, int32_t height,
               uint64_t* d_depth_keys, uint8_t* d_rgba);

/* ---- CUDA graph replay of the fused batch ---------------------------------------------- */

/* One vox_gen_mesh_batch launch (same arguments, the context's tuning at capture time)
 * captured as a CUDA graph. Replaces the per-tick dispatch of ChunkGenerator
 * (src/chunk_builder.rs:69-132) when the same batch buffers are refilled every tick: the
 * caller rewrites the contents of d_coords / d_nbr_mask in place and calls
 * vox_graph_launch, which replays the launch on the context's stream without any
 * per-launch host work. The graph owns its scratch; the context must outlive it.
 * Device-side errors are latched in the context (vox_ctx_sync). */
typedef struct vox_graph vox_graph;
int vox_graph_capture(vox_ctx* ctx, const vox_chunk_coord* d_coords, const uint8_t* d_nbr_mask,
                      int32_t n, int64_t chunk_index_base, void* d_out0, void* d_out1,
                      uint64_t cap_faces, uint64_t* d_face_offsets, vox_graph** out);
int vox_graph_launch(vox_graph* graph);
int vox_graph_destroy(vox_graph* graph);

/* Page-locked host memory for the host-pointer entry points (cudaMallocHost). */
int vox_host_alloc(size_t bytes, void** out);
int vox_host_free(void* p);

/* ---- Frustum ---------------------------------------------------------------------------- */

/* Gribb-Hartmann planes from a column-major 4x4 matrix (src/frustum_culling.rs:47-85).
 * Output: 6 planes (a, b, c, d) in the order near, far, left, right, top, bottom. */
int vox_frustum_planes(const float m_colmajor[16], float planes[24]);

/* d_visible[i] = 1 iff some corner of chunk i's AABB lies on the inner side of all six
 * planes (src/frustum_culling.rs:16-40), with the AABB edge = chunk_size. */
int vox_frustum_cull(vox_ctx* ctx, const float planes[24], const vox_chunk_coord* d_coords,
                     int32_t n, uint8_t* d_visible);

/* One indexed indirect draw (the layout of wgpu's DrawIndexedIndirectArgs), 20 bytes. */
typedef struct vox_draw_indexed_indirect {
  uint32_t index_count;
  uint32_t instance_count;
  uint32_t first_index;
  int32_t base_vertex;
  uint32_t first_instance;
} vox_draw_indexed_indirect;

/* World::render (src/world.rs:24-40) as a draw list: for every chunk i of a meshed batch
 * (d_face_offsets: its n + 1 offsets) that passes the vox_frustum_cull test and has faces,
 * one record in d_draws, in chunk order; *d_count receives the number of records.
 * Vertex layout: {6 * faces, 1, 6 * face_offsets[i], 4 * face_offsets[i], 0} (the indices
 * are chunk-local). Instanced layout: {6, faces, 0, 0, face_offsets[i]} over the quad's
 * six indices. d_draws needs room for n records. Offsets beyond the 32-bit fields latch
 * VOX_ERR_CAPACITY (vox_ctx_sync) and zero the record. */
int vox_draw_list(vox_ctx* ctx, const float planes[24], const vox_chunk_coord* d_coords,
                  const uint64_t* d_face_offsets, int32_t n, vox_draw_indexed_indirect* d_draws,
                  uint32_t* d_count);

#ifdef __cplusplus
}
#endif

#endif /* VOXGPU_H */
