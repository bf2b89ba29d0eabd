// voxgpu_sys.rs — raw Rust binding of the C ABI (include/voxgpu.h, include/voxgpu_serve.h).
//
// Every entry point with its structs in their C layout. The voxel engine's crate adds this
// module next to src/chunk.rs and calls it where Chunk::new / Chunk::create_mesh
// (src/chunk.rs:21-57) and the ChunkGenerator dispatch (src/chunk_builder.rs:69-132) run
// today. tests/test_abi.py checks that this file binds every declared function and that
// the field lists of its structs match the C headers.
use std::os::raw::{c_char, c_int, c_void};

#[repr(C)] #[derive(Clone, Copy, Default)] pub struct vox_chunk_coord { pub x: i32, pub y: i32, pub z: i32 }
#[repr(C)] #[derive(Clone, Copy)] pub struct vox_generator {
    pub kind: i32, pub octaves: i32, pub seed: u64, pub frequency: f32, pub lacunarity: f32,
    pub gain: f32, pub amplitude: f32, pub base_height: f32, pub y_ref: f32, pub y_scale: f32,
    pub solid_below_zero: i32,
}
#[repr(C)] #[derive(Clone, Copy)] pub struct vox_config {
    pub chunk_size: i32, pub cull_mode: i32, pub layout: i32, pub texture_index: [u32; 6],
    pub gen: vox_generator,
}
#[repr(C)] #[derive(Clone, Copy)] pub struct vox_vertex { pub position: [f32; 3], pub tex_coords: [f32; 2], pub face: u32 }
#[repr(C)] #[derive(Clone, Copy)] pub struct vox_instance_raw { pub t_matrix: [[f32; 4]; 4], pub texture_index: u32 }
#[repr(C)] #[derive(Clone, Copy, Default)] pub struct vox_sizes {
    pub occ_words_per_chunk: u32, pub bytes_per_face_out0: u32, pub bytes_per_face_out1: u32,
    pub max_faces_per_chunk: u32,
}
#[repr(C)] #[derive(Clone, Copy, Default)] pub struct vox_tuning {
    pub threads: i32, pub stage_faces: i32, pub ctas_per_sm: i32, pub schedule: i32,
    pub slab_chunks: i32, pub halo_staging: i32,
}
#[repr(C)] #[derive(Clone, Copy, Default)] pub struct vox_draw_indexed_indirect {
    pub index_count: u32, pub instance_count: u32, pub first_index: u32, pub base_vertex: i32,
    pub first_instance: u32,
}
#[repr(C)] #[derive(Clone, Copy)] pub struct vox_serve_config {
    pub chunk: vox_config, pub view_radius: i32, pub y_min: i32, pub y_max: i32,
    pub max_batch: i32, pub slots: i32, pub cache_budget_bytes: u64, pub neighbour_rebuild: i32,
}
#[repr(C)] #[derive(Clone, Copy, Default)] pub struct vox_serve_stats {
    pub frames: u64, pub requested: u64, pub completed: u64, pub evicted: u64, pub launches: u64,
    pub faces_resident: u64, pub cache_bytes: u64, pub resident: u64, pub pending: u64,
    pub latency_p50_ms: f64, pub latency_p99_ms: f64, pub latency_max_ms: f64, pub busy_s: f64,
    pub cancelled: u64, pub rebuilt: u64, pub rebuild_launches: u64,
}
#[repr(C)] pub struct vox_ctx { _p: [u8; 0] }
#[repr(C)] pub struct vox_graph { _p: [u8; 0] }
#[repr(C)] pub struct vox_serve { _p: [u8; 0] }

pub const VOX_OK: c_int = 0;
pub const VOX_ERR_INVALID: c_int = 1;
pub const VOX_ERR_OOM: c_int = 2;
pub const VOX_ERR_CUDA: c_int = 3;
pub const VOX_ERR_TIMEOUT: c_int = 4;
pub const VOX_ERR_CAPACITY: c_int = 5;
pub const VOX_ERR_NO_DEVICE: c_int = 6;
pub const VOX_GEN_HEIGHTMAP: i32 = 0;
pub const VOX_GEN_DENSITY: i32 = 1;
pub const VOX_GEN_BERNOULLI: i32 = 2;
pub const VOX_CULL_REFERENCE: i32 = 0;
pub const VOX_CULL_FULL6: i32 = 1;
pub const VOX_LAYOUT_VERTEX: i32 = 0;
pub const VOX_LAYOUT_INSTANCED: i32 = 1;
pub const VOX_SCHEDULE_LOOKBACK: i32 = 0;
pub const VOX_SCHEDULE_PHASED: i32 = 1;
pub const VOX_SCHEDULE_OVERLAP: i32 = 2;
pub const VOX_REQ_UNKNOWN: i32 = 0;
pub const VOX_REQ_PENDING: i32 = 1;
pub const VOX_REQ_RESIDENT: i32 = 2;

extern "C" {
    // context, status, sizes
    pub fn vox_ctx_create(cfg: *const vox_config, stream: *mut c_void, out: *mut *mut vox_ctx) -> c_int;
    pub fn vox_ctx_destroy(ctx: *mut vox_ctx) -> c_int;
    pub fn vox_ctx_sync(ctx: *mut vox_ctx) -> c_int;
    pub fn vox_ctx_stream(ctx: *mut vox_ctx) -> *mut c_void;
    pub fn vox_ctx_last_error(ctx: *mut vox_ctx) -> *const c_char;
    pub fn vox_status_string(status: c_int) -> *const c_char;
    pub fn vox_abi_version() -> c_int;
    pub fn vox_query_sizes(cfg: *const vox_config, out: *mut vox_sizes) -> c_int;
    // Chunk::new (chunk.rs:21-46) and the block-id array
    pub fn vox_generate(ctx: *mut vox_ctx, d_coords: *const vox_chunk_coord, n: i32,
                        chunk_index_base: i64, d_occ: *mut u32) -> c_int;
    pub fn vox_generate_slots(ctx: *mut vox_ctx, d_coords: *const vox_chunk_coord, n: i32,
                              chunk_index_base: i64, d_occ_pool: *mut u32, pool_slots: i32,
                              d_slots: *const i32) -> c_int;
    pub fn vox_occ_to_cubes(ctx: *mut vox_ctx, d_occ: *const u32, n: i32, d_cubes: *mut u8) -> c_int;
    pub fn vox_cubes_to_occ(ctx: *mut vox_ctx, d_cubes: *const u8, n: i32, d_occ: *mut u32) -> c_int;
    // Chunk::create_mesh (chunk.rs:48-245): one chunk, or a batch from resident occupancy
    pub fn vox_mesh(ctx: *mut vox_ctx, d_occ: *const u32, d_nbr: *const *const u32,
                    coord: vox_chunk_coord, d_out0: *mut c_void, d_out1: *mut c_void,
                    cap_faces: u64, d_face_count: *mut u64) -> c_int;
    pub fn vox_mesh_batch(ctx: *mut vox_ctx, d_occ_pool: *const u32, pool_slots: i32,
                          d_slots: *const i32, d_nbr_slots: *const i32,
                          d_coords: *const vox_chunk_coord, n: i32, d_out0: *mut c_void,
                          d_out1: *mut c_void, cap_faces: u64, d_face_offsets: *mut u64) -> c_int;
    // the pool's Chunk::new + create_mesh for a batch (chunk_builder.rs:80-84)
    pub fn vox_gen_mesh_batch(ctx: *mut vox_ctx, d_coords: *const vox_chunk_coord,
                              d_nbr_mask: *const u8, n: i32, chunk_index_base: i64,
                              d_out0: *mut c_void, d_out1: *mut c_void, cap_faces: u64,
                              d_face_offsets: *mut u64) -> c_int;
    pub fn vox_gen_mesh_batch_noalloc(cfg: *const vox_config, stream: *mut c_void,
                                      d_coords: *const vox_chunk_coord, d_nbr_mask: *const u8,
                                      n: i32, chunk_index_base: i64, d_out0: *mut c_void,
                                      d_out1: *mut c_void, cap_faces: u64,
                                      d_face_offsets: *mut u64) -> c_int;
    pub fn vox_gen_mesh_host(ctx: *mut vox_ctx, h_coords: *const vox_chunk_coord,
                             h_nbr_mask: *const u8, n: i32, chunk_index_base: i64,
                             h_out0: *mut c_void, h_out1: *mut c_void, cap_faces: u64,
                             h_face_offsets: *mut u64) -> c_int;
    // launch shape
    pub fn vox_ctx_get_tuning(ctx: *mut vox_ctx, out: *mut vox_tuning) -> c_int;
    pub fn vox_ctx_set_tuning(ctx: *mut vox_ctx, tuning: *const vox_tuning) -> c_int;
    pub fn vox_autotune(ctx: *mut vox_ctx, d_coords: *const vox_chunk_coord, d_nbr_mask: *const u8,
                        n: i32, chunk_index_base: i64, d_out0: *mut c_void, d_out1: *mut c_void,
                        cap_faces: u64, d_face_offsets: *mut u64, iters: i32,
                        out: *mut vox_tuning) -> c_int;
    pub fn vox_selftest_lookback_timeout(ctx: *mut vox_ctx, spin_limit: i32) -> c_int;
    // the per-tick dispatch as a replayed CUDA graph
    pub fn vox_graph_capture(ctx: *mut vox_ctx, d_coords: *const vox_chunk_coord,
                             d_nbr_mask: *const u8, n: i32, chunk_index_base: i64,
                             d_out0: *mut c_void, d_out1: *mut c_void, cap_faces: u64,
                             d_face_offsets: *mut u64, out: *mut *mut vox_graph) -> c_int;
    pub fn vox_graph_launch(graph: *mut vox_graph) -> c_int;
    pub fn vox_graph_destroy(graph: *mut vox_graph) -> c_int;
    pub fn vox_host_alloc(bytes: usize, out: *mut *mut c_void) -> c_int;
    pub fn vox_host_free(p: *mut c_void) -> c_int;
    // Frustum (frustum_culling.rs:16-85), World::render's draw loop, headless images
    pub fn vox_frustum_planes(m_colmajor: *const f32, planes: *mut f32) -> c_int;
    pub fn vox_frustum_cull(ctx: *mut vox_ctx, planes: *const f32, d_coords: *const vox_chunk_coord,
                            n: i32, d_visible: *mut u8) -> c_int;
    pub fn vox_draw_list(ctx: *mut vox_ctx, planes: *const f32, d_coords: *const vox_chunk_coord,
                         d_face_offsets: *const u64, n: i32,
                         d_draws: *mut vox_draw_indexed_indirect, d_count: *mut u32) -> c_int;
    pub fn vox_raster(ctx: *mut vox_ctx, view_proj_colmajor: *const f32, d_vertices: *const c_void,
                      d_indices: *const c_void, faces: u64, width: i32, height: i32,
                      d_depth_keys: *mut u64, d_rgba: *mut u8) -> c_int;
    // ChunkGenerator / World (chunk_builder.rs, world.rs) as a streaming engine
    pub fn vox_serve_create(cfg: *const vox_serve_config, out: *mut *mut vox_serve) -> c_int;
    pub fn vox_serve_destroy(s: *mut vox_serve) -> c_int;
    pub fn vox_serve_now() -> f64;
    pub fn vox_serve_frame(s: *mut vox_serve, view_proj: *const f32, eye: *const f32, now_s: f64) -> c_int;
    pub fn vox_serve_submit(s: *mut vox_serve, coords: *const vox_chunk_coord, n: i32, now_s: f64,
                            ids_out: *mut u64) -> c_int;
    pub fn vox_serve_poll(s: *mut vox_serve, id: u64, state: *mut i32) -> c_int;
    pub fn vox_serve_wait(s: *mut vox_serve, id: u64, timeout_s: f64) -> c_int;
    pub fn vox_serve_cancel(s: *mut vox_serve, id: u64) -> c_int;
    pub fn vox_serve_drain(s: *mut vox_serve) -> c_int;
    pub fn vox_serve_get_stats(s: *mut vox_serve, out: *mut vox_serve_stats) -> c_int;
    pub fn vox_serve_latency(s: *mut vox_serve, requested_after_s: f64, p50_ms: *mut f64,
                             p99_ms: *mut f64, max_ms: *mut f64, count: *mut u64) -> c_int;
    pub fn vox_serve_lookup(s: *mut vox_serve, c: vox_chunk_coord, d_out0: *mut *const c_void,
                            d_out1: *mut *const c_void, faces: *mut u64) -> c_int;
    pub fn vox_camera_global_matrix(eye: *const f32, dir: *const f32, aspect: f32, fovy: f32,
                                    znear: f32, zfar: f32, out_colmajor: *mut f32) -> c_int;
    pub fn vox_world_to_chunk(pos: *const f32, chunk_size: i32) -> vox_chunk_coord;
}
