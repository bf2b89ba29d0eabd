/*
 * voxgpu_serve.h — C ABI of the chunk streaming engine (the request loop that replaces
 * the reference's ChunkGenerator / World, src/chunk_builder.rs:11-353, src/world.rs:14-59)
 * and of the camera / coordinate helpers it uses (src/camera.rs:41-51,
 * src/coordinate.rs:13-65).
 *
 * Every frame the engine frustum-culls the chunks within the view radius on the device,
 * turns the visible chunks that are neither resident nor pending into requests ordered by
 * distance to the eye, admits them into batches as batch slots free up (several batches
 * in flight on their own streams: continuous batching), and integrates finished batches
 * into a device mesh cache kept under a byte budget with least-recently-used eviction.
 * It records, per chunk, the time from its request to the moment its mesh is resident.
 *
 * By default, unlike the reference (one chunk dispatched and one integrated per 7 frames,
 * meshes rebuilt as neighbours arrive), a chunk's halo comes from the generator itself, so
 * its mesh is the final one (all four lateral neighbours present) whatever else is loaded:
 * the same bytes alone, in any batch, and in any order of arrival. With
 * neighbour_rebuild = 1 the engine keeps the reference's semantics instead: occupancy stays
 * resident, a chunk's halo comes from its resident neighbours, and the neighbours are
 * remeshed as chunks arrive, so that once the engine is drained every resident chunk's
 * mesh is the one the reference builds with its resident neighbours.
 */
#ifndef VOXGPU_SERVE_H
#define VOXGPU_SERVE_H

#include <stddef.h>
#include <stdint.h>

#include "voxgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vox_serve_config {
  vox_config chunk;            /* generator, chunk size, culling, layout */
  int32_t view_radius;         /* chunks: requests only within this xz distance of the eye */
  int32_t y_min, y_max;        /* chunk layers that are requested (the reference: 0..0) */
  int32_t max_batch;           /* chunks per launch */
  int32_t slots;               /* batches in flight at once (one stream each) */
  uint64_t cache_budget_bytes; /* device bytes for resident meshes (LRU eviction beyond) */
  int32_t neighbour_rebuild;   /* 0: every halo from the generator (a chunk's first mesh is
                                  final); 1: the reference's semantics: a chunk is meshed
                                  against the neighbours resident at launch (absent ones
                                  emit their border faces) and remeshed from its cached
                                  occupancy when a neighbour arrives or leaves. Mode 1 also
                                  holds a device occupancy pool of one slot per chunk that
                                  the budget can hold at 4 N^2 faces per chunk */
} vox_serve_config;

typedef struct vox_serve_stats {
  uint64_t frames;             /* vox_serve_frame calls */
  uint64_t requested;          /* chunks requested */
  uint64_t completed;          /* chunks whose mesh became resident */
  uint64_t evicted;            /* chunks evicted from the cache */
  uint64_t launches;           /* fused gen+mesh launches */
  uint64_t faces_resident;     /* faces held by resident chunks */
  uint64_t cache_bytes;        /* bytes held by resident mesh blocks */
  uint64_t resident;           /* resident chunks */
  uint64_t pending;            /* requested, not yet resident */
  double latency_p50_ms;       /* request -> resident, over all completed chunks */
  double latency_p99_ms;
  double latency_max_ms;
  double busy_s;               /* wall time between the first request and the last completion */
  uint64_t cancelled;          /* requests withdrawn by vox_serve_cancel */
  uint64_t rebuilt;            /* meshes rebuilt from cached occupancy (neighbour_rebuild) */
  uint64_t rebuild_launches;   /* mesh-only launches of those rebuilds */
} vox_serve_stats;

typedef struct vox_serve vox_serve;

int vox_serve_create(const vox_serve_config* cfg, vox_serve** out);
int vox_serve_destroy(vox_serve* s);

/* The engine's monotonic clock in seconds (request and completion times use it). */
double vox_serve_now(void);

/* One frame: `view_proj` is the camera's column-major global matrix (frustum planes are
 * taken from it as in Frustum::matrix_to_planes), `eye` the camera position in world
 * units, `now_s` the frame's time on the engine clock (negative: read the clock). Culls,
 * requests, admits new batches and integrates finished ones (a chunk's latency ends when
 * the engine sees its batch finished); does not wait for the GPU. */
int vox_serve_frame(vox_serve* s, const float view_proj[16], const float eye[3], double now_s);

/* Explicit requests (the reference's ChunkGenerator enqueue, chunk_builder.rs:54-66,
 * without the camera): requests every chunk of coords[0..n) that is neither pending nor
 * resident, refreshes the others, writes each chunk's request id to ids_out (may be NULL)
 * and admits what fits. A chunk keeps its id while it is pending or resident. */
int vox_serve_submit(vox_serve* s, const vox_chunk_coord* coords, int32_t n, double now_s,
                     uint64_t* ids_out);

/* Request states. UNKNOWN: never issued, or evicted since. */
enum { VOX_REQ_UNKNOWN = 0, VOX_REQ_PENDING = 1, VOX_REQ_RESIDENT = 2 };

/* Integrates finished batches, admits queued requests and reports the request's state. */
int vox_serve_poll(vox_serve* s, uint64_t id, int32_t* state);

/* Drives the engine until request `id` is resident (VOX_OK), or returns VOX_ERR_TIMEOUT
 * after timeout_s seconds, VOX_ERR_INVALID for an unknown id, VOX_ERR_OOM if the cache
 * budget cannot hold its batch. */
int vox_serve_wait(vox_serve* s, uint64_t id, double timeout_s);

/* Withdraws a pending request. A queued chunk leaves the queue; a chunk whose batch is
 * already on the GPU is discarded when the batch completes (its mesh never becomes
 * resident). The id becomes VOX_REQ_UNKNOWN. Returns VOX_ERR_INVALID for an unknown id or
 * a request that is already resident (nothing to withdraw). The reference drops queued
 * chunks that leave the view the same way (src/chunk_builder.rs:334-352). */
int vox_serve_cancel(vox_serve* s, uint64_t id);

/* Waits for every batch in flight (and every queued request) and integrates them. */
int vox_serve_drain(vox_serve* s);

int vox_serve_get_stats(vox_serve* s, vox_serve_stats* out);

/* Request -> resident latency over the completed requests issued at or after
 * requested_after_s (engine clock): p50, p99 and max in ms and their count; for example the
 * steady state after the first view fill. Any output pointer may be NULL. */
int vox_serve_latency(vox_serve* s, double requested_after_s, double* p50_ms, double* p99_ms,
                      double* max_ms, uint64_t* count);

/* The resident mesh of chunk `c`: device pointers to its records (out1 NULL for the
 * instanced layout) and its face count. Returns VOX_ERR_INVALID if it is not resident. */
int vox_serve_lookup(vox_serve* s, vox_chunk_coord c, const void** d_out0, const void** d_out1,
                     uint64_t* faces);

/* Camera::update_global_matrix (src/camera.rs:41-51): OPENGL_TO_WGPU * perspective *
 * look_at_rh(eye, eye + dir, +y), column-major. dir is the viewing direction, fovy in
 * radians (the reference passes fov.to_degrees() here; pass that value to reproduce it). */
int vox_camera_global_matrix(const float eye[3], const float dir[3], float aspect, float fovy,
                             float znear, float zfar, float out_colmajor[16]);

/* Coord3DF::to_chunk_coord (src/coordinate.rs:33-38) for chunk size n: floor(v) >> log2(n). */
vox_chunk_coord vox_world_to_chunk(const float pos[3], int32_t chunk_size);

#ifdef __cplusplus
}
#endif

#endif /* VOXGPU_SERVE_H */
