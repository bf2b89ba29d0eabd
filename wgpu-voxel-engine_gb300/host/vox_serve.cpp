// vox_serve.cpp — chunk streaming engine over the C ABI (include/voxgpu_serve.h).
//
// Host-side restatement of the reference's ChunkGenerator / World loop
// (src/chunk_builder.rs:45-352, src/world.rs:14-59) built for a GPU: device frustum
// culling of the view disk (Frustum::contains, src/frustum_culling.rs:16-40), requests
// ordered by distance, continuous batching over several streams, and a device mesh cache
// with a byte budget and LRU eviction (the reference evicts everything outside a +-5
// chunk box, chunk_builder.rs:334-352). Only the public C ABI and the CUDA runtime's
// stream/event/stream-ordered-allocation calls are used here.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <thread>
#include <unordered_map>
#include <vector>

#include "voxgpu.h"
#include "voxgpu_serve.h"
#include "../csrc/vox_trace.h"

namespace {

struct CoordHash {
  size_t operator()(const vox_chunk_coord& c) const {
    uint64_t h = (uint64_t)(uint32_t)c.x * 0x9E3779B97F4A7C15ull;
    h ^= (uint64_t)(uint32_t)c.y * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
    h ^= (uint64_t)(uint32_t)c.z * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
    return (size_t)h;
  }
};
struct CoordEq {
  bool operator()(const vox_chunk_coord& a, const vox_chunk_coord& b) const {
    return a.x == b.x && a.y == b.y && a.z == b.z;
  }
};

double mono_now() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// A batch's output block in device memory, shared by the chunks meshed in it.
struct Block {
  void* out0 = nullptr;
  void* out1 = nullptr;
  uint64_t bytes = 0;
  int refs = 0;
  cudaStream_t stream = nullptr;
};

struct Entry {
  enum State { PENDING, RESIDENT } state = PENDING;
  bool in_flight = false;  // its batch is on the GPU (a chunk requested again after a
                           // cancellation waits for its own batch)
  uint64_t id = 0;  // request id (vox_serve_submit / poll / wait)
  double requested_at = 0.0;
  uint64_t last_seen = 0;
  std::shared_ptr<Block> block;
  uint64_t offset = 0;
  uint64_t faces = 0;
};

struct Slot {
  vox_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t start = nullptr;  // recorded before the batch's first copy
  cudaEvent_t done = nullptr;   // recorded after its offsets reach the host
  double launched_at = 0.0;     // engine clock when `start` was recorded
  bool busy = false;
  vox_chunk_coord* d_coords = nullptr;
  uint8_t* d_mask = nullptr;
  uint64_t* d_offsets = nullptr;
  uint64_t* h_offsets = nullptr;  // pinned
  std::vector<vox_chunk_coord> chunks;
  std::shared_ptr<Block> block;
  uint64_t cap_faces = 0;
};

}  // namespace

struct vox_serve {
  vox_serve_config cfg{};
  vox_sizes sizes{};
  int n = 0;
  uint64_t bytes_per_face = 0;
  uint64_t est_faces_per_chunk = 0;
  std::vector<Slot> slots;
  // culling
  vox_ctx* cull_ctx = nullptr;
  cudaStream_t cull_stream = nullptr;
  vox_chunk_coord* d_cand = nullptr;
  uint8_t* d_vis = nullptr;
  uint8_t* h_vis = nullptr;  // pinned
  std::vector<vox_chunk_coord> cand;
  size_t cand_cap = 0;
  bool have_center = false;
  vox_chunk_coord center{0, 0, 0};
  // state
  std::unordered_map<vox_chunk_coord, Entry, CoordHash, CoordEq> entries;
  std::unordered_map<uint64_t, vox_chunk_coord> by_id;  // request id -> chunk
  uint64_t next_id = 1;
  std::vector<vox_chunk_coord> queue;
  std::vector<double> latencies;
  vox_serve_stats stats{};
  uint64_t frame = 0;
  double first_request = -1.0, last_completion = -1.0;
  float eye[3] = {0, 0, 0};
};

namespace {

void free_block(Block* b) {
  if (b->out0) cudaFreeAsync(b->out0, b->stream);
  if (b->out1) cudaFreeAsync(b->out1, b->stream);
  b->out0 = b->out1 = nullptr;
}

float dist2(const vox_serve* s, const vox_chunk_coord& c) {
  const float h = 0.5f * (float)s->n;
  const float dx = (float)(c.x * s->n) + h - s->eye[0];
  const float dy = (float)(c.y * s->n) + h - s->eye[1];
  const float dz = (float)(c.z * s->n) + h - s->eye[2];
  return dx * dx + dy * dy + dz * dz;
}

// Drops one resident chunk's reference to its block (freeing the block at zero).
void release(vox_serve* s, Entry& e) {
  if (e.block) {
    if (--e.block->refs == 0) {
      s->stats.cache_bytes -= e.block->bytes;
      free_block(e.block.get());
    }
    e.block.reset();
  }
  s->stats.faces_resident -= e.faces;
}

// Evicts least-recently-seen resident chunks until `need` more bytes fit in the budget:
// first those not seen this frame, then (when the visible set alone exceeds the budget)
// visible ones. Returns false if the budget cannot hold `need` at all.
bool make_room(vox_serve* s, uint64_t need) {
  if (need > s->cfg.cache_budget_bytes) return false;
  while (s->stats.cache_bytes + need > s->cfg.cache_budget_bytes) {
    auto victim = s->entries.end();
    for (int pass = 0; pass < 2 && victim == s->entries.end(); ++pass) {
      for (auto it = s->entries.begin(); it != s->entries.end(); ++it) {
        if (it->second.state != Entry::RESIDENT) continue;
        if (pass == 0 && it->second.last_seen >= s->frame) continue;
        if (victim == s->entries.end() || it->second.last_seen < victim->second.last_seen)
          victim = it;
      }
    }
    if (victim == s->entries.end()) return false;
    release(s, victim->second);
    s->by_id.erase(victim->second.id);
    s->entries.erase(victim);
    ++s->stats.evicted;
    --s->stats.resident;
  }
  return true;
}

int launch_batch(vox_serve* s, Slot& sl, std::vector<vox_chunk_coord>&& chunks) {
  const int m = (int)chunks.size();
  const uint64_t cap = (uint64_t)m * s->est_faces_per_chunk;
  const uint64_t bytes = cap * s->bytes_per_face;
  if (!make_room(s, bytes)) return VOX_ERR_OOM;
  auto blk = std::make_shared<Block>();
  blk->stream = sl.stream;
  blk->bytes = bytes;
  const uint64_t b0 = s->sizes.bytes_per_face_out0, b1 = s->sizes.bytes_per_face_out1;
  if (cudaMallocAsync(&blk->out0, cap * b0, sl.stream) != cudaSuccess ||
      (b1 && cudaMallocAsync(&blk->out1, cap * b1, sl.stream) != cudaSuccess)) {
    cudaGetLastError();
    free_block(blk.get());
    return VOX_ERR_OOM;
  }
  s->stats.cache_bytes += bytes;
  std::vector<uint8_t> masks(m, s->cfg.chunk.cull_mode == VOX_CULL_FULL6 ? 0x3F : 0x0F);
  sl.launched_at = mono_now();
  cudaEventRecord(sl.start, sl.stream);
  cudaMemcpyAsync(sl.d_coords, chunks.data(), sizeof(vox_chunk_coord) * m, cudaMemcpyHostToDevice,
                  sl.stream);
  cudaMemcpyAsync(sl.d_mask, masks.data(), (size_t)m, cudaMemcpyHostToDevice, sl.stream);
  int st = vox_gen_mesh_batch(sl.ctx, sl.d_coords, sl.d_mask, m, 0, blk->out0, blk->out1, cap,
                              sl.d_offsets);
  if (st != VOX_OK) return st;
  cudaMemcpyAsync(sl.h_offsets, sl.d_offsets, sizeof(uint64_t) * (m + 1), cudaMemcpyDeviceToHost,
                  sl.stream);
  cudaEventRecord(sl.done, sl.stream);
  for (const vox_chunk_coord& c : chunks) {
    auto it = s->entries.find(c);
    if (it != s->entries.end()) it->second.in_flight = true;
  }
  sl.chunks = std::move(chunks);
  sl.block = blk;
  sl.cap_faces = cap;
  sl.busy = true;
  ++s->stats.launches;
  return VOX_OK;
}

// Integrates a finished batch; a batch whose output did not fit is relaunched with room
// for the faces it reported.
int integrate(vox_serve* s, Slot& sl, double now) {
  const int status = vox_ctx_sync(sl.ctx);
  const int m = (int)sl.chunks.size();
  const uint64_t total = sl.h_offsets[m];
  sl.busy = false;
  if (status == VOX_ERR_CAPACITY || total > sl.cap_faces) {
    s->stats.cache_bytes -= sl.block->bytes;
    free_block(sl.block.get());
    sl.block.reset();
    s->est_faces_per_chunk = std::max<uint64_t>(s->est_faces_per_chunk, (total + m - 1) / m + 1);
    std::vector<vox_chunk_coord> again = std::move(sl.chunks);
    sl.chunks.clear();
    return launch_batch(s, sl, std::move(again));
  }
  if (status != VOX_OK) return status;
  sl.block->refs = m;
  for (int i = 0; i < m; ++i) {
    auto it = s->entries.find(sl.chunks[i]);
    if (it == s->entries.end() || !it->second.in_flight) {  // cancelled meanwhile
      if (--sl.block->refs == 0) {
        s->stats.cache_bytes -= sl.block->bytes;
        free_block(sl.block.get());
      }
      continue;
    }
    Entry& e = it->second;
    e.in_flight = false;
    e.state = Entry::RESIDENT;
    e.block = sl.block;
    e.offset = sl.h_offsets[i];
    e.faces = sl.h_offsets[i + 1] - sl.h_offsets[i];
    s->stats.faces_resident += e.faces;
    ++s->stats.completed;
    ++s->stats.resident;
    --s->stats.pending;
    s->latencies.push_back((now - e.requested_at) * 1e3);
  }
  s->last_completion = now;
  sl.block.reset();
  sl.chunks.clear();
  return VOX_OK;
}

// Requests chunk c (or refreshes it when already pending or resident) and returns its
// request id.
uint64_t request(vox_serve* s, const vox_chunk_coord& c, double now_s) {
  auto it = s->entries.find(c);
  if (it != s->entries.end()) {
    it->second.last_seen = s->frame;
    return it->second.id;
  }
  Entry e;
  e.state = Entry::PENDING;
  e.id = s->next_id++;
  e.requested_at = now_s;
  e.last_seen = s->frame;
  s->entries.emplace(c, e);
  s->by_id.emplace(e.id, c);
  s->queue.push_back(c);
  ++s->stats.requested;
  ++s->stats.pending;
  if (s->first_request < 0.0) s->first_request = now_s;
  return e.id;
}

int poll_and_admit(vox_serve* s, bool wait) {
  for (Slot& sl : s->slots) {
    if (!sl.busy) continue;
    cudaError_t q = wait ? cudaEventSynchronize(sl.done) : cudaEventQuery(sl.done);
    if (q == cudaErrorNotReady) continue;
    if (q != cudaSuccess) return VOX_ERR_CUDA;
    // Completion time from the GPU's own timestamps (the slot's stream is idle when a
    // batch is admitted, so `start` fires as the batch is enqueued), not from when the
    // host happened to poll.
    float ms = 0.0f;
    const double t_done = cudaEventElapsedTime(&ms, sl.start, sl.done) == cudaSuccess
                              ? sl.launched_at + (double)ms * 1e-3
                              : mono_now();
    const int st = integrate(s, sl, t_done);
    if (st != VOX_OK) return st;
  }
  // admit: nearest requests first
  if (!s->queue.empty()) {
    std::sort(s->queue.begin(), s->queue.end(),
              [s](const vox_chunk_coord& a, const vox_chunk_coord& b) {
                return dist2(s, a) < dist2(s, b);
              });
    size_t head = 0;
    // a batch reserves est_faces_per_chunk faces per chunk; keep one batch within the budget
    const uint64_t per_chunk = s->est_faces_per_chunk * s->bytes_per_face;
    const size_t fit = (size_t)std::max<uint64_t>(1, s->cfg.cache_budget_bytes / per_chunk);
    for (Slot& sl : s->slots) {
      if (sl.busy || head >= s->queue.size()) continue;
      const size_t take =
          std::min<size_t>(std::min<size_t>((size_t)s->cfg.max_batch, fit), s->queue.size() - head);
      std::vector<vox_chunk_coord> chunks(s->queue.begin() + head, s->queue.begin() + head + take);
      const int st = launch_batch(s, sl, std::move(chunks));
      if (st == VOX_ERR_OOM) break;  // the cache is full of visible chunks: retry later
      if (st != VOX_OK) return st;
      head += take;
    }
    s->queue.erase(s->queue.begin(), s->queue.begin() + head);
  }
  return VOX_OK;
}

int rebuild_candidates(vox_serve* s, vox_chunk_coord c) {
  s->cand.clear();
  const int R = s->cfg.view_radius;
  for (int y = s->cfg.y_min; y <= s->cfg.y_max; ++y)
    for (int dz = -R; dz <= R; ++dz)
      for (int dx = -R; dx <= R; ++dx)
        if (dx * dx + dz * dz <= R * R) s->cand.push_back({c.x + dx, y, c.z + dz});
  const size_t n = s->cand.size();
  if (n > s->cand_cap) {
    cudaFree(s->d_cand);
    cudaFree(s->d_vis);
    cudaFreeHost(s->h_vis);
    if (cudaMalloc(&s->d_cand, n * sizeof(vox_chunk_coord)) != cudaSuccess ||
        cudaMalloc(&s->d_vis, n) != cudaSuccess || cudaMallocHost(&s->h_vis, n) != cudaSuccess)
      return VOX_ERR_OOM;
    s->cand_cap = n;
  }
  if (cudaMemcpyAsync(s->d_cand, s->cand.data(), n * sizeof(vox_chunk_coord),
                      cudaMemcpyHostToDevice, s->cull_stream) != cudaSuccess)
    return VOX_ERR_CUDA;
  s->center = c;
  s->have_center = true;
  return VOX_OK;
}

}  // namespace

extern "C" {

int vox_serve_create(const vox_serve_config* cfg, vox_serve** out) {
  if (!cfg || !out || cfg->view_radius < 0 || cfg->max_batch < 1 || cfg->slots < 1 ||
      cfg->y_max < cfg->y_min || cfg->cache_budget_bytes == 0)
    return VOX_ERR_INVALID;
  *out = nullptr;
  // a failure below releases whatever was created so far (vox_serve_destroy skips the rest)
  struct Destroy {
    void operator()(vox_serve* p) const { vox_serve_destroy(p); }
  };
  std::unique_ptr<vox_serve, Destroy> s(new vox_serve());
  s->cfg = *cfg;
  int st = vox_query_sizes(&cfg->chunk, &s->sizes);
  if (st != VOX_OK) return st;
  s->n = cfg->chunk.chunk_size;
  s->bytes_per_face = s->sizes.bytes_per_face_out0 + s->sizes.bytes_per_face_out1;
  s->est_faces_per_chunk = (uint64_t)4 * s->n * s->n;
  // keep freed blocks in the stream-ordered pool instead of returning them to the driver
  int dev = 0;
  cudaGetDevice(&dev);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = cfg->cache_budget_bytes;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  s->slots.resize(cfg->slots);
  for (Slot& sl : s->slots) {
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&sl.start) != cudaSuccess || cudaEventCreate(&sl.done) != cudaSuccess)
      return VOX_ERR_CUDA;
    if ((st = vox_ctx_create(&cfg->chunk, sl.stream, &sl.ctx)) != VOX_OK) return st;
    if (cudaMalloc(&sl.d_coords, sizeof(vox_chunk_coord) * cfg->max_batch) != cudaSuccess ||
        cudaMalloc(&sl.d_mask, (size_t)cfg->max_batch) != cudaSuccess ||
        cudaMalloc(&sl.d_offsets, sizeof(uint64_t) * (cfg->max_batch + 1)) != cudaSuccess ||
        cudaMallocHost(&sl.h_offsets, sizeof(uint64_t) * (cfg->max_batch + 1)) != cudaSuccess)
      return VOX_ERR_OOM;
  }
  if (cudaStreamCreateWithFlags(&s->cull_stream, cudaStreamNonBlocking) != cudaSuccess)
    return VOX_ERR_CUDA;
  if ((st = vox_ctx_create(&cfg->chunk, s->cull_stream, &s->cull_ctx)) != VOX_OK) return st;
  *out = s.release();
  return VOX_OK;
}

int vox_serve_destroy(vox_serve* s) {
  if (!s) return VOX_OK;
  for (Slot& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
  }
  for (auto& kv : s->entries) release(s, kv.second);
  for (Slot& sl : s->slots) {
    if (sl.block) free_block(sl.block.get());
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    vox_ctx_destroy(sl.ctx);
    cudaFree(sl.d_coords);
    cudaFree(sl.d_mask);
    cudaFree(sl.d_offsets);
    if (sl.h_offsets) cudaFreeHost(sl.h_offsets);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.start) cudaEventDestroy(sl.start);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  vox_ctx_destroy(s->cull_ctx);
  cudaFree(s->d_cand);
  cudaFree(s->d_vis);
  if (s->h_vis) cudaFreeHost(s->h_vis);
  if (s->cull_stream) cudaStreamDestroy(s->cull_stream);
  delete s;
  return VOX_OK;
}

double vox_serve_now(void) { return mono_now(); }

int vox_serve_frame(vox_serve* s, const float view_proj[16], const float eye[3], double now_s) {
  vox::TraceRange trace_("vox_serve_frame");
  if (!s || !view_proj || !eye) return VOX_ERR_INVALID;
  if (now_s < 0.0) now_s = mono_now();
  ++s->frame;
  ++s->stats.frames;
  std::memcpy(s->eye, eye, sizeof s->eye);
  const vox_chunk_coord c = vox_world_to_chunk(eye, s->n);
  int st;
  if (!s->have_center || c.x != s->center.x || c.z != s->center.z) {
    if ((st = rebuild_candidates(s, c)) != VOX_OK) return st;
  }
  float planes[24];
  vox_frustum_planes(view_proj, planes);
  const int n = (int)s->cand.size();
  if ((st = vox_frustum_cull(s->cull_ctx, planes, s->d_cand, n, s->d_vis)) != VOX_OK) return st;
  if (cudaMemcpyAsync(s->h_vis, s->d_vis, (size_t)n, cudaMemcpyDeviceToHost, s->cull_stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(s->cull_stream) != cudaSuccess)
    return VOX_ERR_CUDA;
  for (int i = 0; i < n; ++i)
    if (s->h_vis[i]) request(s, s->cand[i], now_s);
  return poll_and_admit(s, false);
}

int vox_serve_submit(vox_serve* s, const vox_chunk_coord* coords, int32_t n, double now_s,
                     uint64_t* ids_out) {
  vox::TraceRange trace_("vox_serve_submit");
  if (!s || n < 0 || (n > 0 && !coords)) return VOX_ERR_INVALID;
  if (now_s < 0.0) now_s = mono_now();
  for (int32_t i = 0; i < n; ++i) {
    const uint64_t id = request(s, coords[i], now_s);
    if (ids_out) ids_out[i] = id;
  }
  return poll_and_admit(s, false);
}

static int32_t request_state(vox_serve* s, uint64_t id) {
  auto it = s->by_id.find(id);
  if (it == s->by_id.end()) return VOX_REQ_UNKNOWN;
  auto e = s->entries.find(it->second);
  if (e == s->entries.end()) return VOX_REQ_UNKNOWN;
  return e->second.state == Entry::RESIDENT ? VOX_REQ_RESIDENT : VOX_REQ_PENDING;
}

int vox_serve_poll(vox_serve* s, uint64_t id, int32_t* state) {
  vox::TraceRange trace_("vox_serve_poll");
  if (!s || !state) return VOX_ERR_INVALID;
  const int st = poll_and_admit(s, false);
  if (st != VOX_OK) return st;
  *state = request_state(s, id);
  return VOX_OK;
}

int vox_serve_wait(vox_serve* s, uint64_t id, double timeout_s) {
  vox::TraceRange trace_("vox_serve_wait");
  if (!s) return VOX_ERR_INVALID;
  const double deadline = mono_now() + timeout_s;
  for (;;) {
    int st = poll_and_admit(s, false);
    if (st != VOX_OK) return st;
    const int32_t r = request_state(s, id);
    if (r == VOX_REQ_RESIDENT) return VOX_OK;
    if (r == VOX_REQ_UNKNOWN) return VOX_ERR_INVALID;
    bool busy = false;
    for (Slot& sl : s->slots) busy = busy || sl.busy;
    if (!busy && !s->queue.empty()) return VOX_ERR_OOM;  // the budget cannot hold its batch
    if (mono_now() >= deadline) return VOX_ERR_TIMEOUT;
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

int vox_serve_cancel(vox_serve* s, uint64_t id) {
  vox::TraceRange trace_("vox_serve_cancel");
  if (!s) return VOX_ERR_INVALID;
  auto it = s->by_id.find(id);
  if (it == s->by_id.end()) return VOX_ERR_INVALID;
  auto e = s->entries.find(it->second);
  if (e == s->entries.end() || e->second.state != Entry::PENDING) return VOX_ERR_INVALID;
  // a queued chunk leaves the queue; a launched one is dropped by integrate()
  auto q = std::find_if(s->queue.begin(), s->queue.end(),
                        [&](const vox_chunk_coord& c) { return CoordEq()(c, it->second); });
  if (q != s->queue.end()) s->queue.erase(q);
  s->entries.erase(e);
  s->by_id.erase(it);
  --s->stats.pending;
  ++s->stats.cancelled;
  return VOX_OK;
}

int vox_serve_drain(vox_serve* s) {
  vox::TraceRange trace_("vox_serve_drain");
  if (!s) return VOX_ERR_INVALID;
  for (;;) {
    bool busy = false;
    for (Slot& sl : s->slots) busy = busy || sl.busy;
    if (!busy && s->queue.empty()) return VOX_OK;
    const int st = poll_and_admit(s, true);
    if (st != VOX_OK) return st;
    bool launched = false;
    for (Slot& sl : s->slots) launched = launched || sl.busy;
    // nothing in flight and nothing admitted: the budget cannot hold the next batch
    if (!launched && !s->queue.empty()) return VOX_ERR_OOM;
  }
}

int vox_serve_get_stats(vox_serve* s, vox_serve_stats* out) {
  if (!s || !out) return VOX_ERR_INVALID;
  *out = s->stats;
  std::vector<double> v = s->latencies;
  auto pct = [&](double q) {
    if (v.empty()) return 0.0;
    size_t k = (size_t)std::min<double>((double)v.size() - 1, std::floor(q * (double)v.size()));
    std::nth_element(v.begin(), v.begin() + (long)k, v.end());
    return v[k];
  };
  out->latency_p50_ms = pct(0.50);
  out->latency_p99_ms = pct(0.99);
  out->latency_max_ms = v.empty() ? 0.0 : *std::max_element(v.begin(), v.end());
  out->busy_s = s->first_request >= 0.0 && s->last_completion >= 0.0
                    ? s->last_completion - s->first_request
                    : 0.0;
  return VOX_OK;
}

int vox_serve_lookup(vox_serve* s, vox_chunk_coord c, const void** d_out0, const void** d_out1,
                     uint64_t* faces) {
  if (!s) return VOX_ERR_INVALID;
  auto it = s->entries.find(c);
  if (it == s->entries.end() || it->second.state != Entry::RESIDENT) return VOX_ERR_INVALID;
  const Entry& e = it->second;
  const uint64_t b0 = s->sizes.bytes_per_face_out0, b1 = s->sizes.bytes_per_face_out1;
  if (d_out0) *d_out0 = static_cast<const char*>(e.block->out0) + e.offset * b0;
  if (d_out1) *d_out1 = b1 ? static_cast<const char*>(e.block->out1) + e.offset * b1 : nullptr;
  if (faces) *faces = e.faces;
  return VOX_OK;
}

int vox_camera_global_matrix(const float eye[3], const float dir[3], float aspect, float fovy,
                             float znear, float zfar, float out[16]) {
  if (!eye || !dir || !out || aspect <= 0.0f || znear <= 0.0f || zfar <= znear)
    return VOX_ERR_INVALID;
  // look_at_rh(eye, eye + dir, +y)
  float f[3] = {dir[0], dir[1], dir[2]};
  float fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  if (fl == 0.0f) return VOX_ERR_INVALID;
  for (float& v : f) v /= fl;
  const float up[3] = {0.0f, 1.0f, 0.0f};
  float sx[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2],
                 f[0] * up[1] - f[1] * up[0]};
  float sl = std::sqrt(sx[0] * sx[0] + sx[1] * sx[1] + sx[2] * sx[2]);
  if (sl == 0.0f) return VOX_ERR_INVALID;
  for (float& v : sx) v /= sl;
  const float u[3] = {sx[1] * f[2] - sx[2] * f[1], sx[2] * f[0] - sx[0] * f[2],
                      sx[0] * f[1] - sx[1] * f[0]};
  float V[4][4] = {{sx[0], sx[1], sx[2], -(sx[0] * eye[0] + sx[1] * eye[1] + sx[2] * eye[2])},
                   {u[0], u[1], u[2], -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2])},
                   {-f[0], -f[1], -f[2], (f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2])},
                   {0.0f, 0.0f, 0.0f, 1.0f}};
  // OpenGL-style perspective
  const float t = 1.0f / std::tan(fovy * 0.5f);
  float P[4][4] = {{t / aspect, 0, 0, 0},
                   {0, t, 0, 0},
                   {0, 0, (zfar + znear) / (znear - zfar), 2.0f * zfar * znear / (znear - zfar)},
                   {0, 0, -1.0f, 0}};
  // OPENGL_TO_WGPU_MATRIX as written in src/camera.rs:18-23 (Matrix4::new takes rows)
  float G[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 0.5f, 0}, {0, 0, 0.5f, 1}};
  float GP[4][4], M[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float a = 0.0f;
      for (int k = 0; k < 4; ++k) a += G[i][k] * P[k][j];
      GP[i][j] = a;
    }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float a = 0.0f;
      for (int k = 0; k < 4; ++k) a += GP[i][k] * V[k][j];
      M[i][j] = a;
    }
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) out[c * 4 + r] = M[r][c];
  return VOX_OK;
}

vox_chunk_coord vox_world_to_chunk(const float pos[3], int32_t n) {
  vox_chunk_coord c{0, 0, 0};
  if (!pos || n <= 0) return c;
  int sh = 0;
  while ((1 << sh) < n) ++sh;
  c.x = (int32_t)std::floor(pos[0]) >> sh;
  c.y = (int32_t)std::floor(pos[1]) >> sh;
  c.z = (int32_t)std::floor(pos[2]) >> sh;
  return c;
}

}  // extern "C"
