// vox_serve.cpp — chunk streaming engine over the C ABI (include/voxgpu_serve.h).
//
// Host-side restatement of the reference's ChunkGenerator / World loop
// (src/chunk_builder.rs:45-352, src/world.rs:14-59) built for a GPU: device frustum
// culling of the view disk (Frustum::contains, src/frustum_culling.rs:16-40), requests
// ordered by distance, continuous batching over several streams, and a device mesh cache
// with a byte budget and LRU eviction (the reference evicts everything outside a +-5
// chunk box, chunk_builder.rs:334-352). Only the public C ABI and the CUDA runtime's
// stream/event/stream-ordered-allocation calls are used here.
//
// Two ways to get a chunk's halo:
//  - generated (the default): every batch regenerates the lateral halo of its chunks from
//    the generator, so a chunk's first mesh is already its final one;
//  - neighbour rebuild (vox_serve_config.neighbour_rebuild): the reference's semantics.
//    Each resident chunk keeps its occupancy in a device pool; a new chunk is meshed
//    against the neighbours resident when its batch is launched (an absent neighbour's
//    border faces are emitted, src/chunk.rs:102-107), and when a chunk becomes resident
//    the resident neighbours whose meshes did not see it are remeshed from the pool
//    (ChunkGenerator::rebuild_adjacent_chunks and process_rebuild_queue,
//    src/chunk_builder.rs:89-112, 269-300, 310-332), in mesh-only batches.
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
#include "vox_flat_map.h"
#include "vox_order.h"
#include "../csrc/vox_trace.h"

namespace {

using vox::CoordEq;
using vox::CoordHash;
using vox::FlatMap;
using vox::IdEq;
using vox::IdHash;

double mono_now() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Neighbour directions in the order of the halo masks: -x, +x, -z, +z, -y, +y.
constexpr int kDx[6] = {-1, 1, 0, 0, 0, 0};
constexpr int kDy[6] = {0, 0, 0, 0, -1, 1};
constexpr int kDz[6] = {0, 0, -1, 1, 0, 0};
constexpr int kOpposite[6] = {1, 0, 3, 2, 5, 4};

vox_chunk_coord neighbour(const vox_chunk_coord& c, int d) {
  return {c.x + kDx[d], c.y + kDy[d], c.z + kDz[d]};
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
  bool in_flight = false;  // its load batch is on the GPU (a chunk requested again after a
                           // cancellation waits for its own batch)
  uint64_t id = 0;  // request id (vox_serve_submit / poll / wait)
  double requested_at = 0.0;
  uint64_t last_seen = 0;
  std::shared_ptr<Block> block;
  uint64_t offset = 0;
  uint64_t faces = 0;
  // neighbour-rebuild mode
  int occ_slot = -1;            // the chunk's occupancy in the pool (resident chunks)
  uint8_t nbr_used = 0;         // neighbours (halo-mask bits) its current mesh was built with
  bool rebuild_queued = false;  // waiting in the rebuild queue
  bool rebuild_in_flight = false;
};

enum BatchKind { kLoad = 0, kRebuild = 1 };

// Pinned input bytes a slot holds per chunk: coordinates (12), occupancy slot (4),
// neighbour slots (24), neighbour mask (1), rounded up.
constexpr size_t kInputBytesPerChunk = 48;

struct Slot {
  vox_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t start = nullptr;  // recorded before the batch's first copy
  cudaEvent_t done = nullptr;   // recorded after its offsets reach the host
  double launched_at = 0.0;     // engine clock when `start` was recorded
  bool busy = false;
  int kind = kLoad;
  uint64_t seq = 0;             // launch sequence number
  vox_chunk_coord* d_coords = nullptr;
  uint8_t* d_mask = nullptr;
  int32_t* d_slots = nullptr;      // neighbour-rebuild mode: occupancy slot per chunk
  int32_t* d_nbr_slots = nullptr;  // ... and per chunk and direction (-1: absent)
  uint64_t* d_offsets = nullptr;
  uint64_t* h_offsets = nullptr;  // pinned
  // pinned copies of the batch's inputs (coordinates, masks, occupancy and neighbour slots):
  // the host-to-device copies run asynchronously from them; the slot reuses them only after
  // its batch has finished
  unsigned char* h_inputs = nullptr;
  std::vector<vox_chunk_coord> chunks;
  std::vector<int32_t> occ_slots;  // host copies of d_slots
  std::vector<uint8_t> nbr_used;   // per chunk: the neighbours its mesh is built with
  std::shared_ptr<Block> block;
  uint64_t cap_faces = 0;
};

}  // namespace

struct vox_serve {
  vox_serve_config cfg{};
  vox_sizes sizes{};
  int n = 0;
  int dirs = 4;  // halo directions consulted: the lateral four, or all six (VOX_CULL_FULL6)
  uint64_t bytes_per_face = 0;
  uint64_t est_faces_per_chunk = 0;
  std::vector<Slot> slots;
  uint64_t launch_seq = 0;
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
  // neighbour-rebuild mode: the occupancy pool and its free slots; a freed slot is reused
  // only after every batch launched before it was freed has finished (such a batch may
  // still read it as a neighbour)
  uint32_t* d_occ_pool = nullptr;
  int32_t occ_pool_slots = 0;
  std::vector<int32_t> occ_free;
  std::vector<std::pair<int32_t, uint64_t>> occ_deferred;  // (slot, launch_seq when freed)
  std::vector<vox_chunk_coord> rebuild_queue;
  // state
  FlatMap<vox_chunk_coord, Entry, CoordHash, CoordEq> entries;
  FlatMap<uint64_t, vox_chunk_coord, IdHash, IdEq> by_id;  // request id -> chunk
  uint64_t next_id = 1;
  std::vector<vox_chunk_coord> queue;
  bool queue_sorted = true;  // queue in distance order for the current eye
  std::vector<std::pair<double, double>> latencies;  // (request time, latency in ms)
  vox_serve_stats stats{};
  uint64_t frame = 0;
  double first_request = -1.0, last_completion = -1.0;
  float eye[3] = {0, 0, 0};
};

namespace {

bool rebuild_mode(const vox_serve* s) { return s->cfg.neighbour_rebuild != 0; }

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

// Orders q by distance from the eye, ties in their current order (a stable sort), every
// distance computed once.
void sort_by_distance(const vox_serve* s, std::vector<vox_chunk_coord>& q) {
  const size_t n = q.size();
  std::vector<float> d(n);
  for (size_t i = 0; i < n; ++i) d[i] = dist2(s, q[i]);
  std::vector<uint32_t> order;
  vox::radix_order(d.data(), n, order);
  std::vector<vox_chunk_coord> sorted(n);
  for (size_t i = 0; i < n; ++i) sorted[i] = q[order[i]];
  q.swap(sorted);
}

Entry* resident_entry(vox_serve* s, const vox_chunk_coord& c) {
  auto it = s->entries.find(c);
  return it != s->entries.end() && it->second.state == Entry::RESIDENT ? &it->second : nullptr;
}

// Drops one chunk's reference to its mesh block (freeing the block at zero).
void release_mesh(vox_serve* s, Entry& e) {
  if (e.block) {
    if (--e.block->refs == 0) {
      s->stats.cache_bytes -= e.block->bytes;
      free_block(e.block.get());
    }
    e.block.reset();
  }
  s->stats.faces_resident -= e.faces;
  e.faces = 0;
}

void free_occ_slot(vox_serve* s, int32_t slot) {
  if (slot >= 0) s->occ_deferred.emplace_back(slot, s->launch_seq);
}

// Moves deferred occupancy slots whose readers have all finished to the free list.
void recycle_occ_slots(vox_serve* s) {
  uint64_t oldest = UINT64_MAX;  // sequence number of the oldest batch still on the GPU
  for (const Slot& sl : s->slots)
    if (sl.busy) oldest = std::min(oldest, sl.seq);
  size_t keep = 0;
  for (const auto& d : s->occ_deferred) {
    if (d.second < oldest) s->occ_free.push_back(d.first);
    else s->occ_deferred[keep++] = d;
  }
  s->occ_deferred.resize(keep);
}

void queue_rebuild(vox_serve* s, const vox_chunk_coord& c, Entry& e) {
  if (e.rebuild_queued || e.rebuild_in_flight) return;  // an in-flight rebuild re-checks
  e.rebuild_queued = true;
  s->rebuild_queue.push_back(c);
}

// The halo-mask bits of c's neighbours that are resident now.
uint8_t resident_neighbours(vox_serve* s, const vox_chunk_coord& c) {
  uint8_t m = 0;
  for (int d = 0; d < s->dirs; ++d)
    if (resident_entry(s, neighbour(c, d))) m |= (uint8_t)(1u << d);
  return m;
}

// Evicts one resident chunk: its mesh, its occupancy slot, and (rebuild mode) a rebuild of
// every resident neighbour whose mesh was built against it.
void evict(vox_serve* s, FlatMap<vox_chunk_coord, Entry, CoordHash, CoordEq>::iterator it) {
  const vox_chunk_coord c = it->first;
  Entry& e = it->second;
  release_mesh(s, e);
  free_occ_slot(s, e.occ_slot);
  auto id = s->by_id.find(e.id);
  if (id != s->by_id.end()) s->by_id.erase(id);
  s->entries.erase(it);  // e is gone from here on
  ++s->stats.evicted;
  --s->stats.resident;
  if (!rebuild_mode(s)) return;
  for (int d = 0; d < s->dirs; ++d) {
    const vox_chunk_coord q = neighbour(c, d);
    Entry* y = resident_entry(s, q);
    if (y && ((y->nbr_used >> kOpposite[d]) & 1u)) queue_rebuild(s, q, *y);
  }
}

size_t occ_available(vox_serve* s) {
  recycle_occ_slots(s);
  return s->occ_free.size();
}

// Evicts least-recently-seen resident chunks until `need` more mesh bytes fit in the budget
// and (rebuild mode) `need_occ` occupancy slots are free: first chunks not seen this frame,
// then (when the visible set alone exceeds the budget) visible ones. Returns false if that
// cannot be reached now.
bool evict_lru(vox_serve* s) {
  auto victim = s->entries.end();
  for (int pass = 0; pass < 2 && victim == s->entries.end(); ++pass) {
    for (auto it = s->entries.begin(); it != s->entries.end(); ++it) {
      // chunks whose rebuild is being launched or is on the GPU stay
      if (it->second.state != Entry::RESIDENT || it->second.rebuild_in_flight) continue;
      if (pass == 0 && it->second.last_seen >= s->frame) continue;
      if (victim == s->entries.end() || it->second.last_seen < victim->second.last_seen)
        victim = it;
    }
  }
  if (victim == s->entries.end()) return false;
  evict(s, victim);
  return true;
}

bool make_room(vox_serve* s, uint64_t need, size_t need_occ) {
  if (need > s->cfg.cache_budget_bytes) return false;
  if (rebuild_mode(s) && need_occ > (size_t)s->occ_pool_slots) return false;
  while (s->stats.cache_bytes + need > s->cfg.cache_budget_bytes)
    if (!evict_lru(s)) return false;
  if (need_occ > 0) {
    // slots freed by evictions are reusable once the batches in flight have finished
    while (occ_available(s) + s->occ_deferred.size() < need_occ)
      if (!evict_lru(s)) return false;
    if (occ_available(s) < need_occ) return false;  // retry when those batches finish
  }
  return true;
}

// Launches a batch on slot `sl`: a load batch generates and meshes `chunks` (rebuild mode:
// occupancy into their pool slots `occ`, halo from resident or same-batch neighbours); a
// rebuild batch remeshes resident chunks from the pool.
int launch_batch(vox_serve* s, Slot& sl, int kind, std::vector<vox_chunk_coord>&& chunks,
                 std::vector<int32_t>&& occ) {
  const int m = (int)chunks.size();
  const uint64_t cap = (uint64_t)m * s->est_faces_per_chunk;
  const uint64_t bytes = cap * s->bytes_per_face;
  const bool rb = rebuild_mode(s);
  const size_t need_occ = rb && kind == kLoad && occ.empty() ? (size_t)m : 0;
  if (!make_room(s, bytes, need_occ)) return VOX_ERR_OOM;
  if (need_occ) {
    occ.resize(m);
    for (int i = 0; i < m; ++i) {
      occ[i] = s->occ_free.back();
      s->occ_free.pop_back();
    }
  }
  auto blk = std::make_shared<Block>();
  blk->stream = sl.stream;
  blk->bytes = bytes;
  const uint64_t b0 = s->sizes.bytes_per_face_out0, b1 = s->sizes.bytes_per_face_out1;
  if (cudaMallocAsync(&blk->out0, cap * b0, sl.stream) != cudaSuccess ||
      (b1 && cudaMallocAsync(&blk->out1, cap * b1, sl.stream) != cudaSuccess)) {
    cudaGetLastError();
    free_block(blk.get());
    for (int32_t o : occ)
      if (need_occ) s->occ_free.push_back(o);  // never written: reusable at once
    return VOX_ERR_OOM;
  }
  s->stats.cache_bytes += bytes;
  sl.seq = ++s->launch_seq;
  sl.launched_at = mono_now();
  cudaEventRecord(sl.start, sl.stream);
  // pinned inputs: [coords | occupancy slots | neighbour slots | masks], each 4-byte aligned
  const size_t mcap = (size_t)s->cfg.max_batch;
  vox_chunk_coord* h_coords = reinterpret_cast<vox_chunk_coord*>(sl.h_inputs);
  int32_t* h_slots = reinterpret_cast<int32_t*>(sl.h_inputs + 12 * mcap);
  int32_t* h_nbr = reinterpret_cast<int32_t*>(sl.h_inputs + 16 * mcap);
  uint8_t* h_mask = sl.h_inputs + 40 * mcap;
  std::memcpy(h_coords, chunks.data(), sizeof(vox_chunk_coord) * m);
  cudaMemcpyAsync(sl.d_coords, h_coords, sizeof(vox_chunk_coord) * m, cudaMemcpyHostToDevice,
                  sl.stream);
  int st;
  std::vector<uint8_t> used(m, 0);
  if (!rb) {
    std::memset(h_mask, s->cfg.chunk.cull_mode == VOX_CULL_FULL6 ? 0x3F : 0x0F, (size_t)m);
    cudaMemcpyAsync(sl.d_mask, h_mask, (size_t)m, cudaMemcpyHostToDevice, sl.stream);
    st = vox_gen_mesh_batch(sl.ctx, sl.d_coords, sl.d_mask, m, 0, blk->out0, blk->out1, cap,
                            sl.d_offsets);
  } else {
    // halo sources: a chunk of this batch, else a resident neighbour's pool slot
    std::unordered_map<vox_chunk_coord, int32_t, CoordHash, CoordEq> in_batch;
    if (kind == kLoad)
      for (int i = 0; i < m; ++i) in_batch.emplace(chunks[i], occ[i]);
    std::vector<int32_t> nbr((size_t)6 * m, -1);
    for (int i = 0; i < m; ++i)
      for (int d = 0; d < s->dirs; ++d) {
        const vox_chunk_coord q = neighbour(chunks[i], d);
        int32_t slot = -1;
        auto b = in_batch.find(q);
        if (b != in_batch.end()) slot = b->second;
        else if (const Entry* y = resident_entry(s, q)) slot = y->occ_slot;
        nbr[(size_t)6 * i + d] = slot;
        if (slot >= 0) used[i] |= (uint8_t)(1u << d);
      }
    std::memcpy(h_slots, occ.data(), sizeof(int32_t) * m);
    std::memcpy(h_nbr, nbr.data(), sizeof(int32_t) * 6 * m);
    cudaMemcpyAsync(sl.d_slots, h_slots, sizeof(int32_t) * m, cudaMemcpyHostToDevice, sl.stream);
    cudaMemcpyAsync(sl.d_nbr_slots, h_nbr, sizeof(int32_t) * 6 * m, cudaMemcpyHostToDevice,
                    sl.stream);
    st = kind == kLoad ? vox_generate_slots(sl.ctx, sl.d_coords, m, 0, s->d_occ_pool,
                                            s->occ_pool_slots, sl.d_slots)
                       : VOX_OK;
    if (st == VOX_OK)
      st = vox_mesh_batch(sl.ctx, s->d_occ_pool, s->occ_pool_slots, sl.d_slots, sl.d_nbr_slots,
                          sl.d_coords, m, blk->out0, blk->out1, cap, sl.d_offsets);
  }
  if (st != VOX_OK) {
    // nothing of the batch is kept: the block is freed behind whatever the stream already
    // runs, and the occupancy slots taken above return once that work has finished
    cudaStreamSynchronize(sl.stream);
    s->stats.cache_bytes -= bytes;
    free_block(blk.get());
    if (need_occ)
      for (int32_t o : occ) s->occ_free.push_back(o);
    return st;
  }
  cudaMemcpyAsync(sl.h_offsets, sl.d_offsets, sizeof(uint64_t) * (m + 1), cudaMemcpyDeviceToHost,
                  sl.stream);
  cudaEventRecord(sl.done, sl.stream);
  for (const vox_chunk_coord& c : chunks) {
    auto it = s->entries.find(c);
    if (it == s->entries.end()) continue;
    if (kind == kLoad) it->second.in_flight = true;
    else it->second.rebuild_in_flight = true;
  }
  sl.kind = kind;
  sl.chunks = std::move(chunks);
  sl.occ_slots = std::move(occ);
  sl.nbr_used = std::move(used);
  sl.block = blk;
  sl.cap_faces = cap;
  sl.busy = true;
  if (kind == kLoad) ++s->stats.launches;
  else ++s->stats.rebuild_launches;
  return VOX_OK;
}

// After chunk c became resident or was remeshed (rebuild mode): queue a rebuild of every
// resident neighbour whose mesh did not see c, and of c itself if its resident neighbours
// changed after its mesh was launched (one arrived, or one it saw was evicted).
void schedule_rebuilds(vox_serve* s, const vox_chunk_coord& c, Entry& e) {
  for (int d = 0; d < s->dirs; ++d) {
    const vox_chunk_coord q = neighbour(c, d);
    Entry* y = resident_entry(s, q);
    if (y && !((y->nbr_used >> kOpposite[d]) & 1u)) queue_rebuild(s, q, *y);
  }
  if (resident_neighbours(s, c) != e.nbr_used) queue_rebuild(s, c, e);
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
    const int kind = sl.kind;
    const std::vector<vox_chunk_coord> keep = sl.chunks;
    const std::vector<int32_t> keep_occ = sl.occ_slots;
    std::vector<vox_chunk_coord> again = std::move(sl.chunks);
    std::vector<int32_t> occ = std::move(sl.occ_slots);
    sl.chunks.clear();
    sl.occ_slots.clear();
    if (kind == kLoad && s->stats.launches > 0) --s->stats.launches;
    if (kind == kRebuild && s->stats.rebuild_launches > 0) --s->stats.rebuild_launches;
    const int st = launch_batch(s, sl, kind, std::move(again), std::move(occ));
    if (st == VOX_OK) return VOX_OK;
    // no room to relaunch now: the chunks go back to their queues
    for (size_t i = 0; i < keep.size(); ++i) {
      auto it = s->entries.find(keep[i]);
      if (kind == kLoad) {
        if (!keep_occ.empty()) free_occ_slot(s, keep_occ[i]);
        if (it != s->entries.end() && it->second.in_flight) {
          it->second.in_flight = false;
          s->queue.push_back(keep[i]);
          s->queue_sorted = false;
        }
      } else if (it != s->entries.end() && it->second.state == Entry::RESIDENT &&
                 it->second.rebuild_in_flight) {
        it->second.rebuild_in_flight = false;
        queue_rebuild(s, keep[i], it->second);
      }
    }
    return st == VOX_ERR_OOM ? VOX_OK : st;
  }
  if (status != VOX_OK) return status;
  sl.block->refs = m;
  std::vector<vox_chunk_coord> changed;
  for (int i = 0; i < m; ++i) {
    const vox_chunk_coord c = sl.chunks[i];
    auto it = s->entries.find(c);
    const bool keep = it != s->entries.end() &&
                      (sl.kind == kLoad ? it->second.in_flight
                                        : it->second.rebuild_in_flight &&
                                              it->second.state == Entry::RESIDENT);
    if (!keep) {  // cancelled or evicted meanwhile
      if (--sl.block->refs == 0) {
        s->stats.cache_bytes -= sl.block->bytes;
        free_block(sl.block.get());
      }
      if (sl.kind == kLoad && !sl.occ_slots.empty()) free_occ_slot(s, sl.occ_slots[i]);
      continue;
    }
    Entry& e = it->second;
    if (sl.kind == kLoad) {
      e.in_flight = false;
      e.state = Entry::RESIDENT;
      if (!sl.occ_slots.empty()) e.occ_slot = sl.occ_slots[i];
      ++s->stats.completed;
      ++s->stats.resident;
      --s->stats.pending;
      s->latencies.emplace_back(e.requested_at, (now - e.requested_at) * 1e3);
    } else {
      release_mesh(s, e);
      e.rebuild_in_flight = false;
      ++s->stats.rebuilt;
    }
    e.block = sl.block;
    e.offset = sl.h_offsets[i];
    e.faces = sl.h_offsets[i + 1] - sl.h_offsets[i];
    e.nbr_used = sl.nbr_used[i];
    s->stats.faces_resident += e.faces;
    changed.push_back(c);
  }
  if (rebuild_mode(s))
    for (const vox_chunk_coord& c : changed) {
      Entry* e = resident_entry(s, c);
      if (e) schedule_rebuilds(s, c, *e);
    }
  if (sl.kind == kLoad) s->last_completion = now;
  sl.block.reset();
  sl.chunks.clear();
  sl.occ_slots.clear();
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
  s->queue_sorted = false;
  ++s->stats.requested;
  ++s->stats.pending;
  if (s->first_request < 0.0) s->first_request = now_s;
  return e.id;
}

bool any_busy(const vox_serve* s) {
  for (const Slot& sl : s->slots)
    if (sl.busy) return true;
  return false;
}

// wait: block until the oldest batch in flight has finished (the other slots keep running
// while it is integrated and refilled).
int poll_and_admit(vox_serve* s, bool wait) {
  const Slot* oldest = nullptr;
  if (wait)
    for (const Slot& sl : s->slots)
      if (sl.busy && (!oldest || sl.seq < oldest->seq)) oldest = &sl;
  for (Slot& sl : s->slots) {
    if (!sl.busy) continue;
    cudaError_t q = &sl == oldest ? cudaEventSynchronize(sl.done) : cudaEventQuery(sl.done);
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
  // admit requests first, nearest first; rebuilds take the slots that are left
  const uint64_t per_chunk = s->est_faces_per_chunk * s->bytes_per_face;
  const size_t fit = (size_t)std::max<uint64_t>(1, s->cfg.cache_budget_bytes / per_chunk);
  const size_t batch = std::min<size_t>((size_t)s->cfg.max_batch, fit);
  if (!s->queue.empty()) {
    if (!s->queue_sorted) sort_by_distance(s, s->queue);
    s->queue_sorted = true;
    size_t head = 0;
    for (Slot& sl : s->slots) {
      if (sl.busy || head >= s->queue.size()) continue;
      const size_t take = std::min<size_t>(batch, s->queue.size() - head);
      std::vector<vox_chunk_coord> chunks(s->queue.begin() + head, s->queue.begin() + head + take);
      const int st = launch_batch(s, sl, kLoad, std::move(chunks), {});
      if (st == VOX_ERR_OOM) break;  // the cache is full of visible chunks: retry later
      if (st != VOX_OK) {
        s->queue.erase(s->queue.begin(), s->queue.begin() + head);  // those are on the GPU
        return st;
      }
      head += take;
    }
    s->queue.erase(s->queue.begin(), s->queue.begin() + head);
  }
  if (!s->rebuild_queue.empty() && s->queue.empty()) {
    for (Slot& sl : s->slots) {
      if (sl.busy || s->rebuild_queue.empty()) continue;
      std::vector<vox_chunk_coord> chunks;
      std::vector<int32_t> occ;
      size_t used = 0;
      for (; used < s->rebuild_queue.size() && chunks.size() < batch; ++used) {
        const vox_chunk_coord c = s->rebuild_queue[used];
        Entry* e = resident_entry(s, c);
        if (!e || !e->rebuild_queued) continue;  // evicted since it was queued
        e->rebuild_queued = false;
        e->rebuild_in_flight = true;  // not evicted while its batch is being launched
        chunks.push_back(c);
        occ.push_back(e->occ_slot);
      }
      s->rebuild_queue.erase(s->rebuild_queue.begin(), s->rebuild_queue.begin() + used);
      if (chunks.empty()) continue;
      std::vector<vox_chunk_coord> keep = chunks;
      const int st = launch_batch(s, sl, kRebuild, std::move(chunks), std::move(occ));
      if (st != VOX_OK)
        for (const vox_chunk_coord& c : keep)
          if (Entry* e = resident_entry(s, c)) e->rebuild_in_flight = false;
      if (st == VOX_ERR_OOM) {  // no room for the new meshes now: back to the queue
        for (const vox_chunk_coord& c : keep)
          if (Entry* e = resident_entry(s, c)) queue_rebuild(s, c, *e);
        break;
      }
      if (st != VOX_OK) return st;
    }
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
    s->d_cand = nullptr;
    s->d_vis = nullptr;
    s->h_vis = nullptr;
    s->cand_cap = 0;
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
  s->dirs = cfg->chunk.cull_mode == VOX_CULL_FULL6 ? 6 : 4;
  s->bytes_per_face = s->sizes.bytes_per_face_out0 + s->sizes.bytes_per_face_out1;
  s->est_faces_per_chunk = (uint64_t)4 * s->n * s->n;
  // keep freed blocks in the stream-ordered pool instead of returning them to the CUDA driver
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
        cudaMalloc(&sl.d_slots, sizeof(int32_t) * cfg->max_batch) != cudaSuccess ||
        cudaMalloc(&sl.d_nbr_slots, sizeof(int32_t) * 6 * cfg->max_batch) != cudaSuccess ||
        cudaMalloc(&sl.d_offsets, sizeof(uint64_t) * (cfg->max_batch + 1)) != cudaSuccess ||
        cudaMallocHost(&sl.h_offsets, sizeof(uint64_t) * (cfg->max_batch + 1)) != cudaSuccess ||
        cudaMallocHost(&sl.h_inputs, kInputBytesPerChunk * (size_t)cfg->max_batch) != cudaSuccess)
      return VOX_ERR_OOM;
  }
  if (cfg->neighbour_rebuild) {
    // one occupancy slot per chunk the mesh budget can hold at the estimated faces per
    // chunk, and at least enough for every batch in flight plus one
    const uint64_t per_chunk = s->est_faces_per_chunk * s->bytes_per_face;
    const uint64_t want = std::max<uint64_t>(cfg->cache_budget_bytes / per_chunk,
                                             (uint64_t)cfg->max_batch * (cfg->slots + 1));
    s->occ_pool_slots = (int32_t)std::min<uint64_t>(want, 1u << 20);
    const size_t bytes = (size_t)s->occ_pool_slots * s->sizes.occ_words_per_chunk * 4;
    if (cudaMalloc(&s->d_occ_pool, bytes) != cudaSuccess) return VOX_ERR_OOM;
    s->occ_free.reserve(s->occ_pool_slots);
    for (int32_t k = s->occ_pool_slots - 1; k >= 0; --k) s->occ_free.push_back(k);
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
  for (auto& kv : s->entries) release_mesh(s, kv.second);
  for (Slot& sl : s->slots) {
    if (sl.block) free_block(sl.block.get());
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    vox_ctx_destroy(sl.ctx);
    cudaFree(sl.d_coords);
    cudaFree(sl.d_mask);
    cudaFree(sl.d_slots);
    cudaFree(sl.d_nbr_slots);
    cudaFree(sl.d_offsets);
    if (sl.h_offsets) cudaFreeHost(sl.h_offsets);
    if (sl.h_inputs) cudaFreeHost(sl.h_inputs);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.start) cudaEventDestroy(sl.start);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  vox_ctx_destroy(s->cull_ctx);
  cudaFree(s->d_cand);
  cudaFree(s->d_vis);
  cudaFree(s->d_occ_pool);
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
  if (std::memcmp(s->eye, eye, sizeof s->eye) != 0) s->queue_sorted = false;
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
  // room for every new request at once (no rehash per growth step)
  s->entries.reserve(s->entries.size() + (size_t)n);
  s->by_id.reserve(s->by_id.size() + (size_t)n);
  s->queue.reserve(s->queue.size() + (size_t)n);
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
    if (!any_busy(s) && !s->queue.empty()) return VOX_ERR_OOM;  // the budget cannot hold its batch
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
    if (!any_busy(s) && s->queue.empty() && s->rebuild_queue.empty()) return VOX_OK;
    const int st = poll_and_admit(s, true);
    if (st != VOX_OK) return st;
    // nothing in flight and nothing admitted: the budget cannot hold the next batch
    if (!any_busy(s) && (!s->queue.empty() || !s->rebuild_queue.empty())) return VOX_ERR_OOM;
  }
}

int vox_serve_get_stats(vox_serve* s, vox_serve_stats* out) {
  if (!s || !out) return VOX_ERR_INVALID;
  *out = s->stats;
  double p50 = 0, p99 = 0, mx = 0;
  uint64_t cnt = 0;
  vox_serve_latency(s, -1e300, &p50, &p99, &mx, &cnt);
  out->latency_p50_ms = p50;
  out->latency_p99_ms = p99;
  out->latency_max_ms = mx;
  out->busy_s = s->first_request >= 0.0 && s->last_completion >= 0.0
                    ? s->last_completion - s->first_request
                    : 0.0;
  return VOX_OK;
}

int vox_serve_latency(vox_serve* s, double requested_after_s, double* p50_ms, double* p99_ms,
                      double* max_ms, uint64_t* count) {
  if (!s) return VOX_ERR_INVALID;
  std::vector<double> v;
  v.reserve(s->latencies.size());
  for (const auto& l : s->latencies)
    if (l.first >= requested_after_s) v.push_back(l.second);
  auto pct = [&](double q) {
    if (v.empty()) return 0.0;
    size_t k = (size_t)std::min<double>((double)v.size() - 1, std::floor(q * (double)v.size()));
    std::nth_element(v.begin(), v.begin() + (long)k, v.end());
    return v[k];
  };
  if (p50_ms) *p50_ms = pct(0.50);
  if (p99_ms) *p99_ms = pct(0.99);
  if (max_ms) *max_ms = v.empty() ? 0.0 : *std::max_element(v.begin(), v.end());
  if (count) *count = (uint64_t)v.size();
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
