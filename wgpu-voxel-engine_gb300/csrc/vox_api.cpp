// vox_api.cpp — the C ABI (include/voxgpu.h): contexts, argument checks, launches.
//
// Host code only; kernels are reached through the KernelSet tables of the per-size
// translation units. Every CUDA failure becomes a status code plus a message kept in
// the context; nothing here aborts the process (the reference panics via unwrap where
// these calls return an error).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "voxgpu.h"
#include "vox_kernels.h"
#include "vox_tables.h"
#include "vox_trace.h"
#include "vox_types.h"

using namespace vox;

// Staging windows of a warp: one 32-face buffer (32) or two (64).
constexpr int kStageSingle = 32;
constexpr int kStageDouble = 64;

// Buffers of the staged-halo path for batches of up to `cap` chunks (see vox_halo.cu): the
// coordinate hash map, the neighbour slots, the identity slots, the neighbours outside the
// batch and their count, and the occupancy pool (cap * (1 + dirs) slots).
struct HaloScratch {
  size_t cap = 0;
  int dirs = 4;
  unsigned long long* keys = nullptr;
  int* vals = nullptr;
  unsigned cap_mask = 0;
  int* nbr = nullptr;
  int* ident = nullptr;
  vox_chunk_coord* extra = nullptr;
  uint8_t* extra_dir = nullptr;
  unsigned* extra_count = nullptr;
  uint32_t* pool = nullptr;

  void release() {
    cudaFree(keys);
    cudaFree(vals);
    cudaFree(nbr);
    cudaFree(ident);
    cudaFree(extra);
    cudaFree(extra_dir);
    cudaFree(extra_count);
    cudaFree(pool);
    *this = HaloScratch{};
  }
};

struct vox_ctx {
  vox_config cfg{};
  int device = 0;
  int num_sms = 0;
  int max_smem_optin = 0;  // shared memory one block may opt in to
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::mutex mu;
  const KernelSet* ks = nullptr;
  GenDev gen{};
  int gm = GM_HEIGHT;
  // tuning: CTA-size option, staging window (0 = direct stores), resident CTAs per SM,
  // schedule (look-back, phased or overlap)
  int topt = 0;
  int stage_faces = 0;
  int ctas_per_sm = 0;
  int schedule = VOX_SCHEDULE_LOOKBACK;
  int spin_limit = kSpinLimit;
  int slab_chunks = 0;  // chunks per launch of a batch (0: the whole batch in one launch)
  int halo_staging = 0; // 0: halos regenerated in the fused launch; 1: staged from a pool
  HaloScratch halo;     // the staged-halo path's buffers
  int batch_grid[4] = {0, 0, 0, 0};   // persistent grid per gen mode (look-back kernel)
  int phased_grid[4] = {0, 0, 0, 0};  // co-resident grid per gen mode (phased kernel)
  int overlap_grid[4] = {0, 0, 0, 0}; // persistent grid per gen mode (overlap kernel)
  int host_grid[4] = {0, 0, 0, 0};    // grid of launches that write host memory (staged)
  // phased and overlap schedules: per-chunk occupancy + halo spill and face totals
  uint32_t* d_scratch = nullptr;
  uint32_t* d_counts = nullptr;
  size_t scratch_cap = 0;  // chunks
  TablesDev* d_tables = nullptr;
  TablesDev h_tables{};  // the fused batch kernels take the tables as a kernel parameter
  BatchCtl* d_ctl = nullptr;
  BatchCtl* h_ctl = nullptr;  // pinned
  unsigned* h_err_mirror = nullptr;  // page-locked, mapped: status of host-output launches
  unsigned* d_err_mirror = nullptr;  // its device address
  unsigned long long* d_state = nullptr;
  size_t state_cap = 0;
  unsigned long long launches = 0;
  // buffers of the host-pointer entry point
  void* d_in = nullptr;
  size_t in_cap = 0;
  unsigned long long* d_offsets = nullptr;
  size_t offsets_cap = 0;
  void* d_out0 = nullptr;
  void* d_out1 = nullptr;
  size_t out_cap_faces = 0;
  std::string last_error;
};

// One captured fused batch launch (vox_graph_capture). The graph owns the scratch of its
// schedule, so later calls on the context never move a buffer the graph points at; the
// queue/epoch/error word is the context's (launches on one stream never overlap).
struct vox_graph {
  vox_ctx* ctx = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int schedule = VOX_SCHEDULE_LOOKBACK;
  unsigned long long* d_state = nullptr;  // look-back states (n)
  uint32_t* d_scratch = nullptr;          // phased: occupancy + halo spill (n chunks)
  uint32_t* d_counts = nullptr;           // phased: face totals (n)
  size_t state_bytes = 0;
  unsigned long long wiped_at = 0;        // context launch count when d_state was zeroed
  int launches = 1;                       // kernel launches per replay (slabs of the batch)
  HaloScratch halo;                       // staged-halo buffers of the captured batch
};

namespace {

int fail(vox_ctx* ctx, int status, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->last_error = buf;
  }
  return status;
}

int cuda_fail(vox_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? VOX_ERR_OOM : VOX_ERR_CUDA, "%s: %s (%s)",
              what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define VOX_CUDA(ctx, call, what)                  \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
  } while (0)

const KernelSet* kernel_set_for(int n) {
  switch (n) {
    case 8: return &kernel_set_8();
    case 16: return &kernel_set_16();
    case 32: return &kernel_set_32();
    case 64: return &kernel_set_64();
    default: return nullptr;
  }
}

int words_per_chunk(int n) { return n * n * (n > 32 ? n / 32 : 1); }
int bytes_out0(int layout) { return layout == VOX_LAYOUT_INSTANCED ? 68 : 96; }
int bytes_out1(int layout) { return layout == VOX_LAYOUT_INSTANCED ? 0 : 24; }

int validate_config(const vox_config* c, std::string* why) {
  if (!c) {
    *why = "config is NULL";
    return VOX_ERR_INVALID;
  }
  if (!kernel_set_for(c->chunk_size)) {
    *why = "chunk_size must be 8, 16, 32 or 64";
    return VOX_ERR_INVALID;
  }
  if (c->cull_mode != VOX_CULL_REFERENCE && c->cull_mode != VOX_CULL_FULL6) {
    *why = "unknown cull_mode";
    return VOX_ERR_INVALID;
  }
  if (c->layout != VOX_LAYOUT_VERTEX && c->layout != VOX_LAYOUT_INSTANCED) {
    *why = "unknown layout";
    return VOX_ERR_INVALID;
  }
  const vox_generator& g = c->gen;
  if (g.kind != VOX_GEN_HEIGHTMAP && g.kind != VOX_GEN_DENSITY && g.kind != VOX_GEN_BERNOULLI) {
    *why = "unknown generator kind";
    return VOX_ERR_INVALID;
  }
  if (g.kind != VOX_GEN_BERNOULLI && (g.octaves < 1 || g.octaves > 16)) {
    *why = "octaves must be in 1..16";
    return VOX_ERR_INVALID;
  }
  return VOX_OK;
}

int gen_mode_of(int kind) {
  switch (kind) {
    case VOX_GEN_HEIGHTMAP: return GM_HEIGHT;
    case VOX_GEN_DENSITY: return GM_DENSITY;
    default: return GM_BERNOULLI;
  }
}

// The default tuning (before any autotuning), the shape that measured fastest on the
// heightmap, density and stress batches: the overlap schedule with one staging buffer per
// warp, and the larger CTA size for chunks up to 32^3.
constexpr int kDefaultSchedule = VOX_SCHEDULE_OVERLAP;
int default_topt(int chunk_size) { return chunk_size <= 32 ? 1 : 0; }

// Allows `fn` up to `smem` bytes of dynamic shared memory (capped at what the device
// grants one block beyond the kernel's static shared memory).
int prepare_kernel(vox_ctx* ctx, const void* fn, int smem) {
  cudaFuncAttributes fa;
  VOX_CUDA(ctx, cudaFuncGetAttributes(&fa, fn), "cudaFuncGetAttributes");
  const int limit = ctx->max_smem_optin - (int)fa.sharedSizeBytes;
  VOX_CUDA(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     std::min(smem, limit)),
           "cudaFuncSetAttribute");
  return VOX_OK;
}

// Validates a tuning and computes the persistent grid of every generator mode for it.
int apply_tuning(vox_ctx* ctx, int topt, int stage_faces, int ctas_per_sm, int schedule,
                 int slab_chunks, int halo_staging) {
  const KernelSet& ks = *ctx->ks;
  const int layout = ctx->cfg.layout;
  if (topt < 0 || topt > 1) return fail(ctx, VOX_ERR_INVALID, "unsupported CTA size");
  if (slab_chunks < 0) return fail(ctx, VOX_ERR_INVALID, "slab_chunks must be >= 0");
  if (halo_staging != 0 && halo_staging != 1)
    return fail(ctx, VOX_ERR_INVALID, "halo_staging must be 0 (regenerate) or 1 (pool)");
  if (stage_faces != 0 && stage_faces != kStageSingle && stage_faces != kStageDouble)
    return fail(ctx, VOX_ERR_INVALID, "stage_faces must be 0 (direct stores), %d or %d",
                kStageSingle, kStageDouble);
  if (ctas_per_sm < 0) return fail(ctx, VOX_ERR_INVALID, "ctas_per_sm must be >= 0");
  if (schedule != VOX_SCHEDULE_LOOKBACK && schedule != VOX_SCHEDULE_PHASED &&
      schedule != VOX_SCHEDULE_OVERLAP)
    return fail(ctx, VOX_ERR_INVALID, "unknown schedule");
  const int smem = ks.smem_total(layout, ks.threads[topt], stage_faces);
  if (smem > ctx->max_smem_optin - 256)
    return fail(ctx, VOX_ERR_INVALID, "staging window exceeds shared memory");
  int grid[4], pgrid[4], hgrid[4], ogrid[4];
  const int hsmem = ks.smem_total(layout, ks.threads[topt], kStageSingle);
  for (int gm = 0; gm < 4; ++gm) {
    for (int k = 0; k < 4; ++k) {
      // the phased kernel's grid must be co-resident (cooperative launch): its occupancy
      // is an upper bound, never exceeded. k = 3: the selected schedule's kernel with one
      // staging buffer per warp (launches whose outputs are in host memory)
      const void* fn = k == 0 ? ks.batch[gm][layout][topt]
                     : k == 1 ? ks.phased[gm][layout][topt]
                     : k == 2 ? ks.overlap[gm][layout][topt]
                     : schedule == VOX_SCHEDULE_PHASED  ? ks.phased[gm][layout][topt]
                     : schedule == VOX_SCHEDULE_OVERLAP ? ks.overlap[gm][layout][topt]
                                                        : ks.batch[gm][layout][topt];
      int per_sm = 0;
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, ks.threads[topt],
                                                                    k == 3 ? hsmem : smem);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
      if (per_sm < 1) return fail(ctx, VOX_ERR_INVALID, "kernel does not fit on an SM");
      if (ctas_per_sm > 0) per_sm = std::min(per_sm, ctas_per_sm);
      (k == 0 ? grid : k == 1 ? pgrid : k == 2 ? ogrid : hgrid)[gm] = per_sm * ctx->num_sms;
    }
  }
  ctx->topt = topt;
  ctx->stage_faces = stage_faces;
  ctx->ctas_per_sm = ctas_per_sm;
  ctx->schedule = schedule;
  ctx->slab_chunks = slab_chunks;
  ctx->halo_staging = halo_staging;
  for (int gm = 0; gm < 4; ++gm) {
    ctx->batch_grid[gm] = grid[gm];
    ctx->phased_grid[gm] = pgrid[gm];
    ctx->overlap_grid[gm] = ogrid[gm];
    ctx->host_grid[gm] = hgrid[gm];
  }
  return VOX_OK;
}

// Scratch of the phased schedule for n chunks (grows; never shrinks).
int ensure_scratch(vox_ctx* ctx, size_t n) {
  if (n <= ctx->scratch_cap) return VOX_OK;
  const size_t cap = std::max<size_t>(n, 1024);
  cudaFree(ctx->d_scratch);
  cudaFree(ctx->d_counts);
  ctx->d_scratch = nullptr;
  ctx->d_counts = nullptr;
  ctx->scratch_cap = 0;
  VOX_CUDA(ctx, cudaMalloc(&ctx->d_scratch, cap * (size_t)ctx->ks->spill_bytes),
           "cudaMalloc(scratch)");
  VOX_CUDA(ctx, cudaMalloc(&ctx->d_counts, cap * sizeof(uint32_t)), "cudaMalloc(counts)");
  ctx->scratch_cap = cap;
  return VOX_OK;
}

int ensure_state(vox_ctx* ctx, size_t n) {
  if (n <= ctx->state_cap) return VOX_OK;
  size_t cap = std::max<size_t>(n, 1024);
  if (ctx->d_state) cudaFree(ctx->d_state);
  ctx->d_state = nullptr;
  ctx->state_cap = 0;
  VOX_CUDA(ctx, cudaMalloc(&ctx->d_state, cap * sizeof(unsigned long long)), "cudaMalloc(state)");
  VOX_CUDA(ctx, cudaMemsetAsync(ctx->d_state, 0, cap * sizeof(unsigned long long), ctx->stream),
           "cudaMemsetAsync(state)");
  ctx->state_cap = cap;
  return VOX_OK;
}

// Look-back states are tagged with a 24-bit launch epoch. A launch advances it by one, and a
// launch that timed out by at most two (the host moves a failed launch to a fresh epoch), so
// a wipe every 2^22 launches comes well before a tag can repeat.
constexpr unsigned long long kStateWipePeriod = 1ull << 22;
int before_batch_launch(vox_ctx* ctx) {
  if (ctx->launches > 0 && (ctx->launches & (kStateWipePeriod - 1)) == 0 && ctx->d_state) {
    VOX_CUDA(ctx, cudaMemsetAsync(ctx->d_state, 0, ctx->state_cap * sizeof(unsigned long long),
                                  ctx->stream),
             "cudaMemsetAsync(state)");
  }
  ++ctx->launches;
  return VOX_OK;
}

MeshArgs base_args(vox_ctx* ctx) {
  MeshArgs a;
  std::memset(&a, 0, sizeof a);
  a.tables = ctx->d_tables;
  a.ctl = ctx->d_ctl;
  a.state = ctx->d_state;
  a.gen = ctx->gen;
  a.full6 = ctx->cfg.cull_mode == VOX_CULL_FULL6 ? 1 : 0;
  a.stage_faces = ctx->stage_faces;
  a.spin_limit = ctx->spin_limit;
  a.scratch = ctx->d_scratch;
  a.counts = ctx->d_counts;
  return a;
}

int launch(vox_ctx* ctx, const void* fn, int grid, int threads, int smem, void** params) {
  VOX_CUDA(ctx, cudaLaunchKernel(fn, dim3(grid), dim3(threads), params, (size_t)smem, ctx->stream),
           "cudaLaunchKernel");
  return VOX_OK;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

int check_outputs(vox_ctx* ctx, void* out0, void* out1, uint64_t cap) {
  if (cap == 0) return VOX_OK;
  if (!out0) return fail(ctx, VOX_ERR_INVALID, "out0 is NULL with cap_faces > 0");
  // Outputs are written with TMA bulk copies, which need 16-byte aligned addresses.
  if (ctx->cfg.layout == VOX_LAYOUT_VERTEX) {
    if (!out1) return fail(ctx, VOX_ERR_INVALID, "out1 (indices) is NULL with cap_faces > 0");
    if (!aligned(out0, 16) || !aligned(out1, 16))
      return fail(ctx, VOX_ERR_INVALID, "vertex and index outputs must be 16-byte aligned");
  } else if (!aligned(out0, 16)) {
    return fail(ctx, VOX_ERR_INVALID, "instance output must be 16-byte aligned");
  }
  return VOX_OK;
}

// Issues one fused batch launch with the context's tuning on `stream`; the scratch of the
// schedule (a.state, or a.scratch + a.counts) is already in `a`.
int issue_batch(vox_ctx* ctx, MeshArgs& a, int gm, bool host_out, cudaStream_t stream) {
  const int layout = ctx->cfg.layout;
  const int threads = ctx->ks->threads[ctx->topt];
  const int smem = ctx->ks->smem_total(layout, threads, host_out ? kStageSingle : ctx->stage_faces);
  if (host_out) {
    a.stage_faces = kStageSingle;
    a.lane_flush = 1;
  }
  void* params[] = {&a, &ctx->h_tables};
  if (ctx->schedule == VOX_SCHEDULE_PHASED || ctx->schedule == VOX_SCHEDULE_OVERLAP) {
    const bool phased = ctx->schedule == VOX_SCHEDULE_PHASED;
    const void* fn = (phased ? ctx->ks->phased : ctx->ks->overlap)[gm][layout][ctx->topt];
    const int grid = std::max(1, std::min(a.n, host_out ? ctx->host_grid[gm]
                                             : phased ? ctx->phased_grid[gm] : ctx->overlap_grid[gm]));
    // emission items per chunk: one for small chunks unless there are fewer chunks than
    // CTAs; chunks of 32^3 and up (whose emission dwarfs an item's reload) split until
    // there are about eight items per CTA, which evens out the last wave
    a.split = ctx->cfg.chunk_size >= 32 ? std::max(1, std::min(8, (8 * grid + a.n - 1) / a.n))
                                        : std::max(1, std::min(8, grid / a.n));
    // n + n * split (generation and emission tickets) fits an int
    a.split = std::max(1, std::min(a.split, (0x7FFFFFFF - a.n) / a.n));
    // overlap kernel: with outputs in host memory, emission (bound by the host link) runs
    // two waves of generation items behind, which hides the generation behind the link
    // (density 4096 x 32^3: 4.92 -> 4.25 ms); otherwise every chunk is generated first
    a.lag = host_out ? 2 * grid : -1;
    if (phased)
      VOX_CUDA(ctx, cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), params, (size_t)smem,
                                                stream),
               "cudaLaunchCooperativeKernel");
    else
      VOX_CUDA(ctx, cudaLaunchKernel(fn, dim3(grid), dim3(threads), params, (size_t)smem, stream),
               "cudaLaunchKernel");
    return VOX_OK;
  }
  const void* fn = ctx->ks->batch[gm][layout][ctx->topt];
  const int grid = std::max(1, std::min(a.n, host_out ? ctx->host_grid[gm] : ctx->batch_grid[gm]));
  VOX_CUDA(ctx, cudaLaunchKernel(fn, dim3(grid), dim3(threads), params, (size_t)smem, stream),
           "cudaLaunchKernel");
  return VOX_OK;
}

// Chunks per launch of a batch of n chunks under the context's tuning.
int slab_of(const vox_ctx* ctx, int n) {
  return ctx->slab_chunks > 0 && ctx->slab_chunks < n ? ctx->slab_chunks : n;
}

// Cuts the batch `a` into launches of `slab` chunks and calls issue(b) for each, in order.
// Launch k covers chunks [k * slab, ...): its inputs, offsets and chunk-index base are
// shifted, and its faces follow the previous launch's (base_ptr = its own face_offsets[0],
// which the previous launch on the same stream wrote as its total), so the slabs together
// write exactly what one launch over the batch writes.
template <typename F>
int for_each_slab(const MeshArgs& a, int slab, F&& issue) {
  for (int s = 0; s < a.n; s += slab) {
    MeshArgs b = a;
    b.n = std::min(slab, a.n - s);
    b.index_base = a.index_base + s;
    if (a.coords) b.coords = a.coords + s;
    if (a.nbr_mask) b.nbr_mask = a.nbr_mask + s;
    if (a.slots) b.slots = a.slots + s;
    if (a.nbr_slots) b.nbr_slots = a.nbr_slots + 6 * (size_t)s;
    b.face_offsets = a.face_offsets + s;
    b.base_ptr = s == 0 ? nullptr : a.face_offsets + s;
    const int st = issue(b);
    if (st != VOX_OK) return st;
  }
  return VOX_OK;
}

// Staged-halo buffers for batches of n chunks (grow; never shrink).
int ensure_halo(vox_ctx* ctx, HaloScratch& h, size_t n) {
  const int dirs = ctx->cfg.cull_mode == VOX_CULL_FULL6 ? 6 : 4;
  if (n <= h.cap && h.dirs == dirs) return VOX_OK;
  h.release();
  const size_t cap = std::max<size_t>(n, 256);
  size_t slots = 1;
  while (slots < 2 * cap) slots <<= 1;
  const size_t words = (size_t)ctx->ks->n_size * ctx->ks->n_size *
                       (ctx->ks->n_size > 32 ? ctx->ks->n_size / 32 : 1);
  cudaError_t e;
  if ((e = cudaMalloc(&h.keys, slots * sizeof(unsigned long long))) != cudaSuccess ||
      (e = cudaMalloc(&h.vals, slots * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&h.nbr, 6 * cap * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&h.ident, cap * sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&h.extra, (size_t)dirs * cap * sizeof(vox_chunk_coord))) != cudaSuccess ||
      (e = cudaMalloc(&h.extra_dir, (size_t)dirs * cap)) != cudaSuccess ||
      (e = cudaMalloc(&h.extra_count, sizeof(unsigned))) != cudaSuccess ||
      (e = cudaMalloc(&h.pool, (1 + (size_t)dirs) * cap * words * sizeof(uint32_t))) != cudaSuccess) {
    h.release();
    return cuda_fail(ctx, e, "cudaMalloc(halo staging)");
  }
  h.cap = cap;
  h.dirs = dirs;
  h.cap_mask = (unsigned)(slots - 1);
  return VOX_OK;
}

// The staged-halo pre-pass of a fused batch `a` (generator mode gm): the neighbour lookup,
// then every chunk of the batch generated into the pool, and for every loaded neighbour
// outside it the one plane its batch neighbour reads; `a` becomes the equivalent batch over
// resident occupancy (GM_OCC). The bytes it then writes are the fused launch's: a halo
// plane read from the neighbour's occupancy is the plane the fused launch generates
// (generation is a function of the voxel's world position; Bernoulli chunks have no
// neighbours).
int halo_prepass(vox_ctx* ctx, MeshArgs& a, int gm, HaloScratch& h, cudaStream_t stream) {
  const size_t words = (size_t)ctx->ks->n_size * ctx->ks->n_size *
                       (ctx->ks->n_size > 32 ? ctx->ks->n_size / 32 : 1);
  HaloLookup hl;
  hl.coords = a.coords;
  hl.masks = gm == GM_BERNOULLI ? nullptr : a.nbr_mask;
  hl.n = a.n;
  hl.dirs = h.dirs;
  hl.keys = h.keys;
  hl.vals = h.vals;
  hl.cap_mask = h.cap_mask;
  hl.nbr_slots = h.nbr;
  hl.ident = h.ident;
  hl.extra = h.extra;
  hl.extra_dir = h.extra_dir;
  hl.extra_count = h.extra_count;
  hl.err = &ctx->d_ctl->err;
  VOX_CUDA(ctx, launch_halo_lookup(hl, stream), "halo lookup");
  const int gsmem = ctx->ks->smem_total(VOX_LAYOUT_VERTEX, ctx->ks->gen_threads, 0);
  MeshArgs g = base_args(ctx);
  g.n = a.n;
  g.index_base = a.index_base;
  g.coords = a.coords;
  uint32_t* own = h.pool;
  void* p1[] = {&g, &own};
  VOX_CUDA(ctx, cudaLaunchKernel(ctx->ks->generate[gm], dim3(a.n), dim3(ctx->ks->gen_threads), p1,
                                 (size_t)gsmem, stream),
           "generate (pool)");
  if (hl.masks) {
    MeshArgs x = base_args(ctx);
    x.n = h.dirs * a.n;
    x.coords = h.extra;
    x.n_dev = h.extra_count;
    const uint8_t* xdir = h.extra_dir;
    uint32_t* ext = h.pool + (size_t)a.n * words;
    void* p2[] = {&x, &xdir, &ext};
    // the count is known on the device only: a grid of 2 CTAs per SM loops over it
    const int grid = std::max(1, std::min(x.n, 2 * ctx->num_sms));
    VOX_CUDA(ctx, cudaLaunchKernel(ctx->ks->generate_planes[gm], dim3(grid), dim3(ctx->ks->gen_threads),
                                   p2, (size_t)gsmem, stream),
             "generate (halo planes outside the batch)");
  }
  a.occ_pool = h.pool;
  a.pool_slots = (1 + h.dirs) * a.n;
  a.slots = h.ident;
  a.nbr_slots = h.nbr;
  return VOX_OK;
}

// host_out: the outputs are in host memory; the launch stages every warp's faces in one
// shared-memory buffer and writes them out with plain full-line stores.
int batch_launch(vox_ctx* ctx, MeshArgs& a, int gm, bool host_out = false) {
  int st;
  // Outputs in host memory keep the fused launch: its emission, bound by the host link,
  // overlaps the generation, which the staged-halo path runs first.
  if (ctx->halo_staging && gm != GM_OCC && !host_out) {
    if ((st = ensure_halo(ctx, ctx->halo, (size_t)a.n)) != VOX_OK) return st;
    if ((st = halo_prepass(ctx, a, gm, ctx->halo, ctx->stream)) != VOX_OK) return st;
    gm = GM_OCC;
  }
  const int slab = slab_of(ctx, a.n);
  if (ctx->schedule != VOX_SCHEDULE_LOOKBACK) {  // the spill slots of phases A and C
    if ((st = ensure_scratch(ctx, (size_t)slab)) != VOX_OK) return st;
    a.scratch = ctx->d_scratch;
    a.counts = ctx->d_counts;
  }
  if (ctx->schedule != VOX_SCHEDULE_PHASED) {  // look-back state words
    if ((st = ensure_state(ctx, (size_t)slab)) != VOX_OK) return st;
    a.state = ctx->d_state;
  }
  return for_each_slab(a, slab, [&](MeshArgs& b) {
    if (ctx->schedule == VOX_SCHEDULE_PHASED) {
      ++ctx->launches;
    } else {
      const int s2 = before_batch_launch(ctx);
      if (s2 != VOX_OK) return s2;
    }
    return issue_batch(ctx, b, gm, host_out, ctx->stream);
  });
}

}  // namespace

extern "C" {

int vox_abi_version(void) { return VOX_ABI_VERSION; }

const char* vox_status_string(int s) {
  switch (s) {
    case VOX_OK: return "ok";
    case VOX_ERR_INVALID: return "invalid argument";
    case VOX_ERR_OOM: return "out of memory";
    case VOX_ERR_CUDA: return "CUDA error";
    case VOX_ERR_TIMEOUT: return "device wait timed out";
    case VOX_ERR_CAPACITY: return "output capacity exceeded";
    case VOX_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

int vox_query_sizes(const vox_config* cfg, vox_sizes* out) {
  std::string why;
  if (validate_config(cfg, &why) != VOX_OK || !out) return VOX_ERR_INVALID;
  const int n = cfg->chunk_size;
  out->occ_words_per_chunk = (uint32_t)words_per_chunk(n);
  out->bytes_per_face_out0 = (uint32_t)bytes_out0(cfg->layout);
  out->bytes_per_face_out1 = (uint32_t)bytes_out1(cfg->layout);
  out->max_faces_per_chunk = (uint32_t)(3 * n * n * n + 6 * n * n);
  return VOX_OK;
}

int vox_ctx_create(const vox_config* cfg, void* stream, vox_ctx** out) {
  if (!out) return VOX_ERR_INVALID;
  *out = nullptr;
  std::string why;
  if (validate_config(cfg, &why) != VOX_OK) {
    std::fprintf(stderr, "voxgpu: invalid config: %s\n", why.c_str());
    return VOX_ERR_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return VOX_ERR_NO_DEVICE;
  }
  vox_ctx* ctx = new (std::nothrow) vox_ctx();
  if (!ctx) return VOX_ERR_OOM;
  ctx->cfg = *cfg;
  ctx->ks = kernel_set_for(cfg->chunk_size);
  const vox_generator& g = cfg->gen;
  ctx->gen.kind = g.kind;
  ctx->gen.octaves = g.octaves;
  ctx->gen.seed = g.seed;
  ctx->gen.freq = g.frequency;
  ctx->gen.lac = g.lacunarity;
  ctx->gen.gain = g.gain;
  ctx->gen.amp = g.amplitude;
  ctx->gen.base = g.base_height;
  ctx->gen.y_ref = g.y_ref;
  ctx->gen.y_scale = g.y_scale;
  ctx->gen.solid_below_zero = g.solid_below_zero;
  ctx->gm = gen_mode_of(g.kind);
  int st = VOX_OK;
  auto cleanup = [&](int s) {
    std::fprintf(stderr, "voxgpu: vox_ctx_create failed (%s): %s\n", vox_status_string(s),
                 ctx->last_error.c_str());
    vox_ctx_destroy(ctx);
    return s;
  };
  if (cudaGetDevice(&ctx->device) != cudaSuccess) return cleanup(cuda_fail(ctx, cudaGetLastError(), "cudaGetDevice"));
  if (cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                             ctx->device) != cudaSuccess)
    return cleanup(cuda_fail(ctx, cudaGetLastError(), "cudaDeviceGetAttribute"));
  if (stream) {
    ctx->stream = static_cast<cudaStream_t>(stream);
  } else {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
      return cleanup(VOX_ERR_CUDA);
    ctx->own_stream = true;
  }
  TablesDev tab;
  build_tables(*cfg, tab);
  ctx->h_tables = tab;
  if (cudaMalloc(&ctx->d_tables, sizeof(TablesDev)) != cudaSuccess) return cleanup(VOX_ERR_OOM);
  if (cudaMemcpy(ctx->d_tables, &tab, sizeof tab, cudaMemcpyHostToDevice) != cudaSuccess)
    return cleanup(VOX_ERR_CUDA);
  if (cudaMalloc(&ctx->d_ctl, sizeof(BatchCtl)) != cudaSuccess) return cleanup(VOX_ERR_OOM);
  if (cudaMemset(ctx->d_ctl, 0, sizeof(BatchCtl)) != cudaSuccess) return cleanup(VOX_ERR_CUDA);
  if (cudaMallocHost(&ctx->h_ctl, sizeof(BatchCtl)) != cudaSuccess) return cleanup(VOX_ERR_OOM);
  if (cudaHostAlloc(&ctx->h_err_mirror, sizeof(unsigned), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer(&ctx->d_err_mirror, ctx->h_err_mirror, 0) != cudaSuccess)
    return cleanup(VOX_ERR_OOM);
  *ctx->h_err_mirror = 0u;
  // Every meshing kernel may use up to the full shared memory of an SM; the tuning
  // decides how much a launch actually takes.
  const int layout = cfg->layout;
  for (int gm = 0; gm < 4; ++gm)
    for (int t = 0; t < 2; ++t)
      if ((st = prepare_kernel(ctx, ctx->ks->batch[gm][layout][t], ctx->max_smem_optin)) != VOX_OK ||
          (st = prepare_kernel(ctx, ctx->ks->phased[gm][layout][t], ctx->max_smem_optin)) != VOX_OK ||
          (st = prepare_kernel(ctx, ctx->ks->overlap[gm][layout][t], ctx->max_smem_optin)) != VOX_OK)
        return cleanup(st);
  for (int t = 0; t < 2; ++t)
    if ((st = prepare_kernel(ctx, ctx->ks->single[layout][t], ctx->max_smem_optin)) != VOX_OK)
      return cleanup(st);
  const int gsmem = ctx->ks->smem_total(VOX_LAYOUT_VERTEX, ctx->ks->gen_threads, 0);
  for (int gm = 1; gm < 4; ++gm)
    if ((st = prepare_kernel(ctx, ctx->ks->generate[gm], gsmem)) != VOX_OK ||
        (ctx->ks->generate_planes[gm] &&
         (st = prepare_kernel(ctx, ctx->ks->generate_planes[gm], gsmem)) != VOX_OK))
      return cleanup(st);
  if (apply_tuning(ctx, default_topt(cfg->chunk_size), kStageSingle, 0, kDefaultSchedule, 0, 0) != VOX_OK &&
      (st = apply_tuning(ctx, 0, 0, 0, kDefaultSchedule, 0, 0)) != VOX_OK)  // no room to stage
    return cleanup(st);
  ctx->last_error.clear();
  if ((st = ensure_state(ctx, 1024)) != VOX_OK) return cleanup(st);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return cleanup(VOX_ERR_CUDA);
  *out = ctx;
  return VOX_OK;
}

int vox_ctx_destroy(vox_ctx* ctx) {
  if (!ctx) return VOX_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_tables);
  cudaFree(ctx->d_ctl);
  cudaFree(ctx->d_state);
  cudaFree(ctx->d_scratch);
  cudaFree(ctx->d_counts);
  cudaFree(ctx->d_in);
  cudaFree(ctx->d_offsets);
  cudaFree(ctx->d_out0);
  cudaFree(ctx->d_out1);
  ctx->halo.release();
  if (ctx->h_ctl) cudaFreeHost(ctx->h_ctl);
  if (ctx->h_err_mirror) cudaFreeHost(ctx->h_err_mirror);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return VOX_OK;
}

void* vox_ctx_stream(vox_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

const char* vox_ctx_last_error(vox_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

static int sync_locked(vox_ctx* ctx) {
  VOX_CUDA(ctx, cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost,
                                ctx->stream),
           "cudaMemcpyAsync(ctl)");
  VOX_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  const unsigned err = ctx->h_ctl->err;
  if (err == 0) return VOX_OK;
  // Clear the error bits. After a timeout a launch may have left its queue words and its
  // barrier count mid-way: reset them too, and move to a fresh look-back epoch, so that no
  // state word the failed launch published can match a later launch's tag.
  ctx->h_ctl->err = 0;
  if (err & ERR_TIMEOUT) {
    ctx->h_ctl->next = 0;
    ctx->h_ctl->bar_count = 0;
    ctx->h_ctl->epoch += 1;
  }
  VOX_CUDA(ctx, cudaMemcpyAsync(ctx->d_ctl, ctx->h_ctl, sizeof(BatchCtl), cudaMemcpyHostToDevice,
                                ctx->stream),
           "cudaMemcpyAsync(ctl)");
  VOX_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (err & ERR_TIMEOUT) return fail(ctx, VOX_ERR_TIMEOUT, "a device-side wait gave up");
  if (err & ERR_BAD_INPUT)
    return fail(ctx, VOX_ERR_INVALID,
                "a slot index, or (staged halos) a chunk coordinate, was out of range");
  return fail(ctx, VOX_ERR_CAPACITY, "output capacity exceeded");
}

// sync_locked for a launch that mirrored its status into ctx->h_err_mirror: the stream
// sync alone, then the mirrored word (it holds the error bits of every launch so far); the
// copy path of sync_locked only when there is an error to clear or no mirrored value.
static int sync_mirrored(vox_ctx* ctx) {
  VOX_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  const unsigned m = *reinterpret_cast<volatile unsigned*>(ctx->h_err_mirror);
  *ctx->h_err_mirror = 0u;
  if (m == kMirrorValid) return VOX_OK;
  return sync_locked(ctx);
}

int vox_ctx_sync(vox_ctx* ctx) {
  vox::TraceRange trace_("vox_ctx_sync");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  return sync_locked(ctx);
}

int vox_generate(vox_ctx* ctx, const vox_chunk_coord* d_coords, int32_t n,
                 int64_t chunk_index_base, uint32_t* d_occ) {
  vox::TraceRange trace_("vox_generate");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n < 0 || (n > 0 && (!d_coords || !d_occ))) return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  if (n == 0) return VOX_OK;
  MeshArgs a = base_args(ctx);
  a.n = n;
  a.index_base = chunk_index_base;
  a.coords = d_coords;
  uint32_t* occ = d_occ;
  void* params[] = {&a, &occ};
  return launch(ctx, ctx->ks->generate[ctx->gm], n, ctx->ks->gen_threads,
                ctx->ks->smem_total(VOX_LAYOUT_VERTEX, ctx->ks->gen_threads, 0), params);
}

int vox_generate_slots(vox_ctx* ctx, const vox_chunk_coord* d_coords, int32_t n,
                       int64_t chunk_index_base, uint32_t* d_occ_pool, int32_t pool_slots,
                       const int32_t* d_slots) {
  vox::TraceRange trace_("vox_generate_slots");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n < 0 || (n > 0 && (!d_coords || !d_occ_pool || !d_slots)) || pool_slots < 1)
    return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  if (n == 0) return VOX_OK;
  MeshArgs a = base_args(ctx);
  a.n = n;
  a.index_base = chunk_index_base;
  a.coords = d_coords;
  a.slots = d_slots;
  a.pool_slots = pool_slots;
  uint32_t* occ = d_occ_pool;
  void* params[] = {&a, &occ};
  return launch(ctx, ctx->ks->generate[ctx->gm], n, ctx->ks->gen_threads,
                ctx->ks->smem_total(VOX_LAYOUT_VERTEX, ctx->ks->gen_threads, 0), params);
}

int vox_occ_to_cubes(vox_ctx* ctx, const uint32_t* d_occ, int32_t n, uint8_t* d_cubes) {
  vox::TraceRange trace_("vox_occ_to_cubes");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n < 0 || (n > 0 && (!d_occ || !d_cubes))) return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  VOX_CUDA(ctx, launch_occ_to_cubes(d_occ, n, ctx->cfg.chunk_size, d_cubes, ctx->stream),
           "occ_to_cubes");
  return VOX_OK;
}

int vox_cubes_to_occ(vox_ctx* ctx, const uint8_t* d_cubes, int32_t n, uint32_t* d_occ) {
  vox::TraceRange trace_("vox_cubes_to_occ");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n < 0 || (n > 0 && (!d_occ || !d_cubes))) return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  VOX_CUDA(ctx, launch_cubes_to_occ(d_cubes, n, ctx->cfg.chunk_size, d_occ, ctx->stream),
           "cubes_to_occ");
  return VOX_OK;
}

int vox_mesh(vox_ctx* ctx, const uint32_t* d_occ, const uint32_t* const d_nbr[6],
             vox_chunk_coord coord, void* d_out0, void* d_out1, uint64_t cap_faces,
             uint64_t* d_face_count) {
  vox::TraceRange trace_("vox_mesh");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!d_occ || !d_face_count) return fail(ctx, VOX_ERR_INVALID, "d_occ and d_face_count are required");
  int st = check_outputs(ctx, d_out0, d_out1, cap_faces);
  if (st != VOX_OK) return st;
  MeshArgs a = base_args(ctx);
  a.n = 1;
  a.occ_self = d_occ;
  for (int d = 0; d < 6; ++d) a.occ_nbr[d] = d_nbr ? d_nbr[d] : nullptr;
  a.coord_single = coord;
  a.out0 = d_out0;
  a.out1 = d_out1;
  a.cap = cap_faces;
  a.face_offsets = reinterpret_cast<unsigned long long*>(d_face_count);
  void* params[] = {&a};
  const int layout = ctx->cfg.layout;
  return launch(ctx, ctx->ks->single[layout][ctx->topt], 1, ctx->ks->threads[ctx->topt],
                ctx->ks->smem_total(layout, ctx->ks->threads[ctx->topt], ctx->stage_faces),
                params);
}

int vox_mesh_batch(vox_ctx* ctx, const uint32_t* d_occ_pool, int32_t pool_slots,
                   const int32_t* d_slots, const int32_t* d_nbr_slots,
                   const vox_chunk_coord* d_coords, int32_t n, void* d_out0, void* d_out1,
                   uint64_t cap_faces, uint64_t* d_face_offsets) {
  vox::TraceRange trace_("vox_mesh_batch");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n < 0 || (n > 0 && (!d_occ_pool || !d_slots || !d_coords || !d_face_offsets)) ||
      pool_slots < 1)
    return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  if (n == 0) return VOX_OK;
  int st = check_outputs(ctx, d_out0, d_out1, cap_faces);
  if (st != VOX_OK) return st;
  MeshArgs a = base_args(ctx);
  a.n = n;
  a.coords = d_coords;
  a.occ_pool = d_occ_pool;
  a.pool_slots = pool_slots;
  a.slots = d_slots;
  a.nbr_slots = d_nbr_slots;
  a.out0 = d_out0;
  a.out1 = d_out1;
  a.cap = cap_faces;
  a.face_offsets = reinterpret_cast<unsigned long long*>(d_face_offsets);
  return batch_launch(ctx, a, GM_OCC);
}

int vox_gen_mesh_batch(vox_ctx* ctx, const vox_chunk_coord* d_coords, const uint8_t* d_nbr_mask,
                       int32_t n, int64_t chunk_index_base, void* d_out0, void* d_out1,
                       uint64_t cap_faces, uint64_t* d_face_offsets) {
  vox::TraceRange trace_("vox_gen_mesh_batch");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n < 0 || (n > 0 && (!d_coords || !d_face_offsets)))
    return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  if (n == 0) return VOX_OK;
  int st = check_outputs(ctx, d_out0, d_out1, cap_faces);
  if (st != VOX_OK) return st;
  MeshArgs a = base_args(ctx);
  a.n = n;
  a.index_base = chunk_index_base;
  a.coords = d_coords;
  a.nbr_mask = d_nbr_mask;
  a.out0 = d_out0;
  a.out1 = d_out1;
  a.cap = cap_faces;
  a.face_offsets = reinterpret_cast<unsigned long long*>(d_face_offsets);
  return batch_launch(ctx, a, ctx->gm);
}

static int grow(vox_ctx* ctx, void** p, size_t* cap, size_t need, const char* what) {
  if (need <= *cap) return VOX_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  VOX_CUDA(ctx, cudaMalloc(p, need), what);
  *cap = need;
  return VOX_OK;
}

// Device address of page-locked host memory (cudaMallocHost / cudaHostRegister), or
// nullptr for pageable memory.
static void* mapped_host(const void* h) {
  if (!h) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int vox_gen_mesh_host(vox_ctx* ctx, const vox_chunk_coord* h_coords, const uint8_t* h_nbr_mask,
                      int32_t n, int64_t chunk_index_base, void* h_out0, void* h_out1,
                      uint64_t cap_faces, uint64_t* h_face_offsets) {
  vox::TraceRange trace_("vox_gen_mesh_host");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n < 0 || (n > 0 && (!h_coords || !h_face_offsets)))
    return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  if (cap_faces > 0 && (!h_out0 || (ctx->cfg.layout == VOX_LAYOUT_VERTEX && !h_out1)))
    return fail(ctx, VOX_ERR_INVALID, "output buffers are NULL with cap_faces > 0");
  if (n == 0) return VOX_OK;
  const int layout = ctx->cfg.layout;
  const size_t b0 = (size_t)bytes_out0(layout), b1 = (size_t)bytes_out1(layout);
  const size_t in_bytes = (size_t)n * sizeof(vox_chunk_coord) + (h_nbr_mask ? (size_t)n : 0);
  int st;
  // Page-locked outputs: the kernel writes the faces and the offsets straight into host
  // memory (over NVLink-C2C on Grace systems), staging each warp's faces in shared memory
  // so that every store is a full-line write; one launch, one sync.
  {
    void* z0 = cap_faces > 0 ? mapped_host(h_out0) : nullptr;
    void* z1 = cap_faces > 0 && b1 ? mapped_host(h_out1) : nullptr;
    void* zoff = mapped_host(h_face_offsets);
    const bool outs_ok = cap_faces == 0 || (z0 && aligned(z0, 16) && (b1 == 0 || (z1 && aligned(z1, 16))));
    if (zoff && aligned(zoff, 8) && outs_ok) {
      const void* zc = mapped_host(h_coords);
      const void* zm = h_nbr_mask ? mapped_host(h_nbr_mask) : nullptr;
      const vox_chunk_coord* d_coords = static_cast<const vox_chunk_coord*>(zc);
      const uint8_t* d_mask = static_cast<const uint8_t*>(zm);
      if (!zc || (h_nbr_mask && !zm)) {
        if ((st = grow(ctx, &ctx->d_in, &ctx->in_cap, in_bytes, "cudaMalloc(inputs)")) != VOX_OK)
          return st;
        vox_chunk_coord* dc = static_cast<vox_chunk_coord*>(ctx->d_in);
        uint8_t* dm = h_nbr_mask ? reinterpret_cast<uint8_t*>(dc + n) : nullptr;
        VOX_CUDA(ctx, cudaMemcpyAsync(dc, h_coords, (size_t)n * sizeof(vox_chunk_coord),
                                      cudaMemcpyHostToDevice, ctx->stream),
                 "H2D coords");
        if (h_nbr_mask)
          VOX_CUDA(ctx, cudaMemcpyAsync(dm, h_nbr_mask, (size_t)n, cudaMemcpyHostToDevice, ctx->stream),
                   "H2D mask");
        d_coords = dc;
        d_mask = dm;
      }
      MeshArgs a = base_args(ctx);
      a.n = n;
      a.index_base = chunk_index_base;
      a.coords = d_coords;
      a.nbr_mask = d_mask;
      a.out0 = z0;
      a.out1 = z1;
      a.cap = cap_faces;
      a.face_offsets = static_cast<unsigned long long*>(zoff);
      // the kernel flags a capacity overflow in the error word; the look-back and overlap
      // kernels also mirror that word into page-locked memory at their end
      const bool mirror = ctx->schedule != VOX_SCHEDULE_PHASED;
      if (mirror) {
        *ctx->h_err_mirror = 0u;
        a.err_mirror = ctx->d_err_mirror;
      }
      if ((st = batch_launch(ctx, a, ctx->gm, true)) != VOX_OK) return st;
      return mirror ? sync_mirrored(ctx) : sync_locked(ctx);
    }
  }
  if ((st = grow(ctx, &ctx->d_in, &ctx->in_cap, in_bytes, "cudaMalloc(inputs)")) != VOX_OK) return st;
  size_t off_cap = ctx->offsets_cap * sizeof(unsigned long long);
  void* offp = ctx->d_offsets;
  if ((st = grow(ctx, &offp, &off_cap, ((size_t)n + 1) * sizeof(unsigned long long),
                 "cudaMalloc(offsets)")) != VOX_OK)
    return st;
  ctx->d_offsets = static_cast<unsigned long long*>(offp);
  ctx->offsets_cap = off_cap / sizeof(unsigned long long);
  if (cap_faces > ctx->out_cap_faces) {
    cudaFree(ctx->d_out0);
    cudaFree(ctx->d_out1);
    ctx->d_out0 = ctx->d_out1 = nullptr;
    ctx->out_cap_faces = 0;
    VOX_CUDA(ctx, cudaMalloc(&ctx->d_out0, cap_faces * b0), "cudaMalloc(out0)");
    if (b1) VOX_CUDA(ctx, cudaMalloc(&ctx->d_out1, cap_faces * b1), "cudaMalloc(out1)");
    ctx->out_cap_faces = cap_faces;
  }
  vox_chunk_coord* d_coords = static_cast<vox_chunk_coord*>(ctx->d_in);
  uint8_t* d_mask = h_nbr_mask ? reinterpret_cast<uint8_t*>(d_coords + n) : nullptr;
  VOX_CUDA(ctx, cudaMemcpyAsync(d_coords, h_coords, (size_t)n * sizeof(vox_chunk_coord),
                                cudaMemcpyHostToDevice, ctx->stream),
           "H2D coords");
  if (h_nbr_mask)
    VOX_CUDA(ctx, cudaMemcpyAsync(d_mask, h_nbr_mask, (size_t)n, cudaMemcpyHostToDevice, ctx->stream),
             "H2D mask");
  MeshArgs a = base_args(ctx);
  a.n = n;
  a.index_base = chunk_index_base;
  a.coords = d_coords;
  a.nbr_mask = d_mask;
  a.out0 = ctx->d_out0;
  a.out1 = ctx->d_out1;
  a.cap = cap_faces;
  a.face_offsets = ctx->d_offsets;
  if ((st = batch_launch(ctx, a, ctx->gm)) != VOX_OK) return st;
  VOX_CUDA(ctx, cudaMemcpyAsync(h_face_offsets, ctx->d_offsets, ((size_t)n + 1) * sizeof(uint64_t),
                                cudaMemcpyDeviceToHost, ctx->stream),
           "D2H offsets");
  VOX_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  const uint64_t total = h_face_offsets[n];
  const uint64_t w = std::min<uint64_t>(total, cap_faces);
  if (w > 0) {
    VOX_CUDA(ctx, cudaMemcpyAsync(h_out0, ctx->d_out0, w * b0, cudaMemcpyDeviceToHost, ctx->stream),
             "D2H out0");
    if (b1)
      VOX_CUDA(ctx, cudaMemcpyAsync(h_out1, ctx->d_out1, w * b1, cudaMemcpyDeviceToHost, ctx->stream),
               "D2H out1");
  }
  st = sync_locked(ctx);
  if (st == VOX_OK && total > cap_faces)
    st = fail(ctx, VOX_ERR_CAPACITY, "output capacity exceeded: %llu faces needed",
              (unsigned long long)total);
  return st;
}

int vox_frustum_planes(const float m[16], float planes[24]) {
  if (!m || !planes) return VOX_ERR_INVALID;
  // data[col][row] of the column-major matrix (src/frustum_culling.rs:54-83).
  auto D = [&](int c, int r) { return m[c * 4 + r]; };
  float p[6][4];
  for (int c = 0; c < 4; ++c) {
    p[2][c] = D(c, 3) + D(c, 0);  // left
    p[3][c] = D(c, 3) - D(c, 0);  // right
    p[4][c] = D(c, 3) - D(c, 1);  // top
    p[5][c] = D(c, 3) + D(c, 1);  // bottom
    p[0][c] = D(c, 3) + D(c, 2);  // near
    p[1][c] = D(c, 3) - D(c, 2);  // far
  }
  for (int k = 0; k < 6; ++k)
    for (int c = 0; c < 4; ++c) planes[4 * k + c] = p[k][c];
  return VOX_OK;
}

int vox_frustum_cull(vox_ctx* ctx, const float planes[24], const vox_chunk_coord* d_coords,
                     int32_t n, uint8_t* d_visible) {
  vox::TraceRange trace_("vox_frustum_cull");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!planes || n < 0 || (n > 0 && (!d_coords || !d_visible)))
    return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  Planes pl;
  std::memcpy(pl.p, planes, sizeof pl.p);
  VOX_CUDA(ctx, launch_frustum(pl, d_coords, n, ctx->cfg.chunk_size, d_visible, ctx->stream),
           "frustum");
  return VOX_OK;
}

int vox_draw_list(vox_ctx* ctx, const float planes[24], const vox_chunk_coord* d_coords,
                  const uint64_t* d_face_offsets, int32_t n, vox_draw_indexed_indirect* d_draws,
                  uint32_t* d_count) {
  vox::TraceRange trace_("vox_draw_list");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!planes || !d_count || n < 0 || (n > 0 && (!d_coords || !d_face_offsets || !d_draws)))
    return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  Planes pl;
  std::memcpy(pl.p, planes, sizeof pl.p);
  VOX_CUDA(ctx, launch_draw_list(pl, d_coords, reinterpret_cast<const unsigned long long*>(d_face_offsets),
                                 n, ctx->cfg.chunk_size, ctx->cfg.layout == VOX_LAYOUT_INSTANCED ? 1 : 0,
                                 d_draws, d_count, &ctx->d_ctl->err, ctx->stream),
           "draw list");
  return VOX_OK;
}

int vox_raster(vox_ctx* ctx, const float view_proj_colmajor[16], const void* d_vertices,
               const void* d_indices, uint64_t faces, int32_t width, int32_t height,
               uint64_t* d_depth_keys, uint8_t* d_rgba) {
  vox::TraceRange trace_("vox_raster");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (ctx->cfg.layout != VOX_LAYOUT_VERTEX)
    return fail(ctx, VOX_ERR_INVALID, "the rasteriser takes the vertex layout");
  if (!view_proj_colmajor || width <= 0 || height <= 0 || width > 16384 || height > 16384 ||
      !d_depth_keys || !d_rgba || faces >= (1ull << 31) || (faces > 0 && (!d_vertices || !d_indices)))
    return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  RasterArgs a;
  a.vertices = d_vertices;
  a.indices = d_indices;
  a.faces = faces;
  a.width = width;
  a.height = height;
  std::memcpy(a.m, view_proj_colmajor, sizeof a.m);
  std::memcpy(a.tex, ctx->cfg.texture_index, sizeof a.tex);
  VOX_CUDA(ctx, launch_raster(a, reinterpret_cast<unsigned long long*>(d_depth_keys), d_rgba,
                              ctx->stream),
           "raster");
  return VOX_OK;
}

int vox_ctx_get_tuning(vox_ctx* ctx, vox_tuning* out) {
  if (!ctx || !out) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  out->threads = ctx->ks->threads[ctx->topt];
  out->stage_faces = ctx->stage_faces;
  out->ctas_per_sm = ctx->ctas_per_sm;
  out->schedule = ctx->schedule;
  out->slab_chunks = ctx->slab_chunks;
  out->halo_staging = ctx->halo_staging;
  return VOX_OK;
}

int vox_ctx_set_tuning(vox_ctx* ctx, const vox_tuning* t) {
  if (!ctx || !t) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  int topt = -1;
  for (int k = 0; k < 2; ++k)
    if (ctx->ks->threads[k] == t->threads) topt = k;
  if (topt < 0) return fail(ctx, VOX_ERR_INVALID, "threads must be %d or %d", ctx->ks->threads[0],
                            ctx->ks->threads[1]);
  return apply_tuning(ctx, topt, t->stage_faces, t->ctas_per_sm, t->schedule, t->slab_chunks,
                      t->halo_staging);
}

int vox_autotune(vox_ctx* ctx, const vox_chunk_coord* d_coords, const uint8_t* d_nbr_mask,
                 int32_t n, int64_t chunk_index_base, void* d_out0, void* d_out1,
                 uint64_t cap_faces, uint64_t* d_face_offsets, int32_t iters, vox_tuning* out) {
  vox::TraceRange trace_("vox_autotune");
  if (!ctx) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n <= 0 || !d_coords || !d_face_offsets || iters < 1)
    return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  int st = check_outputs(ctx, d_out0, d_out1, cap_faces);
  if (st != VOX_OK) return st;
  const int stages[] = {0, kStageSingle, kStageDouble};
  const int ctas[] = {0, 4, 2};
  cudaEvent_t e0, e1;
  VOX_CUDA(ctx, cudaEventCreate(&e0), "cudaEventCreate");
  VOX_CUDA(ctx, cudaEventCreate(&e1), "cudaEventCreate");
  const int keep_t = ctx->topt, keep_s = ctx->stage_faces, keep_c = ctx->ctas_per_sm,
            keep_p = ctx->schedule, keep_l = ctx->slab_chunks, keep_h = ctx->halo_staging;
  float best_ms = 1e30f;
  int best_t = keep_t, best_s = keep_s, best_c = keep_c, best_p = keep_p, best_l = 0, best_h = 0;
  auto run = [&]() {
    MeshArgs a = base_args(ctx);
    a.n = n;
    a.index_base = chunk_index_base;
    a.coords = d_coords;
    a.nbr_mask = d_nbr_mask;
    a.out0 = d_out0;
    a.out1 = d_out1;
    a.cap = cap_faces;
    a.face_offsets = reinterpret_cast<unsigned long long*>(d_face_offsets);
    return batch_launch(ctx, a, ctx->gm);
  };
  auto time_candidate = [&](int p, int t, int s, int c, int l, int h) -> bool {  // false: stop
    if ((st = run()) != VOX_OK) return false;
    cudaEventRecord(e0, ctx->stream);
    for (int k = 0; k < iters && st == VOX_OK; ++k) st = run();
    cudaEventRecord(e1, ctx->stream);
    if (st != VOX_OK) return false;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      st = cuda_fail(ctx, cudaGetLastError(), "autotune");
      return false;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best_t = t;
      best_s = s;
      best_c = c;
      best_p = p;
      best_l = l;
      best_h = h;
    }
    return true;
  };
  // 1. the launch shape, every chunk of the batch in one launch
  bool go = true;
  for (int p = 0; p < 3 && go; ++p)
    for (int t = 0; t < 2 && go; ++t)
      for (int s : stages) {
        int full_grid = 0;
        for (int c : ctas) {
          if (apply_tuning(ctx, t, s, c, p, 0, 0) != VOX_OK) continue;
          const int g = p == VOX_SCHEDULE_PHASED    ? ctx->phased_grid[ctx->gm]
                        : p == VOX_SCHEDULE_OVERLAP ? ctx->overlap_grid[ctx->gm]
                                                    : ctx->batch_grid[ctx->gm];
          if (c == 0) full_grid = g;
          else if (g >= full_grid) continue;  // same grid as c = 0
          if (!(go = time_candidate(p, t, s, c, 0, 0))) break;
        }
        if (!go) break;
      }
  // 2. the output slab (chunks per launch) for the best shape: halves, quarters and eighths
  // of the batch, while a launch still holds at least two waves of the persistent grid
  // (a smaller slab keeps a launch's spilled chunk state and its output run L2-sized)
  if (go && apply_tuning(ctx, best_t, best_s, best_c, best_p, 0, 0) == VOX_OK) {
    const int g = best_p == VOX_SCHEDULE_PHASED    ? ctx->phased_grid[ctx->gm]
                  : best_p == VOX_SCHEDULE_OVERLAP ? ctx->overlap_grid[ctx->gm]
                                                   : ctx->batch_grid[ctx->gm];
    for (int div = 2; div <= 8 && go; div *= 2) {
      const int l = (n + div - 1) / div;
      if (l < 2 * g) break;
      if (apply_tuning(ctx, best_t, best_s, best_c, best_p, l, 0) != VOX_OK) continue;
      go = time_candidate(best_p, best_t, best_s, best_c, l, 0);
    }
  }
  // 3. halo staging for the best shape and slab: the halos regenerated in the fused launch
  // (every candidate above), or every chunk generated once into a pool with the halo planes
  // read from the neighbours' occupancy
  if (go && apply_tuning(ctx, best_t, best_s, best_c, best_p, best_l, 1) == VOX_OK)
    go = time_candidate(best_p, best_t, best_s, best_c, best_l, 1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->last_error.clear();
  const int st2 = apply_tuning(ctx, best_t, best_s, best_c, best_p, best_l, best_h);
  if (st == VOX_OK) st = st2;
  if (st == VOX_OK) st = sync_locked(ctx);
  if (st != VOX_OK) apply_tuning(ctx, keep_t, keep_s, keep_c, keep_p, keep_l, keep_h);
  if (out) {
    out->threads = ctx->ks->threads[ctx->topt];
    out->stage_faces = ctx->stage_faces;
    out->ctas_per_sm = ctx->ctas_per_sm;
    out->schedule = ctx->schedule;
    out->slab_chunks = ctx->slab_chunks;
    out->halo_staging = ctx->halo_staging;
  }
  return st;
}

int vox_selftest_lookback_timeout(vox_ctx* ctx, int32_t spin_limit) {
  if (!ctx || spin_limit < 1) return VOX_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  unsigned long long* words = nullptr;
  VOX_CUDA(ctx, cudaMalloc(&words, 2 * sizeof(unsigned long long)), "cudaMalloc(probe)");
  cudaError_t e = cudaMemsetAsync(words, 0, 2 * sizeof(unsigned long long), ctx->stream);
  if (e == cudaSuccess) e = launch_lookback_probe(words, ctx->d_ctl, spin_limit, ctx->stream);
  const int st = e == cudaSuccess ? sync_locked(ctx) : cuda_fail(ctx, e, "lookback probe");
  cudaFree(words);
  return st;
}

static void graph_free(vox_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  cudaFree(g->d_state);
  cudaFree(g->d_scratch);
  cudaFree(g->d_counts);
  g->halo.release();
  delete g;
}

int vox_graph_capture(vox_ctx* ctx, const vox_chunk_coord* d_coords, const uint8_t* d_nbr_mask,
                      int32_t n, int64_t chunk_index_base, void* d_out0, void* d_out1,
                      uint64_t cap_faces, uint64_t* d_face_offsets, vox_graph** out) {
  vox::TraceRange trace_("vox_graph_capture");
  if (!ctx || !out) return VOX_ERR_INVALID;
  *out = nullptr;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n <= 0 || !d_coords || !d_face_offsets) return fail(ctx, VOX_ERR_INVALID, "bad arguments");
  int st = check_outputs(ctx, d_out0, d_out1, cap_faces);
  if (st != VOX_OK) return st;
  vox_graph* g = new (std::nothrow) vox_graph();
  if (!g) return VOX_ERR_OOM;
  g->ctx = ctx;
  g->schedule = ctx->schedule;
  auto bail = [&](int s) {
    graph_free(g);
    return s;
  };
  cudaError_t e;
  MeshArgs a = base_args(ctx);
  a.n = n;
  a.index_base = chunk_index_base;
  a.coords = d_coords;
  a.nbr_mask = d_nbr_mask;
  a.out0 = d_out0;
  a.out1 = d_out1;
  a.cap = cap_faces;
  a.face_offsets = reinterpret_cast<unsigned long long*>(d_face_offsets);
  const int slab = slab_of(ctx, n);
  g->launches = (n + slab - 1) / slab;
  if (g->schedule != VOX_SCHEDULE_LOOKBACK) {
    if ((e = cudaMalloc(&g->d_scratch, (size_t)slab * (size_t)ctx->ks->spill_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&g->d_counts, (size_t)slab * sizeof(uint32_t))) != cudaSuccess)
      return bail(cuda_fail(ctx, e, "cudaMalloc(graph scratch)"));
    a.scratch = g->d_scratch;
    a.counts = g->d_counts;
  }
  if (g->schedule != VOX_SCHEDULE_PHASED) {
    g->state_bytes = (size_t)slab * sizeof(unsigned long long);
    if ((e = cudaMalloc(&g->d_state, g->state_bytes)) != cudaSuccess ||
        (e = cudaMemsetAsync(g->d_state, 0, g->state_bytes, ctx->stream)) != cudaSuccess)
      return bail(cuda_fail(ctx, e, "cudaMalloc(graph state)"));
    g->wiped_at = ctx->launches;
    a.state = g->d_state;
  }
  // the graph owns its staged-halo buffers too (allocated before the capture)
  if (ctx->halo_staging && (st = ensure_halo(ctx, g->halo, (size_t)n)) != VOX_OK) return bail(st);
  // Capture on a private stream (thread-local mode: other threads' CUDA calls are not
  // affected), then replay on the context's stream.
  cudaStream_t cs = nullptr;
  if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(cuda_fail(ctx, e, "cudaStreamCreate(capture)"));
  if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
    cudaStreamDestroy(cs);
    return bail(cuda_fail(ctx, e, "cudaStreamBeginCapture"));
  }
  int gm = ctx->gm;
  if (ctx->halo_staging && (st = halo_prepass(ctx, a, gm, g->halo, cs)) == VOX_OK) gm = GM_OCC;
  if (st == VOX_OK)
    st = for_each_slab(a, slab, [&](MeshArgs& b) { return issue_batch(ctx, b, gm, false, cs); });
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(cs, &graph);
  cudaStreamDestroy(cs);
  g->graph = graph;
  if (st != VOX_OK) return bail(st);
  if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaStreamEndCapture"));
  if ((e = cudaGraphInstantiate(&g->exec, g->graph, 0)) != cudaSuccess)
    return bail(cuda_fail(ctx, e, "cudaGraphInstantiate"));
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
    return bail(cuda_fail(ctx, e, "cudaStreamSynchronize"));
  *out = g;
  return VOX_OK;
}

int vox_graph_launch(vox_graph* g) {
  vox::TraceRange trace_("vox_graph_launch");
  if (!g || !g->ctx) return VOX_ERR_INVALID;
  vox_ctx* ctx = g->ctx;
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->launches += (unsigned long long)g->launches;
  // look-back states carry a 24-bit launch epoch: zero them before a tag can repeat
  if (g->d_state && ctx->launches - g->wiped_at >= kStateWipePeriod) {
    VOX_CUDA(ctx, cudaMemsetAsync(g->d_state, 0, g->state_bytes, ctx->stream), "cudaMemsetAsync(state)");
    g->wiped_at = ctx->launches;
  }
  VOX_CUDA(ctx, cudaGraphLaunch(g->exec, ctx->stream), "cudaGraphLaunch");
  return VOX_OK;
}

int vox_graph_destroy(vox_graph* g) {
  if (!g) return VOX_OK;
  if (g->ctx && g->ctx->stream) cudaStreamSynchronize(g->ctx->stream);
  graph_free(g);
  return VOX_OK;
}

int vox_host_alloc(size_t bytes, void** out) {
  if (!out) return VOX_ERR_INVALID;
  *out = nullptr;
  if (bytes == 0) return VOX_OK;
  cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return VOX_ERR_OOM;
  }
  return VOX_OK;
}

int vox_host_free(void* p) {
  if (p) cudaFreeHost(p);
  return VOX_OK;
}

}  // extern "C"
