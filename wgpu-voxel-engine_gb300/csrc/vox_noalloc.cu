// vox_noalloc.cu — vox_gen_mesh_batch_noalloc: fused generation + meshing that allocates
// no memory.
//
// Some callers cannot call cudaMalloc: hosts that own every byte of device memory through
// their own pool (an engine's allocator, a framework that budgets memory per plugin) or
// code paths where an allocation is not allowed to happen. This entry point serves them.
// The caller passes the inputs and the outputs; the kernel's scratch (the work-queue
// ticket, the look-back epoch and error word, and the look-back states) lives in the
// file-scope array g_noalloc_scratch below, and the per-config tables travel as a kernel
// parameter. The array is part of the library image: every GPU that loads the library
// holds it (about 129 KiB) until the process exits.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it for the life of the
// process; do not use this entry point across cudaDeviceReset, which reloads the module and
// leaves the cached address stale. Every call is synchronous (it reads the launch's status
// back and waits for the stream), so no call may be made on a stream that is being
// captured: such a call returns VOX_ERR_INVALID before it touches the GPU. Every call
// shares the array and it keeps the last call's contents: each call clears the queue
// ticket and the error word before its launch, and calls whose work overlaps on the GPU
// race on the shared array.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "voxgpu.h"
#include "vox_device.cuh"
#include "vox_tables.h"
#include "vox_types.h"

namespace vox {
namespace {

constexpr int kNoAllocMaxChunks = 16384;  // chunks per call

struct NoAllocScratch {
  BatchCtl ctl;                                // queue ticket, epoch, error bits
  unsigned char pad[256 - sizeof(BatchCtl)];   // keeps the states on a 256-byte boundary
  unsigned long long state[kNoAllocMaxChunks]; // look-back states
};
static_assert(sizeof(BatchCtl) <= 256 && offsetof(NoAllocScratch, state) == 256,
              "look-back states start 256 bytes into the scratch");

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// The persistent fused kernel of vox_gen_mesh_batch with its scratch taken from
// g_noalloc_scratch (addresses in a.ctl / a.state) and its tables from the parameter
// space. Direct global stores (no staging window).
template <int N, int GM, int LAYOUT, int T>
__global__ void __launch_bounds__(T)
k_mesh_batch_noalloc(const __grid_constant__ MeshArgs a, const __grid_constant__ TablesDev tab) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChunkSmem<N, LAYOUT> s;
  s.carve(smem_raw);
  load_tables<N, LAYOUT>(s, &tab);
  __shared__ int s_item;
  __shared__ unsigned long long s_base;
  __shared__ unsigned s_epoch;
  if (threadIdx.x == 0) {
    s_epoch = ld_relaxed_u32(&a.ctl->epoch);
    __threadfence();
  }
  __syncthreads();
  const unsigned epoch = s_epoch;
  while (true) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(&a.ctl->next, 1u);
    __syncthreads();
    const int i = s_item;
    if (i >= a.n) {
      if (threadIdx.x == 0 && i == a.n + (int)gridDim.x - 1) {
        a.ctl->next = 0u;
        a.ctl->epoch = epoch + 1u;
      }
      break;
    }
    const vox_chunk_coord c = a.coords[i];
    unsigned m = a.nbr_mask ? a.nbr_mask[i] : 0u;
    if (GM == GM_BERNOULLI) m = 0u;
    if (!a.full6) m &= 0xFu;
    gen_chunk<N, GM, LAYOUT, T>(s, a.gen, c, a.index_base + i, m, true);
    const uint32_t total = count_and_scan<N, LAYOUT, T>(s);
    if (threadIdx.x < 32) {
      const unsigned long long excl = lookback(a.state, a.ctl, epoch, i, total, a.spin_limit);
      if (threadIdx.x == 0) {
        s_base = excl;
        a.face_offsets[i] = excl;
        if (i == a.n - 1) {
          a.face_offsets[a.n] = excl + total;
          if (excl + total > a.cap) atomicOr(&a.ctl->err, ERR_CAPACITY);
        }
      }
    }
    __syncthreads();
    emit_chunk_direct<N, LAYOUT>(s, c, s_base, a.cap, a.out0, a.out1, 0, emit_elems(s));
    __syncthreads();
  }
}

template <int N>
constexpr int noalloc_threads() {
  return N <= 16 ? Shape<N>::T1 : Shape<N>::T0;
}

template <int N>
const void* noalloc_kernel(int gm, int layout) {
  constexpr int T = noalloc_threads<N>();
  if (layout == VOX_LAYOUT_INSTANCED) {
    if (gm == GM_HEIGHT) return (const void*)k_mesh_batch_noalloc<N, GM_HEIGHT, 1, T>;
    if (gm == GM_DENSITY) return (const void*)k_mesh_batch_noalloc<N, GM_DENSITY, 1, T>;
    return (const void*)k_mesh_batch_noalloc<N, GM_BERNOULLI, 1, T>;
  }
  if (gm == GM_HEIGHT) return (const void*)k_mesh_batch_noalloc<N, GM_HEIGHT, 0, T>;
  if (gm == GM_DENSITY) return (const void*)k_mesh_batch_noalloc<N, GM_DENSITY, 0, T>;
  return (const void*)k_mesh_batch_noalloc<N, GM_BERNOULLI, 0, T>;
}

template <int N>
int noalloc_smem(int layout) {
  return layout == VOX_LAYOUT_INSTANCED
             ? SmemPlan<N, VOX_LAYOUT_INSTANCED>::total(noalloc_threads<N>(), 0)
             : SmemPlan<N, VOX_LAYOUT_VERTEX>::total(noalloc_threads<N>(), 0);
}

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
NoAllocScratch* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_launches[kMaxDevices] = {};

int noalloc_fail(int status, const char* msg) {
  std::fprintf(stderr, "voxgpu: vox_gen_mesh_batch_noalloc: %s\n", msg);
  return status;
}

}  // namespace
}  // namespace vox

using namespace vox;

extern "C" int vox_gen_mesh_batch_noalloc(const vox_config* cfg, void* stream,
                                          const vox_chunk_coord* d_coords,
                                          const uint8_t* d_nbr_mask, int32_t n,
                                          int64_t chunk_index_base, void* d_out0, void* d_out1,
                                          uint64_t cap_faces, uint64_t* d_face_offsets) {
  if (!cfg) return noalloc_fail(VOX_ERR_INVALID, "config is NULL");
  vox_sizes sz;
  if (vox_query_sizes(cfg, &sz) != VOX_OK) return noalloc_fail(VOX_ERR_INVALID, "invalid config");
  if (n < 0) return noalloc_fail(VOX_ERR_INVALID, "n is negative");
  if (n > kNoAllocMaxChunks)
    return noalloc_fail(VOX_ERR_INVALID, "n exceeds the 16384-chunk maximum of this entry point");
  if (n == 0) return VOX_OK;
  if (!d_coords || !d_face_offsets) return noalloc_fail(VOX_ERR_INVALID, "missing input/offsets");
  const int layout = cfg->layout;
  if (cap_faces > 0) {
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(d_out0), a1 = reinterpret_cast<uintptr_t>(d_out1);
    if (!d_out0 || (a0 & 15u) || (layout == VOX_LAYOUT_VERTEX && (!d_out1 || (a1 & 15u))))
      return noalloc_fail(VOX_ERR_INVALID, "outputs must be non-NULL and 16-byte aligned");
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return noalloc_fail(VOX_ERR_NO_DEVICE, "no current CUDA device");
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // The call reads its status back and synchronises the stream, which a stream capture
  // does not allow: refuse a capturing stream before any work is queued on it.
  cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap_status) != cudaSuccess) {
    cudaGetLastError();
    return noalloc_fail(VOX_ERR_CUDA, "cudaStreamIsCapturing failed");
  }
  if (cap_status != cudaStreamCaptureStatusNone)
    return noalloc_fail(VOX_ERR_INVALID, "the call is synchronous and cannot run on a capturing stream");
  const int N = cfg->chunk_size;
  const int gm = cfg->gen.kind == VOX_GEN_HEIGHTMAP ? GM_HEIGHT
               : cfg->gen.kind == VOX_GEN_DENSITY   ? GM_DENSITY
                                                    : GM_BERNOULLI;
  const void* fn = nullptr;
  int threads = 0, smem = 0;
  switch (N) {
    case 8: fn = noalloc_kernel<8>(gm, layout); threads = noalloc_threads<8>(); smem = noalloc_smem<8>(layout); break;
    case 16: fn = noalloc_kernel<16>(gm, layout); threads = noalloc_threads<16>(); smem = noalloc_smem<16>(layout); break;
    case 32: fn = noalloc_kernel<32>(gm, layout); threads = noalloc_threads<32>(); smem = noalloc_smem<32>(layout); break;
    default: fn = noalloc_kernel<64>(gm, layout); threads = noalloc_threads<64>(); smem = noalloc_smem<64>(layout); break;
  }
  NoAllocScratch* scratch = nullptr;
  int per_sm = 0, sms = 0;
  {
    // Once per device: the scratch array's device address (with this device current).
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        std::fprintf(stderr, "voxgpu: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
        return VOX_ERR_CUDA;
      }
      g_scratch_ptr[dev] = static_cast<NoAllocScratch*>(p);
    }
    scratch = g_scratch_ptr[dev];
    // Look-back states carry a 24-bit launch epoch, which every launch advances by one (its
    // last work ticket is always drawn); wipe them every 2^22 calls, well before a tag can
    // repeat.
    if (g_launches[dev] > 0 && (g_launches[dev] & ((1ull << 22) - 1)) == 0 &&
        cudaMemsetAsync(scratch->state, 0, sizeof(scratch->state), st) != cudaSuccess)
      return noalloc_fail(VOX_ERR_CUDA, "cudaMemsetAsync(state) failed");
    ++g_launches[dev];
  }
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    return noalloc_fail(VOX_ERR_CUDA, "kernel set-up failed");
  }
  // The queue ticket and the error word must start at zero.
  if (cudaMemsetAsync(&scratch->ctl.next, 0, sizeof(unsigned), st) != cudaSuccess ||
      cudaMemsetAsync(&scratch->ctl.err, 0, sizeof(unsigned), st) != cudaSuccess)
    return noalloc_fail(VOX_ERR_CUDA, "cudaMemsetAsync(ctl) failed");
  TablesDev tab;
  build_tables(*cfg, tab);
  MeshArgs a;
  std::memset(&a, 0, sizeof a);
  a.n = n;
  a.index_base = chunk_index_base;
  a.coords = d_coords;
  a.nbr_mask = d_nbr_mask;
  a.out0 = d_out0;
  a.out1 = d_out1;
  a.cap = cap_faces;
  a.face_offsets = reinterpret_cast<unsigned long long*>(d_face_offsets);
  a.state = scratch->state;
  a.ctl = &scratch->ctl;
  a.gen.kind = cfg->gen.kind;
  a.gen.octaves = cfg->gen.octaves;
  a.gen.seed = cfg->gen.seed;
  a.gen.freq = cfg->gen.frequency;
  a.gen.lac = cfg->gen.lacunarity;
  a.gen.gain = cfg->gen.gain;
  a.gen.amp = cfg->gen.amplitude;
  a.gen.base = cfg->gen.base_height;
  a.gen.y_ref = cfg->gen.y_ref;
  a.gen.y_scale = cfg->gen.y_scale;
  a.gen.solid_below_zero = cfg->gen.solid_below_zero;
  a.full6 = cfg->cull_mode == VOX_CULL_FULL6 ? 1 : 0;
  a.stage_faces = 0;
  a.spin_limit = kSpinLimit;
  const int grid = n < per_sm * sms ? n : per_sm * sms;
  void* params[] = {&a, &tab};
  if (cudaLaunchKernel(fn, dim3(grid), dim3(threads), params, (size_t)smem, st) != cudaSuccess) {
    const cudaError_t e = cudaGetLastError();
    std::fprintf(stderr, "voxgpu: launch failed: %s\n", cudaGetErrorString(e));
    return VOX_ERR_CUDA;
  }
  BatchCtl ctl;
  if (cudaMemcpyAsync(&ctl, &scratch->ctl, sizeof ctl, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    const cudaError_t e = cudaGetLastError();
    std::fprintf(stderr, "voxgpu: %s\n", cudaGetErrorString(e));
    return VOX_ERR_CUDA;
  }
  const unsigned err = ctl.err;
  // A timed-out wait does not stop the kernel from drawing every ticket, so its last
  // ticket has already reset the queue and advanced the epoch: no state word of the
  // failed launch can match a later launch's tag.
  if (err & ERR_TIMEOUT) return VOX_ERR_TIMEOUT;
  if (err & ERR_CAPACITY) return VOX_ERR_CAPACITY;
  return VOX_OK;
}
