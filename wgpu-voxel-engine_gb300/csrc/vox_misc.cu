// vox_misc.cu — small kernels around the hot path: the chunk-frustum test, the indirect
// draw list of the visible meshes, and the conversions between occupancy bitmasks and the
// reference's one-byte-per-voxel cubes.
#include <cstdint>

#include "voxgpu.h"
#include "vox_kernels.h"
#include "vox_types.h"

namespace vox {

namespace {

constexpr uint8_t kGrass = 0;  // CubeType::GRASS (src/cube.rs:17-21)
constexpr uint8_t kAir = 2;    // CubeType::AIR

// One thread per voxel: cubes[x + N*z + N*N*y] from bit x of row (y, z).
__global__ void k_occ_to_cubes(const uint32_t* __restrict__ occ, long long total, int n_size,
                               uint8_t* __restrict__ cubes) {
  const int W = n_size > 32 ? n_size / 32 : 1;
  const long long per = (long long)n_size * n_size * n_size;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < total;
       v += (long long)gridDim.x * blockDim.x) {
    const long long c = v / per;
    const int i = (int)(v - c * per);
    const int x = i % n_size, z = (i / n_size) % n_size, y = i / (n_size * n_size);
    const uint32_t w = occ[c * (long long)n_size * n_size * W + (long long)(y * n_size + z) * W + (x >> 5)];
    cubes[v] = ((w >> (x & 31)) & 1u) ? kGrass : kAir;
  }
}

// One thread per occupancy word: a voxel is solid iff its byte is not AIR (chunk.rs:71).
__global__ void k_cubes_to_occ(const uint8_t* __restrict__ cubes, long long words, int n_size,
                               uint32_t* __restrict__ occ) {
  const int W = n_size > 32 ? n_size / 32 : 1;
  const int bits = n_size < 32 ? n_size : 32;
  const long long per_words = (long long)n_size * n_size * W;
  const long long per = (long long)n_size * n_size * n_size;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < words;
       q += (long long)gridDim.x * blockDim.x) {
    const long long c = q / per_words;
    const int k = (int)(q - c * per_words);
    const int row = k / W, w = k % W;
    const int y = row / n_size, z = row % n_size;
    const uint8_t* src = cubes + c * per + (long long)n_size * z + (long long)n_size * n_size * y + w * 32;
    uint32_t v = 0;
    for (int b = 0; b < bits; ++b) v |= (src[b] != kAir ? 1u : 0u) << b;
    occ[q] = v;
  }
}

// Frustum::contains (src/frustum_culling.rs:16-40) per chunk: corners in the reference's
// order, planes near, far, left, right, top, bottom; dist = ((a*x + b*y) + c*z) + d with
// one rounding per operation (the file is built with -fmad=false).
__device__ __forceinline__ bool frustum_contains(const Planes& pl, vox_chunk_coord c, int extent) {
  const float px = (float)(c.x * extent), py = (float)(c.y * extent), pz = (float)(c.z * extent);
  const float e = (float)extent;
  bool inside_any = false;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float x = (k & 1) ? px + e : px;
    const float z = (k & 2) ? pz + e : pz;
    const float y = (k & 4) ? py + e : py;
    bool inside = true;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const float d = pl.p[4 * j] * x + pl.p[4 * j + 1] * y + pl.p[4 * j + 2] * z + pl.p[4 * j + 3];
      inside = inside && !(d < 0.0f);
    }
    inside_any = inside_any || inside;
  }
  return inside_any;
}

__global__ void k_frustum(Planes pl, const vox_chunk_coord* __restrict__ coords, int n, int extent,
                          uint8_t* __restrict__ visible) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  visible[i] = frustum_contains(pl, coords[i], extent) ? 1 : 0;
}

// World::render (src/world.rs:24-40) as an indirect draw list: one CTA walks the chunks
// in tiles of 1024, tests each (Frustum::contains), and compacts the visible chunks that
// have faces in chunk order (warp ballots, then a scan of the 32 warp totals). Records
// whose counts or offsets do not fit the 32-bit fields latch ERR_CAPACITY and are zeroed.
__global__ void __launch_bounds__(1024)
k_draw_list(Planes pl, const vox_chunk_coord* __restrict__ coords,
            const unsigned long long* __restrict__ offs, int n, int extent, int instanced,
            DrawRecord* __restrict__ out, uint32_t* __restrict__ count, unsigned* err) {
  __shared__ uint32_t wsum[32];
  __shared__ uint32_t s_total;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t base = 0;
  for (int tile = 0; tile < n; tile += 1024) {
    const int i = tile + t;
    bool vis = false;
    unsigned long long f0 = 0, nf = 0;
    if (i < n) {
      f0 = offs[i];
      nf = offs[i + 1] - f0;
      vis = nf > 0 && frustum_contains(pl, coords[i], extent);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, vis);
    const uint32_t before = (uint32_t)__popc(bal & ((1u << lane) - 1u));
    if (lane == 0) wsum[warp] = (uint32_t)__popc(bal);
    __syncthreads();
    if (warp == 0) {
      const uint32_t v = wsum[lane];
      uint32_t incl = v;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += u;
      }
      wsum[lane] = incl - v;
      if (lane == 31) s_total = incl;
    }
    __syncthreads();
    if (vis) {
      DrawRecord r;
      bool fits;
      if (instanced) {  // the quad's 6 indices, one instance per face
        fits = f0 + nf <= 0xFFFFFFFFull;
        r.index_count = 6u;
        r.instance_count = (uint32_t)nf;
        r.first_index = 0u;
        r.base_vertex = 0;
        r.first_instance = (uint32_t)f0;
      } else {          // 6 indices per face, chunk-local indices over 4 vertices per face
        fits = 6ull * (f0 + nf) <= 0xFFFFFFFFull && 4ull * f0 <= 0x7FFFFFFFull;
        r.index_count = (uint32_t)(6ull * nf);
        r.instance_count = 1u;
        r.first_index = (uint32_t)(6ull * f0);
        r.base_vertex = (int32_t)(4ull * f0);
        r.first_instance = 0u;
      }
      if (!fits) {
        atomicOr(err, ERR_CAPACITY);
        r = DrawRecord{0u, 0u, 0u, 0, 0u};
      }
      out[base + wsum[warp] + before] = r;
    }
    base += s_total;
    __syncthreads();
  }
  if (t == 0) *count = base;
}

int grid_for(long long work, int threads) {
  long long g = (work + threads - 1) / threads;
  if (g > 152LL * 32) g = 152LL * 32;
  return g < 1 ? 1 : (int)g;
}

}  // namespace

cudaError_t launch_occ_to_cubes(const uint32_t* occ, int n, int n_size, uint8_t* cubes,
                                cudaStream_t st) {
  const long long total = (long long)n * n_size * n_size * n_size;
  if (total == 0) return cudaSuccess;
  k_occ_to_cubes<<<grid_for(total, 256), 256, 0, st>>>(occ, total, n_size, cubes);
  return cudaGetLastError();
}

cudaError_t launch_cubes_to_occ(const uint8_t* cubes, int n, int n_size, uint32_t* occ,
                                cudaStream_t st) {
  const int W = n_size > 32 ? n_size / 32 : 1;
  const long long words = (long long)n * n_size * n_size * W;
  if (words == 0) return cudaSuccess;
  k_cubes_to_occ<<<grid_for(words, 256), 256, 0, st>>>(cubes, words, n_size, occ);
  return cudaGetLastError();
}

cudaError_t launch_frustum(const Planes& planes, const void* coords, int n, int extent,
                           uint8_t* visible, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_frustum<<<(n + 255) / 256, 256, 0, st>>>(planes, static_cast<const vox_chunk_coord*>(coords),
                                              n, extent, visible);
  return cudaGetLastError();
}

cudaError_t launch_draw_list(const Planes& planes, const void* coords,
                             const unsigned long long* offs, int n, int extent, int instanced,
                             DrawRecord* out, uint32_t* count, unsigned* err, cudaStream_t st) {
  k_draw_list<<<1, 1024, 0, st>>>(planes, static_cast<const vox_chunk_coord*>(coords), offs, n,
                                  extent, instanced, out, count, err);
  return cudaGetLastError();
}

}  // namespace vox

// ---------------------------------------------------------------------------------------
// Bounded-wait self-test: the look-back of chunk 1 waits on chunk 0, which never
// publishes (its state word is zero). The wait must end after spin_limit polls with the
// timeout bit latched, leaving the context usable.
// ---------------------------------------------------------------------------------------
#include "vox_device.cuh"

namespace vox {
namespace {
__global__ void k_lookback_probe(unsigned long long* state2, BatchCtl* ctl, int spin_limit) {
  if (threadIdx.x < 32) (void)lookback(state2, ctl, 0xABCDEFu, 1, 0ull, spin_limit);
}
}  // namespace

cudaError_t launch_lookback_probe(unsigned long long* state2, BatchCtl* ctl, int spin_limit,
                                  cudaStream_t st) {
  k_lookback_probe<<<1, 32, 0, st>>>(state2, ctl, spin_limit);
  return cudaGetLastError();
}
}  // namespace vox
