// vox_halo.cu — the neighbour lookup of the staged-halo path of the fused batch.
//
// The fused launch regenerates every chunk's lateral halo in shared memory. The staged-halo
// path instead generates every chunk of the batch once into an occupancy pool and meshes
// from the pool, taking each halo plane from the neighbour's own occupancy (the rebuild
// path's kernel): the neighbours of chunk i are found by looking its neighbours'
// coordinates up in a hash map of the batch (the World.chunks lookup of
// src/chunk_builder.rs:134-169, on the device). A neighbour whose mask bit is set but that
// is not in the batch gets an extra pool slot, into which only the plane that the meshing
// reads is generated: the halo plane the fused launch would generate.
#include <cstdint>

#include "voxgpu.h"
#include "vox_kernels.h"
#include "vox_types.h"

namespace vox {

namespace {

constexpr unsigned long long kEmptyKey = ~0ull;

// 21 bits per coordinate, two's complement; coordinates outside [-2^20, 2^20) do not fit.
__device__ __forceinline__ bool coord_key(vox_chunk_coord c, unsigned long long& key) {
  const int lim = 1 << 20;
  if (c.x < -lim || c.x >= lim || c.y < -lim || c.y >= lim || c.z < -lim || c.z >= lim)
    return false;
  const unsigned long long m = (1ull << 21) - 1;
  key = (((unsigned long long)(unsigned)c.x & m) << 42) | (((unsigned long long)(unsigned)c.y & m) << 21) |
        ((unsigned long long)(unsigned)c.z & m);
  return true;
}

__device__ __forceinline__ unsigned hash_key(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return (unsigned)k;
}

// Inserts coords[i] -> i (the first insert of a coordinate keeps its index) and writes the
// identity slot ident[i] = i (the batch's own pool slots).
__global__ void k_map_insert(const vox_chunk_coord* __restrict__ coords, int n,
                             unsigned long long* keys, int* vals, unsigned cap_mask, int* ident,
                             unsigned* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ident[i] = i;
  unsigned long long key;
  if (!coord_key(coords[i], key)) {
    atomicOr(err, ERR_BAD_INPUT);
    return;
  }
  unsigned h = hash_key(key) & cap_mask;
  for (unsigned probe = 0; probe <= cap_mask; ++probe) {
    const unsigned long long prev = atomicCAS(&keys[h], kEmptyKey, key);
    if (prev == kEmptyKey) {
      vals[h] = i;  // read only by the next launch
      return;
    }
    if (prev == key) return;  // a duplicate coordinate: the first one stands
    h = (h + 1) & cap_mask;
  }
  atomicOr(err, ERR_BAD_INPUT);  // table full: cannot happen at twice the batch size
}

__device__ __forceinline__ int map_find(const unsigned long long* keys, const int* vals,
                                        unsigned cap_mask, vox_chunk_coord c) {
  unsigned long long key;
  if (!coord_key(c, key)) return -1;
  unsigned h = hash_key(key) & cap_mask;
  for (unsigned probe = 0; probe <= cap_mask; ++probe) {
    const unsigned long long k = keys[h];
    if (k == key) return vals[h];
    if (k == kEmptyKey) return -1;
    h = (h + 1) & cap_mask;
  }
  return -1;
}

// One thread per (chunk, direction): nbr_slots[6 i + d] = the pool slot of the neighbour's
// occupancy when mask bit d is set, else -1. A neighbour outside the batch gets an extra
// slot n + e (its coordinate goes to extra[e], the direction to extra_dir[e]; e < dirs * n
// always, since every chunk and loaded direction claims at most one).
__global__ void k_nbr_lookup(const vox_chunk_coord* __restrict__ coords,
                             const uint8_t* __restrict__ masks, int n, int dirs,
                             const unsigned long long* keys, const int* vals, unsigned cap_mask,
                             int* nbr_slots, vox_chunk_coord* extra, uint8_t* extra_dir,
                             unsigned* extra_count) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= 6ll * n) return;
  const int i = (int)(t / 6), d = (int)(t % 6);
  int slot = -1;
  const unsigned m = masks ? masks[i] : 0u;
  if (d < dirs && ((m >> d) & 1u)) {
    const vox_chunk_coord c = coords[i];
    const vox_chunk_coord q = {c.x + (d == 0 ? -1 : d == 1 ? 1 : 0), c.y + (d == 4 ? -1 : d == 5 ? 1 : 0),
                               c.z + (d == 2 ? -1 : d == 3 ? 1 : 0)};
    slot = map_find(keys, vals, cap_mask, q);
    if (slot < 0) {
      const unsigned e = atomicAdd(extra_count, 1u);
      extra[e] = q;
      extra_dir[e] = (uint8_t)d;
      slot = n + (int)e;
    }
  }
  nbr_slots[t] = slot;
}

}  // namespace

cudaError_t launch_halo_lookup(const HaloLookup& h, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(h.keys, 0xFF, sizeof(unsigned long long) * ((size_t)h.cap_mask + 1), st);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(h.extra_count, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
  const int T = 256;
  k_map_insert<<<(h.n + T - 1) / T, T, 0, st>>>(h.coords, h.n, h.keys, h.vals, h.cap_mask, h.ident,
                                                h.err);
  const long long total = 6ll * h.n;
  k_nbr_lookup<<<(unsigned)((total + T - 1) / T), T, 0, st>>>(h.coords, h.masks, h.n, h.dirs, h.keys,
                                                             h.vals, h.cap_mask, h.nbr_slots, h.extra,
                                                             h.extra_dir, h.extra_count);
  return cudaGetLastError();
}

}  // namespace vox
