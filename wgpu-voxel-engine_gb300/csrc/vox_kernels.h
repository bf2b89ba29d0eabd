// vox_kernels.h — host-side handles of the instantiated kernels (one set per chunk size).
#pragma once

#include <cuda_runtime.h>

#include "voxgpu.h"

namespace vox {

struct KernelSet {
  int n_size;                   // chunk size N
  int threads[2];               // the two CTA sizes the meshing kernels exist in
  const void* batch[4][2][2];   // k_mesh_batch<N, gen mode, layout, threads[t]>
  const void* phased[4][2][2];  // k_mesh_batch_phased<N, gen mode, layout, threads[t]>
  const void* overlap[4][2][2]; // k_mesh_batch_overlap<N, gen mode, layout, threads[t]>
  const void* single[2][2];     // k_mesh_single<N, layout, threads[t]>
  const void* generate[4];      // k_generate<N, gen mode, gen_threads> (index 0 unused)
  const void* generate_planes[4]; // k_generate_planes<N, gen mode, gen_threads> (height, density)
  int gen_threads;
  int spill_bytes;              // chunk state of one chunk (phased scratch)
  // dynamic shared memory of a launch (layout, CTA size, staging window in faces)
  int (*smem_total)(int layout, int threads, int stage_faces);
};

const KernelSet& kernel_set_8();
const KernelSet& kernel_set_16();
const KernelSet& kernel_set_32();
const KernelSet& kernel_set_64();

// Misc kernels (vox_misc.cu).
cudaError_t launch_occ_to_cubes(const uint32_t* occ, int n, int n_size, uint8_t* cubes,
                                cudaStream_t st);
cudaError_t launch_cubes_to_occ(const uint8_t* cubes, int n, int n_size, uint32_t* occ,
                                cudaStream_t st);
struct Planes {
  float p[24];
};
cudaError_t launch_frustum(const Planes& planes, const void* coords, int n, int extent,
                           uint8_t* visible, cudaStream_t st);
using DrawRecord = vox_draw_indexed_indirect;
struct RasterArgs {
  const void* vertices;     // vertex-layout records, 96 B per face
  const void* indices;      // 6 u32 per face
  unsigned long long faces;
  int width, height;
  float m[16];              // global matrix, column-major
  uint32_t tex[6];          // texture index per face slot
};
// Renders the faces into rgba (width x height x 4 bytes); keys: width x height u64.
cudaError_t launch_raster(const RasterArgs& a, unsigned long long* keys, uint8_t* rgba,
                          cudaStream_t st);
cudaError_t launch_draw_list(const Planes& planes, const void* coords,
                             const unsigned long long* offs, int n, int extent, int instanced,
                             DrawRecord* out, uint32_t* count, unsigned* err, cudaStream_t st);

// Neighbour lookup of the staged-halo path (vox_halo.cu): a hash map of the batch's
// coordinates (cap_mask + 1 slots, a power of two at least twice n), then per chunk and
// direction the pool slot of the neighbour's occupancy (-1: not loaded), with the
// neighbours that are not in the batch listed in `extra` (count in *extra_count) for slots
// n, n + 1, ..., with the direction from the batch chunk to each in `extra_dir`.
// Out-of-range coordinates latch ERR_BAD_INPUT in *err.
struct HaloLookup {
  const vox_chunk_coord* coords;
  const uint8_t* masks;  // null: no neighbour is loaded
  int n;
  int dirs;              // 4 lateral directions, or 6 with VOX_CULL_FULL6
  unsigned long long* keys;
  int* vals;
  unsigned cap_mask;
  int* nbr_slots;        // 6 per chunk
  int* ident;            // ident[i] = i (the batch's own pool slots)
  vox_chunk_coord* extra;
  uint8_t* extra_dir;
  unsigned* extra_count;
  unsigned* err;
};
cudaError_t launch_halo_lookup(const HaloLookup& h, cudaStream_t st);

struct BatchCtl;
// One look-back for chunk 1 of a batch whose chunk 0 never publishes: the wait must give
// up after spin_limit polls and latch the timeout bit in ctl (the bounded-wait self-test).
cudaError_t launch_lookback_probe(unsigned long long* state2, BatchCtl* ctl, int spin_limit,
                                  cudaStream_t st);

}  // namespace vox
