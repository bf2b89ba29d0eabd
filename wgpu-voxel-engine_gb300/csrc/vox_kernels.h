// vox_kernels.h — host-side handles of the instantiated kernels (one set per chunk size).
#pragma once

#include <cuda_runtime.h>

namespace vox {

struct KernelSet {
  int n_size;                // chunk size N
  int threads;               // CTA size of every kernel of the set
  const void* batch[4][2];   // k_mesh_batch<N, gen mode, layout>
  const void* single[2];     // k_mesh_single<N, layout>
  const void* generate[4];   // k_generate<N, gen mode> (index 0 unused)
  int smem_fixed[2];         // bytes before the staging window, per layout
  int (*smem_total)(int layout, int stage_faces);
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

}  // namespace vox
