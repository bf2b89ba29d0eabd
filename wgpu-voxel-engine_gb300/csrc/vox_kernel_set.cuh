// vox_kernel_set.cuh — builds the KernelSet of one chunk size (included once per size).
#pragma once

#include "vox_device.cuh"
#include "vox_kernels.h"

namespace vox {

template <int N>
static int smem_total_n(int layout, int stage_faces) {
  return layout == VOX_LAYOUT_INSTANCED ? SmemPlan<N, VOX_LAYOUT_INSTANCED>::total(stage_faces)
                                        : SmemPlan<N, VOX_LAYOUT_VERTEX>::total(stage_faces);
}

template <int N>
static KernelSet make_kernel_set() {
  KernelSet k{};
  k.n_size = N;
  k.threads = Shape<N>::THREADS;
  k.batch[GM_OCC][0] = (const void*)k_mesh_batch<N, GM_OCC, VOX_LAYOUT_VERTEX>;
  k.batch[GM_OCC][1] = (const void*)k_mesh_batch<N, GM_OCC, VOX_LAYOUT_INSTANCED>;
  k.batch[GM_HEIGHT][0] = (const void*)k_mesh_batch<N, GM_HEIGHT, VOX_LAYOUT_VERTEX>;
  k.batch[GM_HEIGHT][1] = (const void*)k_mesh_batch<N, GM_HEIGHT, VOX_LAYOUT_INSTANCED>;
  k.batch[GM_DENSITY][0] = (const void*)k_mesh_batch<N, GM_DENSITY, VOX_LAYOUT_VERTEX>;
  k.batch[GM_DENSITY][1] = (const void*)k_mesh_batch<N, GM_DENSITY, VOX_LAYOUT_INSTANCED>;
  k.batch[GM_BERNOULLI][0] = (const void*)k_mesh_batch<N, GM_BERNOULLI, VOX_LAYOUT_VERTEX>;
  k.batch[GM_BERNOULLI][1] = (const void*)k_mesh_batch<N, GM_BERNOULLI, VOX_LAYOUT_INSTANCED>;
  k.single[0] = (const void*)k_mesh_single<N, VOX_LAYOUT_VERTEX>;
  k.single[1] = (const void*)k_mesh_single<N, VOX_LAYOUT_INSTANCED>;
  k.generate[0] = nullptr;
  k.generate[GM_HEIGHT] = (const void*)k_generate<N, GM_HEIGHT>;
  k.generate[GM_DENSITY] = (const void*)k_generate<N, GM_DENSITY>;
  k.generate[GM_BERNOULLI] = (const void*)k_generate<N, GM_BERNOULLI>;
  k.smem_fixed[0] = SmemPlan<N, VOX_LAYOUT_VERTEX>::kFixed;
  k.smem_fixed[1] = SmemPlan<N, VOX_LAYOUT_INSTANCED>::kFixed;
  k.smem_total = &smem_total_n<N>;
  return k;
}

}  // namespace vox
