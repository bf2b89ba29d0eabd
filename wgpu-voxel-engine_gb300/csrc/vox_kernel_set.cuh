// vox_kernel_set.cuh — builds the KernelSet of one chunk size (included once per size).
#pragma once

#include "vox_device.cuh"
#include "vox_kernels.h"

namespace vox {

template <int N>
static int smem_total_n(int layout, int threads, int stage_faces) {
  return layout == VOX_LAYOUT_INSTANCED
             ? SmemPlan<N, VOX_LAYOUT_INSTANCED>::total(threads, stage_faces)
             : SmemPlan<N, VOX_LAYOUT_VERTEX>::total(threads, stage_faces);
}

template <int N, int GM, int L>
static void fill_batch(KernelSet& k) {
  k.batch[GM][L][0] = (const void*)k_mesh_batch<N, GM, L, Shape<N>::T0>;
  k.batch[GM][L][1] = (const void*)k_mesh_batch<N, GM, L, Shape<N>::T1>;
  k.phased[GM][L][0] = (const void*)k_mesh_batch_phased<N, GM, L, Shape<N>::T0>;
  k.phased[GM][L][1] = (const void*)k_mesh_batch_phased<N, GM, L, Shape<N>::T1>;
  k.overlap[GM][L][0] = (const void*)k_mesh_batch_overlap<N, GM, L, Shape<N>::T0>;
  k.overlap[GM][L][1] = (const void*)k_mesh_batch_overlap<N, GM, L, Shape<N>::T1>;
}

template <int N>
static KernelSet make_kernel_set() {
  KernelSet k{};
  k.n_size = N;
  k.threads[0] = Shape<N>::T0;
  k.threads[1] = Shape<N>::T1;
  fill_batch<N, GM_OCC, VOX_LAYOUT_VERTEX>(k);
  fill_batch<N, GM_OCC, VOX_LAYOUT_INSTANCED>(k);
  fill_batch<N, GM_HEIGHT, VOX_LAYOUT_VERTEX>(k);
  fill_batch<N, GM_HEIGHT, VOX_LAYOUT_INSTANCED>(k);
  fill_batch<N, GM_DENSITY, VOX_LAYOUT_VERTEX>(k);
  fill_batch<N, GM_DENSITY, VOX_LAYOUT_INSTANCED>(k);
  fill_batch<N, GM_BERNOULLI, VOX_LAYOUT_VERTEX>(k);
  fill_batch<N, GM_BERNOULLI, VOX_LAYOUT_INSTANCED>(k);
  k.single[0][0] = (const void*)k_mesh_single<N, VOX_LAYOUT_VERTEX, Shape<N>::T0>;
  k.single[0][1] = (const void*)k_mesh_single<N, VOX_LAYOUT_VERTEX, Shape<N>::T1>;
  k.single[1][0] = (const void*)k_mesh_single<N, VOX_LAYOUT_INSTANCED, Shape<N>::T0>;
  k.single[1][1] = (const void*)k_mesh_single<N, VOX_LAYOUT_INSTANCED, Shape<N>::T1>;
  k.gen_threads = Shape<N>::T1;
  k.spill_bytes = SmemPlan<N, VOX_LAYOUT_VERTEX>::kSpill;
  k.generate[0] = nullptr;
  k.generate[GM_HEIGHT] = (const void*)k_generate<N, GM_HEIGHT, Shape<N>::T1>;
  k.generate[GM_DENSITY] = (const void*)k_generate<N, GM_DENSITY, Shape<N>::T1>;
  k.generate[GM_BERNOULLI] = (const void*)k_generate<N, GM_BERNOULLI, Shape<N>::T1>;
  k.generate_planes[0] = nullptr;
  k.generate_planes[GM_HEIGHT] = (const void*)k_generate_planes<N, GM_HEIGHT, Shape<N>::T1>;
  k.generate_planes[GM_DENSITY] = (const void*)k_generate_planes<N, GM_DENSITY, Shape<N>::T1>;
  k.generate_planes[GM_BERNOULLI] = nullptr;  // Bernoulli chunks have no neighbours
  k.smem_total = &smem_total_n<N>;
  return k;
}

}  // namespace vox
