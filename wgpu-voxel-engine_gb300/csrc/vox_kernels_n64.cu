// Kernel instantiations for chunk size N = 64 (one translation unit per size so the
// build compiles them in parallel).
#include "vox_kernel_set.cuh"

namespace vox {
const KernelSet& kernel_set_64() {
  static const KernelSet k = make_kernel_set<64>();
  return k;
}
}  // namespace vox
