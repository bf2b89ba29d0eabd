// Kernel instantiations for chunk size N = 8 (one translation unit per size so the
// build compiles them in parallel).
#include "vox_kernel_set.cuh"

namespace vox {
const KernelSet& kernel_set_8() {
  static const KernelSet k = make_kernel_set<8>();
  return k;
}
}  // namespace vox
