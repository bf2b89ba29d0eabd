// Kernel instantiations for chunk size N = 32 (one translation unit per size so the
// build compiles them in parallel).
#include "vox_kernel_set.cuh"

namespace vox {
const KernelSet& kernel_set_32() {
  static const KernelSet k = make_kernel_set<32>();
  return k;
}
}  // namespace vox
