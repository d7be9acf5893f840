// Instantiations: fused u64 product for Dif4/Dit4 with integer-pipe additions.
#include "c64_kernels.cuh"

namespace cfft {
template <int A>
static const void* pick(int e) {
  switch (e) {
    case 4: return (const void*)u64_product_kernel<A, 4, kProdThreads>;
    default: return nullptr;
  }
}
const void* u64_product_kernel_emu(int algo, int e) {
  if (algo == 2) return pick<2>(e);
  if (algo == 3) return pick<3>(e);
  return nullptr;
}
}  // namespace cfft
