// Instantiations: c64 shared-memory kernels for Dif4/Dit4 with integer-pipe additions.
#include "c64_kernels.cuh"

namespace cfft {
template <int A, int E>
static const void* pick(bool fwd) {
  return fwd ? (const void*)c64_smem_kernel<A, E, true> : (const void*)c64_smem_kernel<A, E, false>;
}
template <int A>
static const void* pick_e(int e, bool fwd) {
  switch (e) {
    case 4: return pick<A, 4>(fwd);
    default: return nullptr;
  }
}
const void* c64_kernel_emu(int algo, int e, bool fwd) {
  if (algo == 2) return pick_e<2>(e, fwd);
  if (algo == 3) return pick_e<3>(e, fwd);
  return nullptr;
}
}  // namespace cfft
