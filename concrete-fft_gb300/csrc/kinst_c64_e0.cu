// Instantiations: c64 shared-memory kernels, every algorithm, FP64-pipe additions only.
#include "c64_kernels.cuh"

namespace cfft {
template <int A>
static const void* pick(bool fwd) {
  return fwd ? (const void*)c64_smem_kernel<A, 0, true> : (const void*)c64_smem_kernel<A, 0, false>;
}
const void* c64_kernel_e0(int algo, bool fwd) {
  switch (algo) {
    case 0: return pick<0>(fwd);
    case 1: return pick<1>(fwd);
    case 2: return pick<2>(fwd);
    case 3: return pick<3>(fwd);
    case 4: return pick<4>(fwd);
    case 5: return pick<5>(fwd);
    case 6: return pick<6>(fwd);
    case 7: return pick<7>(fwd);
    default: return nullptr;
  }
}
const void* c64_split_ptr_01(int algo, bool fwd, int ls, int mode);
const void* c64_split_ptr_23(int algo, bool fwd, int ls, int mode);
const void* c64_split_ptr_45(int algo, bool fwd, int ls, int mode);
const void* c64_split_ptr_67(int algo, bool fwd, int ls, int mode);
const void* c64_split_kernel_ptr(int algo, bool fwd, int ls, int mode) {
  switch (algo >> 1) {
    case 0: return c64_split_ptr_01(algo, fwd, ls, mode);
    case 1: return c64_split_ptr_23(algo, fwd, ls, mode);
    case 2: return c64_split_ptr_45(algo, fwd, ls, mode);
    case 3: return c64_split_ptr_67(algo, fwd, ls, mode);
    default: return nullptr;
  }
}
}  // namespace cfft
