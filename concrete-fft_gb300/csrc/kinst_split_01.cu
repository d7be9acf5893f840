// Split-transform kernels (split.cuh) for base algorithms 0 and 1; one
// translation unit per algorithm pair so that they compile in parallel.
#include "split.cuh"

namespace cfft {
const void* c64_split_ptr_01(int algo, bool fwd, int ls, int mode) {
  switch (algo) {
    case 0: return split_ptr<0>(fwd, ls, mode);
    case 1: return split_ptr<1>(fwd, ls, mode);
    default: return nullptr;
  }
}
}  // namespace cfft
