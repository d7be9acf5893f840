// Split-transform kernels (split.cuh) for base algorithms 2 and 3; one
// translation unit per algorithm pair so that they compile in parallel.
#include "split.cuh"

namespace cfft {
const void* c64_split_ptr_23(int algo, bool fwd, int ls, int mode) {
  switch (algo) {
    case 2: return split_ptr<2>(fwd, ls, mode);
    case 3: return split_ptr<3>(fwd, ls, mode);
    default: return nullptr;
  }
}
}  // namespace cfft
