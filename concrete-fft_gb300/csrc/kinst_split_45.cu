// Split-transform kernels (split.cuh) for base algorithms 4 and 5; one
// translation unit per algorithm pair so that they compile in parallel.
#include "split.cuh"

namespace cfft {
const void* c64_split_ptr_45(int algo, bool fwd, int ls, int mode) {
  switch (algo) {
    case 4: return split_ptr<4>(fwd, ls, mode);
    case 5: return split_ptr<5>(fwd, ls, mode);
    default: return nullptr;
  }
}
}  // namespace cfft
