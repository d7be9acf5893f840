// Split-transform kernels (split.cuh) for base algorithms 6 and 7; one
// translation unit per algorithm pair so that they compile in parallel.
#include "split.cuh"

namespace cfft {
const void* c64_split_ptr_67(int algo, bool fwd, int ls, int mode) {
  switch (algo) {
    case 6: return split_ptr<6>(fwd, ls, mode);
    case 7: return split_ptr<7>(fwd, ls, mode);
    default: return nullptr;
  }
}
}  // namespace cfft
