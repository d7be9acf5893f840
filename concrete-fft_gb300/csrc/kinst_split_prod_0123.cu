// u64 products split over a cluster (split_product.cuh) for base algorithms
// 0..3; two translation units so that they compile in parallel.
#include "split_product.cuh"

namespace cfft {
const void* u64_product_split_ptr_0123(int algo, int ls, bool big) {
  switch (algo) {
    case 0: return split_product_ptr<0>(ls, big);
    case 1: return split_product_ptr<1>(ls, big);
    case 2: return split_product_ptr<2>(ls, big);
    case 3: return split_product_ptr<3>(ls, big);
    default: return nullptr;
  }
}
}  // namespace cfft
