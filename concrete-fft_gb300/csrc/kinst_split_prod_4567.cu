// u64 products split over a cluster (split_product.cuh) for base algorithms
// 4..7; two translation units so that they compile in parallel.
#include "split_product.cuh"

namespace cfft {
const void* u64_product_split_ptr_4567(int algo, int ls, bool big) {
  switch (algo) {
    case 4: return split_product_ptr<4>(ls, big);
    case 5: return split_product_ptr<5>(ls, big);
    case 6: return split_product_ptr<6>(ls, big);
    case 7: return split_product_ptr<7>(ls, big);
    default: return nullptr;
  }
}
}  // namespace cfft
