// u64 products split over a cluster (split_product.cuh) for base algorithms
// 2 and 3; one translation unit per pair so that they compile in parallel.
#include "split_product.cuh"

namespace cfft {
const void* u64_product_split_ptr_23(int algo, int ls, bool big) {
  switch (algo) {
    case 2: return split_product_ptr<2>(ls, big);
    case 3: return split_product_ptr<3>(ls, big);
    default: return nullptr;
  }
}
const void* u64_product_split0_ptr_23(int algo, int ls, bool sum) {
  switch (algo) {
    case 2: return split0_product_ptr<2>(ls, sum);
    case 3: return split0_product_ptr<3>(ls, sum);
    default: return nullptr;
  }
}
const void* u64_product_split2_ptr_23(int algo, int ls0, int ls1, bool sum) {
  switch (algo) {
    case 2: return split2_product_ptr<2>(ls0, ls1, sum);
    case 3: return split2_product_ptr<3>(ls0, ls1, sum);
    default: return nullptr;
  }
}
}  // namespace cfft
