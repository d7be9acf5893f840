// u64 products split over a cluster (split_product.cuh) for base algorithms
// 0 and 1; one translation unit per pair so that they compile in parallel.
#include "split_product.cuh"

namespace cfft {
const void* u64_product_split_ptr_01(int algo, int ls, bool big) {
  switch (algo) {
    case 0: return split_product_ptr<0>(ls, big);
    case 1: return split_product_ptr<1>(ls, big);
    default: return nullptr;
  }
}
const void* u64_product_split0_ptr_01(int algo, int ls, bool sum) {
  switch (algo) {
    case 0: return split0_product_ptr<0>(ls, sum);
    case 1: return split0_product_ptr<1>(ls, sum);
    default: return nullptr;
  }
}
const void* u64_product_split2_ptr_01(int algo, int ls0, int ls1, bool sum) {
  switch (algo) {
    case 0: return split2_product_ptr<0>(ls0, ls1, sum);
    case 1: return split2_product_ptr<1>(ls0, ls1, sum);
    default: return nullptr;
  }
}
}  // namespace cfft
