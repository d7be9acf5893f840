// u64 products split over a cluster (split_product.cuh) for base algorithms
// 4 and 5; one translation unit per pair so that they compile in parallel.
#include "split_product.cuh"

namespace cfft {
const void* u64_product_split_ptr_45(int algo, int ls, bool big) {
  switch (algo) {
    case 4: return split_product_ptr<4>(ls, big);
    case 5: return split_product_ptr<5>(ls, big);
    default: return nullptr;
  }
}
const void* u64_product_split0_ptr_45(int algo, int ls, bool sum) {
  switch (algo) {
    case 4: return split0_product_ptr<4>(ls, sum);
    case 5: return split0_product_ptr<5>(ls, sum);
    default: return nullptr;
  }
}
const void* u64_product_split2_ptr_45(int algo, int ls0, int ls1, bool sum) {
  switch (algo) {
    case 4: return split2_product_ptr<4>(ls0, ls1, sum);
    case 5: return split2_product_ptr<5>(ls0, ls1, sum);
    default: return nullptr;
  }
}
}  // namespace cfft
