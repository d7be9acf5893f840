// u64 products split over a cluster (split_product.cuh) for base algorithms
// 6 and 7; one translation unit per pair so that they compile in parallel.
#include "split_product.cuh"

namespace cfft {
const void* u64_product_split_ptr_67(int algo, int ls, bool big) {
  switch (algo) {
    case 6: return split_product_ptr<6>(ls, big);
    case 7: return split_product_ptr<7>(ls, big);
    default: return nullptr;
  }
}
const void* u64_product_split0_ptr_67(int algo, int ls, bool sum) {
  switch (algo) {
    case 6: return split0_product_ptr<6>(ls, sum);
    case 7: return split0_product_ptr<7>(ls, sum);
    default: return nullptr;
  }
}
const void* u64_product_split2_ptr_67(int algo, int ls0, int ls1, bool sum) {
  switch (algo) {
    case 6: return split2_product_ptr<6>(ls0, ls1, sum);
    case 7: return split2_product_ptr<7>(ls0, ls1, sum);
    default: return nullptr;
  }
}
}  // namespace cfft
