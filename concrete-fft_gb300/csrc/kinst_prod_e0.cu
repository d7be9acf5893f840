// Instantiations: fused u64 product and operand preparation, every algorithm, FP64-pipe additions only.
#include "c64_kernels.cuh"

namespace cfft {
const void* u64_product_kernel_e0(int algo) {
  switch (algo) {
    case 0: return (const void*)u64_product_kernel<0, 0, kProdThreads>;
    case 1: return (const void*)u64_product_kernel<1, 0, kProdThreads>;
    case 2: return (const void*)u64_product_kernel<2, 0, kProdThreads>;
    case 3: return (const void*)u64_product_kernel<3, 0, kProdThreads>;
    case 4: return (const void*)u64_product_kernel<4, 0, kProdThreads>;
    case 5: return (const void*)u64_product_kernel<5, 0, kProdThreads>;
    case 6: return (const void*)u64_product_kernel<6, 0, kProdThreads>;
    case 7: return (const void*)u64_product_kernel<7, 0, kProdThreads>;
    default: return nullptr;
  }
}
const void* u64_prepare_kernel_ptr(int algo) {
  switch (algo) {
    case 0: return (const void*)u64_prepare_kernel<0, kProdThreads>;
    case 1: return (const void*)u64_prepare_kernel<1, kProdThreads>;
    case 2: return (const void*)u64_prepare_kernel<2, kProdThreads>;
    case 3: return (const void*)u64_prepare_kernel<3, kProdThreads>;
    case 4: return (const void*)u64_prepare_kernel<4, kProdThreads>;
    case 5: return (const void*)u64_prepare_kernel<5, kProdThreads>;
    case 6: return (const void*)u64_prepare_kernel<6, kProdThreads>;
    case 7: return (const void*)u64_prepare_kernel<7, kProdThreads>;
    default: return nullptr;
  }
}
template <int A>
static const void* pick_sum(bool reg_acc) {
  return reg_acc ? (const void*)u64_product_sum_kernel<A, kProdThreads, kSumRegAcc>
                 : (const void*)u64_product_sum_kernel<A, kProdThreads, 0>;
}
const void* u64_product_sum_kernel_ptr(int algo, bool reg_acc) {
  switch (algo) {
    case 0: return pick_sum<0>(reg_acc);
    case 1: return pick_sum<1>(reg_acc);
    case 2: return pick_sum<2>(reg_acc);
    case 3: return pick_sum<3>(reg_acc);
    case 4: return pick_sum<4>(reg_acc);
    case 5: return pick_sum<5>(reg_acc);
    case 6: return pick_sum<6>(reg_acc);
    case 7: return pick_sum<7>(reg_acc);
    default: return nullptr;
  }
}
}  // namespace cfft
