// split_product.cuh -- one negacyclic u64 product (or one Fourier-domain sum
// of products) spread over a thread-block cluster of S = 2^LS CTAs, for
// products whose N/2-point transform does not fit one CTA's shared memory
// (N > 8192) and for small batches.
//
// The transform of n = N/2 points has at least one unordered outer level; its
// level 0 of radix R0 >= S splits it into R0 contiguous slices of m = n/R0
// points that the later levels and the base treat independently (split.cuh).
// CTA c owns part c: points [c*n/S, (c+1)*n/S), i.e. R0/S slices.
//   1. CTA c folds and twists its own part of the input into shared memory.
//   2. Cluster barrier.  Level 0 forward: CTA c takes butterflies
//      [c*m/S, (c+1)*m/S), reads their inputs from the parts of all CTAs and
//      stores each output into the part that owns its slot, both through
//      distributed shared memory.
//   3. Cluster barrier (the peers are done reading the twisted parts).  Levels
//      1.. and the base forward on the CTA's slices, the pointwise product with
//      the resident operand (its permuted order is part-contiguous), added into
//      a register accumulator (steps 1-3 repeat per term of a sum).
//   4. The base and levels .. 1 inverse on the accumulator.
//   5. Cluster barrier.  Level 0 inverse: CTA c takes butterflies
//      [c*m/S, (c+1)*m/S), reads their inputs from the parts of all CTAs,
//      untwists and rounds the R0 outputs of each and stores them; a last
//      cluster barrier keeps every CTA alive while a peer reads its memory.
// Every butterfly and elementwise step does the operations of the one-CTA
// product kernel on the same values, so results are bit-identical to it.
#pragma once
#include <cooperative_groups.h>

#include "../../include/cfft.h"
#include "split.cuh"

namespace cfft {

// CTA sizes of the split product kernel: up to 256 threads (registers for
// several CTAs per SM), and a 512-thread variant for parts of 4096 points,
// where shared memory allows one CTA per SM.
constexpr int kSplitProdThreads = 256;
constexpr int kSplitProdThreadsBig = 512;

// Step 4 for radix R0: butterflies [i0, i1), inputs from the parts `src[j]`,
// outputs k*m + i untwisted by itw and rounded into the product's N words.
template <int R0, int LS>
__device__ __forceinline__ void level0_inv_untwist(double2* const* src, int lm, int log2n, int i0, int i1,
                                                   const double2* __restrict__ wl, const double2* __restrict__ itw,
                                                   uint64_t* __restrict__ op, int tid, int nth) {
  constexpr int LR0 = Log2<R0>::v;
  constexpr int SL = R0 >> LS;
  const int n = 1 << log2n;
  for (int i = i0 + tid; i < i1; i += nth) {
    c64 v[R0];
    const double2* tw = wl + (R0 - 1) * i - 1;
    v[0] = ld(src[0] + i);
#pragma unroll
    for (int k = 1; k < R0; ++k) {
      const int sl = slot<R0>(k);
      v[k] = cmul(ldg(tw + k), ld(src[sl >> (LR0 - LS)] + ((sl & (SL - 1)) << lm) + i));
    }
    Core<R0, false, 0>::run(v);
#pragma unroll
    for (int k = 0; k < R0; ++k) {
      const int j = (k << lm) + i;
      const c64 t = cmul(ldg(itw + j), v[k]);
      __stcs(op + j, round_half_up_mod64(t.re));
      __stcs(op + j + n, round_half_up_mod64(t.im));
    }
  }
}

// Accumulator entries per thread: the CTA sizes keep a part at most 8 entries
// per thread (1024 points / 128 threads, 2048 / 256, 4096 / 512).
constexpr int kSplitAcc = 8;

// One output per cluster of S CTAs (blockIdx.x >> LS): the sum over `terms`
// products a_t * B_t, accumulated in the Fourier domain in term order, then
// one inverse (terms = 1: a plain product).  Shared memory: two buffers of n/S
// points; the accumulator lives in registers.  a: N u64 per term (terms of an
// output consecutive); bhat: n c64 per term at bhat_stride (0: one operand for
// all); out: N u64 per output.  When `items` is not null (terms = 1), product
// p takes its three pointers from items[p] instead.  Requires L.nlevels >= 1,
// 2^L.log2r[0] >= S and n/S <= kSplitAcc x blockDim.x.
template <int ALGO, int LS, int MAXT>
__global__ void __launch_bounds__(MAXT) u64_product_split_kernel(
    const uint64_t* __restrict__ a, const double2* __restrict__ bhat, long bhat_stride, uint64_t* __restrict__ out,
    int terms, const cfft_product_item* __restrict__ items, DevLevels L, const double2* __restrict__ w,
    const double2* __restrict__ winv, const double2* __restrict__ tw, const double2* __restrict__ itw) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double2 smem[];
  const int log2n = L.log2n[0];
  const int log2c = log2n - LS;  // points per part
  const int c = (int)(blockIdx.x & ((1 << LS) - 1));
  const long g = (long)(blockIdx.x >> LS);  // output index
  double2* x = smem;
  double2* y = smem + (1 << log2c);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int n = 1 << log2n;
  const int base = c << log2c;
  const int lr0 = L.log2r[0];
  const int lm = log2n - lr0;
  const int per = (1 << lm) >> LS;
  const int nsl = 1 << (lr0 - LS);
  double2* peer_y[1 << LS];
  double2* peer_x[1 << LS];
#pragma unroll
  for (int j = 0; j < (1 << LS); ++j) {
    peer_y[j] = cl.map_shared_rank(y, (unsigned)j);
    peer_x[j] = cl.map_shared_rank(x, (unsigned)j);
  }
  c64 acc[kSplitAcc];
  double2* src = x;  // input of the inverse
  uint64_t* op = items ? items[g].out : out + (g << (log2n + 1));

  for (int t = 0; t < terms; ++t) {
    const long term = g * terms + t;
    const uint64_t* ap = items ? items[g].a : a + (term << (log2n + 1));
    const double2* bprod = items ? (const double2*)items[g].bhat : bhat + term * bhat_stride;

    // 1. fold and twist this CTA's part into y
    for (int j = tid; j < (1 << log2c); j += nth) {
      const int gj = base + j;
      const c64 v{i64_to_f64_rne((int64_t)__ldcs(ap + gj)), i64_to_f64_rne((int64_t)__ldcs(ap + gj + n))};
      st(y + j, cmul(ldg(tw + gj), v));
    }
    cl.sync();

    // 2. level 0 forward: 1/S of the butterflies, each output into its owner's x
    const double2* wl = w + L.w_off[0];
    if (lr0 == 1) {
      if constexpr (LS <= 1) level0_scatter<2, LS>(peer_y, peer_x, lm, c * per, (c + 1) * per, wl, tid, nth);
    } else if (lr0 == 2) {
      if constexpr (LS <= 2) level0_scatter<4, LS>(peer_y, peer_x, lm, c * per, (c + 1) * per, wl, tid, nth);
    } else {
      level0_scatter<8, LS>(peer_y, peer_x, lm, c * per, (c + 1) * per, wl, tid, nth);
    }
    cl.sync();  // every part's x is complete and every peer has read this CTA's y

    // 3. the slices forward, the pointwise product added into the accumulator
    // (a single term: stored in place, the inverse starts from it)
    const FlatBuf r = unordered_t<true, 0, ALGO>(L, 1, nsl, FlatBuf{x}, FlatBuf{y}, w, tid, nth);
    const double2* bp = bprod + base;
#pragma unroll
    for (int k = 0; k < kSplitAcc; ++k) {
      const int j = tid + k * nth;
      if (j < (1 << log2c)) {
        const c64 p = cmul(ldg(bp + j), ld(r.p + j));
        if (terms == 1) st(r.p + j, p);
        else acc[k] = t == 0 ? p : cadd(acc[k], p);
      }
    }
    __syncthreads();  // r is read before the next term overwrites x and y
    if (terms == 1) src = r.p;
  }

  // 4. the slices inverse, from the accumulator
  if (terms > 1) {
#pragma unroll
    for (int k = 0; k < kSplitAcc; ++k) {
      const int j = tid + k * nth;
      if (j < (1 << log2c)) st(x + j, acc[k]);
    }
    __syncthreads();
  }
  const FlatBuf s = unordered_t<false, 0, ALGO>(L, 1, nsl, FlatBuf{src}, FlatBuf{src == x ? y : x}, winv, tid, nth);
  double2* peer_s[1 << LS];
#pragma unroll
  for (int j = 0; j < (1 << LS); ++j) peer_s[j] = cl.map_shared_rank(s.p, (unsigned)j);
  cl.sync();

  // 5. level 0 inverse, untwist and round
  const double2* wli = winv + L.winv_off[0];
  if (lr0 == 1) {
    if constexpr (LS <= 1) level0_inv_untwist<2, LS>(peer_s, lm, log2n, c * per, (c + 1) * per, wli, itw, op, tid, nth);
  } else if (lr0 == 2) {
    if constexpr (LS <= 2) level0_inv_untwist<4, LS>(peer_s, lm, log2n, c * per, (c + 1) * per, wli, itw, op, tid, nth);
  } else {
    level0_inv_untwist<8, LS>(peer_s, lm, log2n, c * per, (c + 1) * per, wli, itw, op, tid, nth);
  }
  cl.sync();  // no CTA exits while a peer reads its shared memory
}

// kernel pointers by base algorithm (kinst_split_prod_*.cu)
// (big: the 512-thread variant, S = 8 only)
const void* u64_product_split_ptr_0123(int algo, int ls, bool big);
const void* u64_product_split_ptr_4567(int algo, int ls, bool big);

template <int A>
const void* split_product_ptr(int ls, bool big) {
  if (big) return ls == 3 ? (const void*)u64_product_split_kernel<A, 3, kSplitProdThreadsBig> : nullptr;
  switch (ls) {
    case 1: return (const void*)u64_product_split_kernel<A, 1, kSplitProdThreads>;
    case 2: return (const void*)u64_product_split_kernel<A, 2, kSplitProdThreads>;
    case 3: return (const void*)u64_product_split_kernel<A, 3, kSplitProdThreads>;
    default: return nullptr;
  }
}

}  // namespace cfft
