// split_product.cuh -- one negacyclic u64 product (or one Fourier-domain sum
// of products) spread over a thread-block cluster of S = 2^LS CTAs, for
// products whose N/2-point transform does not fit one CTA's shared memory
// (N > 8192) and for small batches.  Two kernels: u64_product_split_kernel
// for plans with an unordered outer level (below) and
// u64_product_split0_kernel for plans without one (n = base_n).
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
// The same for u64_product_split0_kernel, whose launches give at least one
// thread per two points of a part.
constexpr int kSplit0Acc = 2;

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

// One product per cluster of S = 2^LS CTAs (S <= the base radix R) when the
// N/2-point transform has no outer level (n = base_n, e.g. N = 2048 on a
// 1024-point base), for latency: a few products then run on S SMs each
// instead of one.  The residue classes mod S of the base algorithm's passes
// (split.cuh) are the parts: CTA c holds the points j*S + c of the transform,
// compacted to j.
// DIF base: the forward's first pass is shared out (CTA c folds and twists the
// inputs of its butterflies into y, then stores each output into the part of
// its class through distributed shared memory); after a cluster barrier every
// later pass, the pointwise product and the inverse's first pass are local to
// the class -- the inverse's first-pass butterfly p reads the points k*n/R + p,
// all of class p mod S -- and the inverse's first-pass outputs go to the parts
// of their classes (a third buffer z, which no CTA uses before); after a
// second barrier the rest of the inverse, the untwist and the rounding are
// local.
// DIT base: CTA c folds and twists its class, runs every forward pass but the
// last alone, and takes the last pass's butterflies p = c + b*S, whose inputs
// come from every part and whose outputs (the points k*n/R + p) all belong to
// class c: the pointwise product is applied as they are stored into z.  Every
// inverse pass but the last is local; the last reads every part and its
// outputs are untwisted, rounded and stored.
// SUM (DIF bases): one output is the Fourier-domain sum of `terms` products:
// each term runs the forward steps and is multiplied and added into a register
// accumulator in term order, as in u64_product_sum_kernel, then one inverse.
// Every butterfly and elementwise step does the operations of the one-CTA
// product kernel on the same values, so results are bit-identical to it.
// Shared memory: three buffers of n/S points.  Requires L.nlevels == 0,
// S <= R, n >= R*S and, for SUM, n/S <= kSplit0Acc x blockDim.x.
template <int ALGO, int LS, bool SUM>
__global__ void __launch_bounds__(256) u64_product_split0_kernel(
    const uint64_t* __restrict__ a, const double2* __restrict__ bhat, long bhat_stride, uint64_t* __restrict__ out,
    int terms, const cfft_product_item* __restrict__ items, DevLevels L, const double2* __restrict__ w,
    const double2* __restrict__ winv, const double2* __restrict__ tw, const double2* __restrict__ itw) {
  constexpr int R = AlgoInfo<ALGO>::R;
  constexpr int LR = Log2<R>::v;
  constexpr int S = 1 << LS;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double2 smem[];
  const int log2n = L.log2n[0];
  const int log2c = log2n - LS;
  const int n = 1 << log2n;
  const int c = (int)(blockIdx.x & (S - 1));
  const long g = (long)(blockIdx.x >> LS);
  double2* x = smem;
  double2* y = smem + (1 << log2c);
  double2* z = smem + (2 << log2c);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lper = log2n - LR;          // log2(n/R)
  const int lpc = lper - LS;            // log2 of the first/last-pass butterflies per CTA
  const int per = 1 << lpc;
  const uint64_t* ap = items ? items[g].a : a + (g << (log2n + 1));
  const double2* bp = items ? (const double2*)items[g].bhat : bhat + g * bhat_stride;
  uint64_t* op = items ? items[g].out : out + (g << (log2n + 1));
  const double2* wf = w + L.w_off[0] + n;  // the base's forward and inverse tables
  const double2* wi = winv + n;

  if constexpr (!AlgoInfo<ALGO>::DIT) {
    double2* peer_x[S];
    double2* peer_z[S];
#pragma unroll
    for (int j = 0; j < S; ++j) {
      peer_x[j] = cl.map_shared_rank(x, (unsigned)j);
      peer_z[j] = cl.map_shared_rank(z, (unsigned)j);
    }
    // SUM: a sum of `terms` products (terms of an output consecutive in a and bhat,
    // bhat at stride bhat_stride): each term forward and multiplied, added into
    // registers in term order, one inverse.  Otherwise one product (terms = 1).
    c64 acc[SUM ? kSplit0Acc : 1];
    const double2* src = x;  // input of the inverse's first pass
    const int nterms = SUM ? terms : 1;
#pragma unroll 1
    for (int t = 0; t < nterms; ++t) {
      const long term = g * nterms + t;
      const uint64_t* tap = SUM ? a + (term << (log2n + 1)) : ap;
      const double2* tbp = SUM ? bhat + term * bhat_stride : bp;
      // every CTA runs, and is done with its x from the previous term, before a peer
      // writes its x
      auto token = cl.barrier_arrive();
      if (t > 0) __syncthreads();  // this CTA is done with y
      // input k of first-pass butterfly c*per + b, folded and twisted, at y[k*per + b]
      for (int q = tid; q < (R << lpc); q += nth) {
        const int j = ((q >> lpc) << lper) + c * per + (q & (per - 1));
        const c64 v{i64_to_f64_rne((int64_t)__ldcs(tap + j)), i64_to_f64_rne((int64_t)__ldcs(tap + j + n))};
        st(y + q, cmul(ldg(tw + j), v));
      }
      __syncthreads();
      cl.barrier_wait(std::move(token));
      first_pass_scatter<R, true, LS>([&](int k, int b, int) { return ld(y + (k << lpc) + b); }, per, c * per, 1,
                                      peer_x, wf, tid, nth);
      cl.sync();  // every part's x is complete
      const FlatBuf r = dif_after_first<R, true>(log2n, LS, FlatBuf{x}, FlatBuf{y}, wf, tid, nth);
      if constexpr (!SUM) {
        for (int j = tid; j < (1 << log2c); j += nth) st(r.p + j, cmul(ldg(tbp + (j << LS) + c), ld(r.p + j)));
        src = r.p;
      } else {
#pragma unroll
        for (int k = 0; k < kSplit0Acc; ++k) {
          const int j = tid + k * nth;
          if (j < (1 << log2c)) {
            const c64 p = cmul(ldg(tbp + (j << LS) + c), ld(r.p + j));
            acc[k] = t == 0 ? p : cadd(acc[k], p);
          }
        }
      }
    }
    if constexpr (SUM) {
      __syncthreads();  // every read of the last term's buffers is done
#pragma unroll
      for (int k = 0; k < kSplit0Acc; ++k) {
        const int j = tid + k * nth;
        if (j < (1 << log2c)) st(y + j, acc[k]);
      }
      src = y;
    }
    __syncthreads();
    first_pass_scatter<R, false, LS>([&](int k, int b, int) { return ld(src + (k << lpc) + b); }, per, c, S, peer_z,
                                     wi, tid, nth);
    cl.sync();  // every part's z is complete (no peer memory is touched after this)
    const FlatBuf s = dif_after_first<R, false>(log2n, LS, FlatBuf{z}, FlatBuf{x}, wi, tid, nth);
    for (int j = tid; j < (1 << log2c); j += nth) {
      const int jg = (j << LS) + c;
      const c64 t = cmul(ldg(itw + jg), ld(s.p + j));
      __stcs(op + jg, round_half_up_mod64(t.re));
      __stcs(op + jg + n, round_half_up_mod64(t.im));
    }
  } else {
    for (int j = tid; j < (1 << log2c); j += nth) {
      const int jg = (j << LS) + c;
      const c64 v{i64_to_f64_rne((int64_t)__ldcs(ap + jg)), i64_to_f64_rne((int64_t)__ldcs(ap + jg + n))};
      st(x + j, cmul(ldg(tw + jg), v));
    }
    __syncthreads();
    const FlatBuf r = dit_before_last<R, true>(log2n, LS, FlatBuf{x}, FlatBuf{y}, wf, tid, nth);
    double2* peer[S];
#pragma unroll
    for (int j = 0; j < S; ++j) peer[j] = cl.map_shared_rank(r.p, (unsigned)j);
    cl.sync();  // every part's forward passes are done
    // last forward pass, butterflies p = c + b*S: output k (the point k*n/R + p) times
    // the operand, into z[k*per + b]
    for (int b = tid; b < per; b += nth) {
      const int p = c + (b << LS);
      const int lo = p << (LR - LS);
      const double2* twp = wf + (p << LR);
      c64 v[R];
      v[0] = ld(peer[0] + lo);
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = cmul(ldg(twp + k), ld(peer[k & (S - 1)] + lo + (k >> LS)));
      Core<R, true, 0>::run(v);
#pragma unroll
      for (int k = 0; k < R; ++k) st(z + (k << lpc) + b, cmul(ldg(bp + (k << lper) + p), v[k]));
    }
    __syncthreads();
    // the inverse ping-pongs between z and the buffer that no peer reads
    const FlatBuf s = dit_before_last<R, false>(log2n, LS, FlatBuf{z}, FlatBuf{r.p == x ? y : x}, wi, tid, nth);
#pragma unroll
    for (int j = 0; j < S; ++j) peer[j] = cl.map_shared_rank(s.p, (unsigned)j);
    cl.sync();  // every part's inverse passes are done
    for (int p = c * per + tid; p < (c + 1) * per; p += nth) {
      const int lo = p << (LR - LS);
      const double2* twp = wi + (p << LR);
      c64 v[R];
      v[0] = ld(peer[0] + lo);
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = cmul(ldg(twp + k), ld(peer[k & (S - 1)] + lo + (k >> LS)));
      Core<R, false, 0>::run(v);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int jg = (k << lper) + p;
        const c64 t = cmul(ldg(itw + jg), v[k]);
        __stcs(op + jg, round_half_up_mod64(t.re));
        __stcs(op + jg + n, round_half_up_mod64(t.im));
      }
    }
    cl.sync();  // no CTA exits while a peer reads its shared memory
  }
}

// One product per cluster of S = R0 x S1 CTAs when the N/2-point transform has
// exactly one unordered outer level, of radix R0 = 2^LS0 <= 4, over a DIF base of
// m points (e.g. N = 4096 on a 1024-point base: R0 = 2, S1 = 4): for latency, a
// few products then run on up to 8 SMs each, where u64_product_split_kernel
// gives each CTA a whole base transform.  Level 0 splits the transform into R0
// slices of m points; CTA c = s0 * S1 + c1 holds class c1 (mod S1) of slice
// s0, i.e. the slice points j * S1 + c1 after the base's first pass.
//   1. Level 0 forward: CTA c takes the butterflies [c*m/S, (c+1)*m/S),
//      reading its inputs folded and twisted from the product's coefficients;
//      output k (slice slot(k), point i) is stored into the staging buffer y of
//      the CTA of that slice that computes the base's first-pass butterfly
//      i mod (m/R), through distributed shared memory.
//   2. Cluster barrier.  The base's first pass on the slice, 1/S1 of the
//      butterflies per CTA, each output into the part of its class (as in
//      u64_product_split0_kernel).
//   3. Cluster barrier.  The later passes, the pointwise product and the
//      inverse's first pass are local to the class; the inverse's first-pass
//      outputs go to the parts of their classes (buffer z).
//   4. Cluster barrier.  The rest of the base inverse, locally.
//   5. Cluster barrier.  Level 0 inverse: CTA c takes the butterflies
//      [c*m/S, (c+1)*m/S), reading point i of every slice from the CTA that
//      holds its class, and untwists, rounds and stores the outputs; a last
//      cluster barrier keeps every CTA alive while a peer reads its memory.
// Every butterfly and elementwise step does the operations of the one-CTA
// product kernel on the same values, so results are bit-identical to it.
// SUM: one output is the Fourier-domain sum of `terms` products (steps 1-3 per
// term, added into a register accumulator in term order, then one inverse).
// Shared memory: three buffers of m/S1 points.  Requires L.nlevels == 1,
// 2^L.log2r[0] == R0, S1 <= the base radix R, m >= R*S1 and, for SUM,
// m/S1 <= kSplit0Acc x blockDim.x.
template <int ALGO, int LS0, int LS1, bool SUM>
__global__ void __launch_bounds__(256) u64_product_split2_kernel(
    const uint64_t* __restrict__ a, const double2* __restrict__ bhat, long bhat_stride, uint64_t* __restrict__ out,
    int terms, const cfft_product_item* __restrict__ items, DevLevels L, const double2* __restrict__ w,
    const double2* __restrict__ winv, const double2* __restrict__ tw, const double2* __restrict__ itw) {
  constexpr int R = AlgoInfo<ALGO>::R;
  constexpr int LR = Log2<R>::v;
  constexpr int R0 = 1 << LS0;
  constexpr int S1 = 1 << LS1;
  constexpr int LS = LS0 + LS1;
  constexpr int S = 1 << LS;
  static_assert(!AlgoInfo<ALGO>::DIT, "DIF base algorithms only");
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double2 smem[];
  const int log2n = L.log2n[0];
  const int log2m = L.log2n[1];
  const int n = 1 << log2n, m = 1 << log2m;
  const int log2c = log2m - LS1;  // points per CTA
  const int c = (int)(blockIdx.x & (S - 1));
  const long g = (long)(blockIdx.x >> LS);
  const int s0 = c >> LS1, c1 = c & (S1 - 1);
  double2* x = smem;
  double2* y = smem + (1 << log2c);
  double2* z = smem + (2 << log2c);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lq = log2m - LR;  // log2(m/R): the base's first-pass stride
  const int lpp = lq - LS1;   // log2 of the first-pass butterflies per CTA
  const int pp = 1 << lpp;
  const uint64_t* ap = items ? items[g].a : a + (g << (log2n + 1));
  const double2* bp = items ? (const double2*)items[g].bhat : bhat + g * bhat_stride;
  uint64_t* op = items ? items[g].out : out + (g << (log2n + 1));
  const double2* wl = w + L.w_off[0];
  const double2* wli = winv + L.winv_off[0];
  const double2* wf = w + L.w_off[1] + m;  // the base's forward and inverse tables
  const double2* wi = winv + m;
  double2* peer_x[S1];
  double2* peer_z[S1];
#pragma unroll
  for (int j = 0; j < S1; ++j) {
    peer_x[j] = cl.map_shared_rank(x, (unsigned)((s0 << LS1) + j));
    peer_z[j] = cl.map_shared_rank(z, (unsigned)((s0 << LS1) + j));
  }
  const int cnt = m >> LS;
  const int i0 = c * cnt;
  // SUM: a sum of `terms` products (terms of an output consecutive in a and bhat,
  // bhat at stride bhat_stride), steps 1-3 per term, each product added into a
  // register accumulator in term order, one inverse.  Otherwise one product.
  c64 acc[SUM ? kSplit0Acc : 1];
  const double2* src = nullptr;  // input of the inverse's first pass
  const int nterms = SUM ? terms : 1;
#pragma unroll 1
  for (int t = 0; t < nterms; ++t) {
  const long term = g * nterms + t;
  const uint64_t* tap = SUM ? a + (term << (log2n + 1)) : ap;
  const double2* tbp = SUM ? bhat + term * bhat_stride : bp;
  // every CTA runs, and is done with its buffers of the previous term, before a
  // peer writes them
  auto token = cl.barrier_arrive();

  // 1. level 0 forward on butterflies [c*m/S, (c+1)*m/S)
  auto load_l0 = [&](int i, c64* v) {
#pragma unroll
    for (int k = 0; k < R0; ++k) {
      const int j = (k << log2m) + i;
      const c64 u{i64_to_f64_rne((int64_t)__ldcs(tap + j)), i64_to_f64_rne((int64_t)__ldcs(tap + j + n))};
      v[k] = cmul(ldg(tw + j), u);
    }
  };
  c64 v0[R0];
  if (tid < cnt) load_l0(i0 + tid, v0);
  cl.barrier_wait(std::move(token));
  for (int b = tid; b < cnt; b += nth) {
    const int i = i0 + b;
    c64 v[R0];
    if (b == tid) {
#pragma unroll
      for (int k = 0; k < R0; ++k) v[k] = v0[k];
    } else {
      load_l0(i, v);
    }
    Core<R0, true, 0>::run(v);
    const double2* twl = wl + (R0 - 1) * i - 1;
    const int p = i & ((1 << lq) - 1);
    const int dst = (((i >> lq) << lpp) + (p & (pp - 1)));
    const int cls = p >> lpp;
#pragma unroll
    for (int k = 0; k < R0; ++k) {
      const c64 o = k == 0 ? v[0] : cmul(ldg(twl + k), v[k]);
      st(cl.map_shared_rank(y, (unsigned)((slot<R0>(k) << LS1) + cls)) + dst, o);
    }
  }
  cl.sync();  // every staging buffer is complete

  // 2. the base's first pass on this slice, butterflies [c1*pp, (c1+1)*pp)
  first_pass_scatter<R, true, LS1>([&](int k, int b, int) { return ld(y + (k << lpp) + b); }, pp, c1 * pp, 1, peer_x,
                                   wf, tid, nth);
  cl.sync();  // every part's x is complete

  // 3. the later passes, the pointwise product, the inverse's first pass
  const FlatBuf r = dif_after_first<R, true>(log2m, LS1, FlatBuf{x}, FlatBuf{y}, wf, tid, nth);
  const double2* bs = tbp + ((long)s0 << log2m) + c1;
  if constexpr (!SUM) {
    for (int j = tid; j < (1 << log2c); j += nth) st(r.p + j, cmul(ldg(bs + (j << LS1)), ld(r.p + j)));
    src = r.p;
  } else {
#pragma unroll
    for (int k = 0; k < kSplit0Acc; ++k) {
      const int j = tid + k * nth;
      if (j < (1 << log2c)) {
        const c64 p = cmul(ldg(bs + (j << LS1)), ld(r.p + j));
        acc[k] = t == 0 ? p : cadd(acc[k], p);
      }
    }
  }
  }
  if constexpr (SUM) {
    __syncthreads();  // every read of the last term's buffers is done
#pragma unroll
    for (int k = 0; k < kSplit0Acc; ++k) {
      const int j = tid + k * nth;
      if (j < (1 << log2c)) st(y + j, acc[k]);
    }
    src = y;
  }
  __syncthreads();
  first_pass_scatter<R, false, LS1>([&](int k, int b, int) { return ld(src + (k << lpp) + b); }, pp, c1, S1, peer_z,
                                    wi, tid, nth);
  cl.sync();  // every part's z is complete

  // 4. the rest of the base inverse
  const FlatBuf sv = dif_after_first<R, false>(log2m, LS1, FlatBuf{z}, FlatBuf{x}, wi, tid, nth);
  cl.sync();  // every slice's inverse is complete

  // 5. level 0 inverse on butterflies [c*m/S, (c+1)*m/S), untwisted and rounded
  for (int b = tid; b < cnt; b += nth) {
    const int i = i0 + b;
    const int cls = i & (S1 - 1);
    const int at = i >> LS1;
    const double2* twl = wli + (R0 - 1) * i - 1;
    c64 v[R0];
    v[0] = ld(cl.map_shared_rank(sv.p, (unsigned)cls) + at);
#pragma unroll
    for (int k = 1; k < R0; ++k)
      v[k] = cmul(ldg(twl + k), ld(cl.map_shared_rank(sv.p, (unsigned)((slot<R0>(k) << LS1) + cls)) + at));
    Core<R0, false, 0>::run(v);
#pragma unroll
    for (int k = 0; k < R0; ++k) {
      const int j = (k << log2m) + i;
      const c64 t = cmul(ldg(itw + j), v[k]);
      __stcs(op + j, round_half_up_mod64(t.re));
      __stcs(op + j + n, round_half_up_mod64(t.im));
    }
  }
  cl.sync();  // no CTA exits while a peer reads its shared memory
}

// kernel pointers by base algorithm (kinst_split_prod_*.cu, one unit per pair)
// (big: the 512-thread variant, for parts of 4096 points)
const void* u64_product_split_ptr_01(int algo, int ls, bool big);
const void* u64_product_split_ptr_23(int algo, int ls, bool big);
const void* u64_product_split_ptr_45(int algo, int ls, bool big);
const void* u64_product_split_ptr_67(int algo, int ls, bool big);
inline const void* u64_product_split_ptr(int algo, int ls, bool big) {
  return algo < 2 ? u64_product_split_ptr_01(algo, ls, big)
                  : algo < 4 ? u64_product_split_ptr_23(algo, ls, big)
                             : algo < 6 ? u64_product_split_ptr_45(algo, ls, big) : u64_product_split_ptr_67(algo, ls, big);
}
// the kernel for plans without an outer level (sum: its Fourier-domain sum
// variant); nullptr where S = 2^ls exceeds the radix, or a sum on a DIT base
const void* u64_product_split0_ptr_01(int algo, int ls, bool sum);
const void* u64_product_split0_ptr_23(int algo, int ls, bool sum);
const void* u64_product_split0_ptr_45(int algo, int ls, bool sum);
const void* u64_product_split0_ptr_67(int algo, int ls, bool sum);
// the one-level kernel (DIF bases only; sum: its Fourier-domain sum variant);
// nullptr where the shape is not instantiated
const void* u64_product_split2_ptr_01(int algo, int ls0, int ls1, bool sum);
const void* u64_product_split2_ptr_23(int algo, int ls0, int ls1, bool sum);
const void* u64_product_split2_ptr_45(int algo, int ls0, int ls1, bool sum);
const void* u64_product_split2_ptr_67(int algo, int ls0, int ls1, bool sum);
inline const void* u64_product_split2_ptr(int algo, int ls0, int ls1, bool sum) {
  return algo < 2 ? u64_product_split2_ptr_01(algo, ls0, ls1, sum)
                  : algo < 4 ? u64_product_split2_ptr_23(algo, ls0, ls1, sum)
                             : algo < 6 ? u64_product_split2_ptr_45(algo, ls0, ls1, sum)
                                        : u64_product_split2_ptr_67(algo, ls0, ls1, sum);
}
inline const void* u64_product_split0_ptr(int algo, int ls, bool sum) {
  return algo < 2 ? u64_product_split0_ptr_01(algo, ls, sum)
                  : algo < 4 ? u64_product_split0_ptr_23(algo, ls, sum)
                             : algo < 6 ? u64_product_split0_ptr_45(algo, ls, sum)
                                        : u64_product_split0_ptr_67(algo, ls, sum);
}

template <int A>
const void* split_product_ptr(int ls, bool big) {
  if (big) {
    switch (ls) {
      case 1: return (const void*)u64_product_split_kernel<A, 1, kSplitProdThreadsBig>;
      case 2: return (const void*)u64_product_split_kernel<A, 2, kSplitProdThreadsBig>;
      case 3: return (const void*)u64_product_split_kernel<A, 3, kSplitProdThreadsBig>;
      default: return nullptr;
    }
  }
  switch (ls) {
    case 1: return (const void*)u64_product_split_kernel<A, 1, kSplitProdThreads>;
    case 2: return (const void*)u64_product_split_kernel<A, 2, kSplitProdThreads>;
    case 3: return (const void*)u64_product_split_kernel<A, 3, kSplitProdThreads>;
    default: return nullptr;
  }
}

template <int A, bool SUM>
const void* split0_product_ptr_t(int ls) {
  constexpr int LRA = Log2<AlgoInfo<A>::R>::v;
  switch (ls) {
    case 1: return (const void*)u64_product_split0_kernel<A, 1, SUM>;
    case 2: if constexpr (LRA >= 2) return (const void*)u64_product_split0_kernel<A, 2, SUM>; else return nullptr;
    case 3: if constexpr (LRA >= 3) return (const void*)u64_product_split0_kernel<A, 3, SUM>; else return nullptr;
    default: return nullptr;
  }
}
// sum: the Fourier-domain sum variant (DIF bases only)
template <int A>
const void* split0_product_ptr(int ls, bool sum) {
  if (!sum) return split0_product_ptr_t<A, false>(ls);
  if constexpr (AlgoInfo<A>::DIT) return nullptr;
  else return split0_product_ptr_t<A, true>(ls);
}

// (R0, S1) = (2, 2), (2, 4), (4, 2) for DIF bases with S1 <= R
template <int A, bool SUM>
const void* split2_product_ptr_t(int ls0, int ls1) {
  if constexpr (AlgoInfo<A>::DIT) {
    return nullptr;
  } else {
    constexpr int LRA = Log2<AlgoInfo<A>::R>::v;
    if (ls0 == 1 && ls1 == 1) return (const void*)u64_product_split2_kernel<A, 1, 1, SUM>;
    if (ls0 == 2 && ls1 == 1) return (const void*)u64_product_split2_kernel<A, 2, 1, SUM>;
    if constexpr (LRA >= 2) {
      if (ls0 == 1 && ls1 == 2) return (const void*)u64_product_split2_kernel<A, 1, 2, SUM>;
      // 16-CTA clusters
      if (ls0 == 2 && ls1 == 2) return (const void*)u64_product_split2_kernel<A, 2, 2, SUM>;
      if (ls0 == 3 && ls1 == 1) return (const void*)u64_product_split2_kernel<A, 3, 1, SUM>;
    }
    return nullptr;
  }
}
// sum: the Fourier-domain sum variant
template <int A>
const void* split2_product_ptr(int ls0, int ls1, bool sum) {
  return sum ? split2_product_ptr_t<A, true>(ls0, ls1) : split2_product_ptr_t<A, false>(ls0, ls1);
}

}  // namespace cfft
