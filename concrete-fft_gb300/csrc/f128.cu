// f128.cu -- fft128::Plan (double-double negacyclic FFT) and the u128 product.
//
// A transform of up to 4096 points (32 bytes each in split re0/re1/im0/im1
// form) is held by one CTA in shared memory and runs every radix-2 stage
// there, in place, one barrier per stage.  Larger transforms run their widest
// stages in global memory (forward: first, inverse: last) until the remaining
// blocks fit a CTA.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "cfft_internal.h"
#include "f128_device.cuh"
#include "runtime.h"

using namespace cfft;

namespace cfft {

constexpr int kF128SmemLog2 = 12;  // 4096 points x 32 B = 128 KiB
constexpr int kF128BlockLog2Auto = 9;

// Blocks of 2^log2c points; 2^log2t consecutive blocks per CTA iteration (whole
// transforms of fewer than 128 points are packed so that a stage's butterflies
// fill whole warps: a group of threads per block, every group through the same
// barriers).
template <bool FWD>
__global__ void __launch_bounds__(256) f128_smem_kernel(F128Arrays g, int log2n, int log2c, long nblocks, F128Tw tw,
                                                        int log2t) {
  extern __shared__ double sm[];
  const int c = 1 << log2c;
  const int tc = c << log2t;  // points per CTA iteration
  F128Arrays s{sm, sm + tc, sm + 2 * tc, sm + 3 * tc};
  const int tid = threadIdx.x, nth = blockDim.x;
  const int gsize = nth >> log2t;  // threads per block
  const int grp = tid / gsize, gtid = tid - grp * gsize;
  const long per_transform = 1L << (log2n - log2c);
  const long total = nblocks << log2c;
  grid_dependency_wait();
  for (long first = (long)blockIdx.x << log2t; first < nblocks; first += (long)gridDim.x << log2t) {
    const long off = first << log2c;
    for (int i = tid; i < tc; i += nth) {
      if (off + i >= total) break;
      s.re0[i] = g.re0[off + i];
      s.re1[i] = g.re1[off + i];
      s.im0[i] = g.im0[off + i];
      s.im1[i] = g.im1[off + i];
    }
    __syncthreads();
    const long sb = (first + grp) % per_transform;  // sub-block index inside its transform
    const F128Arrays sg{s.re0 + grp * c, s.re1 + grp * c, s.im0 + grp * c, s.im1 + grp * c};
    f128_stages_smem<FWD>(sg, log2n, log2c, sb, tw, gtid, gsize);  // past the batch's end: unused values
    for (int i = tid; i < tc; i += nth) {
      if (off + i >= total) break;
      g.re0[off + i] = s.re0[i];
      g.re1[off + i] = s.re1[i];
      g.im0[off + i] = s.im0[i];
      g.im1[off + i] = s.im1[i];
    }
    __syncthreads();
  }
}

// Cluster layouts of one transform of 2^log2n points over S = 2^LS CTAs: a
// stage of half-size t >= S pairs points of one residue class mod S, a stage
// of t < S points of one block of n/S.  CTA c holds class c (the points
// j*S + c, compacted to j) in A for the wide stages and block c (the points
// c*n/S ..) in B for the narrow ones; two warps per 32 butterflies
// (f128_half_stage).  The butterflies and twiddles are those of the one-CTA
// kernel, so the results are bit-identical.
template <bool FWD, int LS>
__device__ __forceinline__ void f128_wide_stage(const F128Arrays& A, double* xs, int log2n, int c, int log2t,
                                                const F128Tw& tw, int tid, int nth) {
  const int lt = log2t - LS;
  const long m = 1L << (log2n - 1 - log2t);
  f128_half_stage<FWD>(A, xs, 1 << (log2n - LS - 1), [&](int b, int& qa, int& qb, long& widx) {
    qa = ((b >> lt) << (lt + 1)) + (b & ((1 << lt) - 1));
    qb = qa + (1 << lt);
    widx = m + ((((long)qa << LS) + c) >> (log2t + 1));
  }, tw, tid, nth);
}
template <bool FWD, int LS>
__device__ __forceinline__ void f128_narrow_stage(const F128Arrays& B, double* xs, int log2n, int c, int log2t,
                                                  const F128Tw& tw, int tid, int nth) {
  const int lnp = log2n - LS;
  const long m = 1L << (log2n - 1 - log2t);
  f128_half_stage<FWD>(B, xs, 1 << (lnp - 1), [&](int b, int& qa, int& qb, long& widx) {
    qa = ((b >> log2t) << (log2t + 1)) + (b & ((1 << log2t) - 1));
    qb = qa + (1 << log2t);
    widx = m + ((((long)c << lnp) + qa) >> (log2t + 1));
  }, tw, tid, nth);
}
// class c (A) -> the blocks (B) of the cluster, through distributed shared memory
template <int LS, class Cluster>
__device__ __forceinline__ void f128_classes_to_blocks(Cluster& cl, const F128Arrays& A, const F128Arrays& B, int lnp,
                                                       int c, int tid, int nth) {
  for (int q = tid; q < (1 << lnp); q += nth) {
    const int p = (q << LS) + c;
    const unsigned o = (unsigned)(p >> lnp);
    const int at = p & ((1 << lnp) - 1);
    cl.map_shared_rank(B.re0, o)[at] = A.re0[q];
    cl.map_shared_rank(B.re1, o)[at] = A.re1[q];
    cl.map_shared_rank(B.im0, o)[at] = A.im0[q];
    cl.map_shared_rank(B.im1, o)[at] = A.im1[q];
  }
}
// block c (B) -> the classes (A) of the cluster
template <int LS, class Cluster>
__device__ __forceinline__ void f128_blocks_to_classes(Cluster& cl, const F128Arrays& A, const F128Arrays& B, int lnp,
                                                       int c, int tid, int nth) {
  for (int q = tid; q < (1 << lnp); q += nth) {
    const int p = (c << lnp) + q;
    const unsigned o = (unsigned)(p & ((1 << LS) - 1));
    const int at = p >> LS;
    cl.map_shared_rank(A.re0, o)[at] = B.re0[q];
    cl.map_shared_rank(A.re1, o)[at] = B.re1[q];
    cl.map_shared_rank(A.im0, o)[at] = B.im0[q];
    cl.map_shared_rank(A.im1, o)[at] = B.im1[q];
  }
}

// One transform of 2^log2n points (64 <= n <= 4096) per cluster of S = 2^LS CTAs,
// for small batches (S SMs per transform).  Forward: t = n/2 .. 1 (wide stages,
// exchange, narrow stages); inverse: t = 1 .. n/2 (narrow, exchange, wide).
// Shared memory: A and B of n/S points each, and the exchange of the inverse's
// differences.
template <bool FWD, int LS>
__global__ void __launch_bounds__(256) f128_cluster_kernel(F128Arrays g, int log2n, F128Tw tw) {
  constexpr int S = 1 << LS;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double sm[];
  grid_dependency_wait();
  const int lnp = log2n - LS;  // points per CTA
  const int np = 1 << lnp;
  const int c = (int)(blockIdx.x & (S - 1));
  const long base = (long)(blockIdx.x >> LS) << log2n;
  const int tid = threadIdx.x, nth = blockDim.x;
  const F128Arrays A{sm, sm + np, sm + 2 * np, sm + 3 * np};
  const F128Arrays B{sm + 4 * np, sm + 5 * np, sm + 6 * np, sm + 7 * np};
  double* xs = sm + 8 * np;
  auto token = cl.barrier_arrive();  // every CTA runs before a peer's memory is written
  if constexpr (FWD) {
    for (int q = tid; q < np; q += nth) {
      const long p = base + ((long)q << LS) + c;
      A.re0[q] = g.re0[p];
      A.re1[q] = g.re1[p];
      A.im0[q] = g.im0[p];
      A.im1[q] = g.im1[p];
    }
    __syncthreads();
    for (int lt = log2n - 1; lt >= LS; --lt) f128_wide_stage<true, LS>(A, xs, log2n, c, lt, tw, tid, nth);
    cl.barrier_wait(std::move(token));
    f128_classes_to_blocks<LS>(cl, A, B, lnp, c, tid, nth);
    cl.sync();  // every block is complete (no peer memory is touched after this)
    for (int lt = LS - 1; lt >= 0; --lt) f128_narrow_stage<true, LS>(B, xs, log2n, c, lt, tw, tid, nth);
    for (int q = tid; q < np; q += nth) {
      const long p = base + ((long)c << lnp) + q;
      g.re0[p] = B.re0[q];
      g.re1[p] = B.re1[q];
      g.im0[p] = B.im0[q];
      g.im1[p] = B.im1[q];
    }
  } else {
    for (int q = tid; q < np; q += nth) {
      const long p = base + ((long)c << lnp) + q;
      B.re0[q] = g.re0[p];
      B.re1[q] = g.re1[p];
      B.im0[q] = g.im0[p];
      B.im1[q] = g.im1[p];
    }
    __syncthreads();
    for (int lt = 0; lt < LS; ++lt) f128_narrow_stage<false, LS>(B, xs, log2n, c, lt, tw, tid, nth);
    cl.barrier_wait(std::move(token));
    f128_blocks_to_classes<LS>(cl, A, B, lnp, c, tid, nth);
    cl.sync();  // every class is complete
    for (int lt = LS; lt <= log2n - 1; ++lt) f128_wide_stage<false, LS>(A, xs, log2n, c, lt, tw, tid, nth);
    for (int q = tid; q < np; q += nth) {
      const long p = base + ((long)q << LS) + c;
      g.re0[p] = A.re0[q];
      g.re1[p] = A.re1[q];
      g.im0[p] = A.im0[q];
      g.im1[p] = A.im1[q];
    }
  }
}

// One stage (half-size 2^log2t) over every transform of the batch, in global memory.
template <bool FWD>
__global__ void __launch_bounds__(256) f128_stage_kernel(F128Arrays g, int log2n, int log2t, long total, F128Tw tw) {
  const long m = 1L << (log2n - 1 - log2t);
  grid_dependency_wait();
  for (long b = (long)blockIdx.x * blockDim.x + threadIdx.x; b < total; b += (long)gridDim.x * blockDim.x) {
    const long tr = b >> (log2n - 1);                 // transform index
    const long bb = b & ((1L << (log2n - 1)) - 1);    // butterfly within transform
    const long i = bb >> log2t;
    const long j = (tr << log2n) + (i << (log2t + 1)) + (bb & ((1L << log2t) - 1));
    if (FWD) f128_fwd_bfly(g, j, 1L << log2t, tw, m + i);
    else f128_inv_bfly(g, j, 1L << log2t, tw, m + i);
  }
}

// Small batches: one stage over every transform of the batch in global memory with
// two warps per 32 butterflies (real and imaginary halves, f128_half_stage), 32
// butterflies per 64-thread CTA, so that a stage of a few thousand butterflies
// keeps twice as many SM sub-partitions' FP64 pipes busy as one thread per
// butterfly.  The butterflies and twiddles of f128_stage_kernel; total < 2^31
// points in the batch.
template <bool FWD>
__global__ void __launch_bounds__(64) f128_half_stage_kernel(F128Arrays g, int log2n, int log2t, long total,
                                                             F128Tw tw) {
  __shared__ double xs[128];  // the inverse's differences: 4 doubles per butterfly
  const long m = 1L << (log2n - 1 - log2t);
  const long first = (long)blockIdx.x * 32;
  const int nb = (int)(total - first < 32 ? total - first : 32);
  grid_dependency_wait();
  f128_half_stage<FWD>(g, xs, nb, [&](int b, int& qa, int& qb, long& widx) {
    const long gb = first + b;
    const long tr = gb >> (log2n - 1);               // transform index
    const long bb = gb & ((1L << (log2n - 1)) - 1);  // butterfly within transform
    const long i = bb >> log2t;
    const long j = (tr << log2n) + (i << (log2t + 1)) + (bb & ((1L << log2t) - 1));
    qa = (int)j;
    qb = (int)(j + (1L << log2t));
    widx = m + i;
  }, tw, threadIdx.x, 64);
}

// Small batches: the stages of one sub-block of 2^log2c points (log2c <= 8) per CTA
// in shared memory, two warps per 32 butterflies (f128_half_stage); the
// butterflies and twiddles of f128_stages_smem.  2^log2c threads per CTA.
template <bool FWD>
__global__ void __launch_bounds__(256) f128_smem_half_kernel(F128Arrays g, int log2n, int log2c, F128Tw tw) {
  __shared__ double sm[4 * 256 + 2 * 256];
  const int c = 1 << log2c;
  const F128Arrays s{sm, sm + c, sm + 2 * c, sm + 3 * c};
  double* xs = sm + 4 * c;
  const int tid = threadIdx.x, nth = blockDim.x;
  const long off = (long)blockIdx.x << log2c;
  const long sb = (long)blockIdx.x & ((1L << (log2n - log2c)) - 1);  // sub-block inside its transform
  grid_dependency_wait();
  for (int i = tid; i < c; i += nth) {
    s.re0[i] = g.re0[off + i];
    s.re1[i] = g.re1[off + i];
    s.im0[i] = g.im0[off + i];
    s.im1[i] = g.im1[off + i];
  }
  __syncthreads();
  for (int st = 0; st < log2c; ++st) {
    const int log2t = FWD ? (log2c - 1 - st) : st;
    const long m = 1L << (log2n - 1 - log2t);
    f128_half_stage<FWD>(s, xs, c >> 1, [&](int b, int& qa, int& qb, long& widx) {
      const int il = b >> log2t;
      qa = (il << (log2t + 1)) + (b & ((1 << log2t) - 1));
      qb = qa + (1 << log2t);
      widx = m + (sb << (log2c - 1 - log2t)) + il;
    }, tw, tid, nth);
  }
  for (int i = tid; i < c; i += nth) {
    g.re0[off + i] = s.re0[i];
    g.re1[off + i] = s.re1[i];
    g.im0[off + i] = s.im0[i];
    g.im1[off + i] = s.im1[i];
  }
}

// One u128 coefficient (lo, hi, read as i128) -> f128: hi = the nearest double, lo =
// the nearest double to the remainder (src/fft128/mod.rs:2006-2016 pattern).
__device__ __forceinline__ void u128_to_f128(uint64_t lo, uint64_t hi, double& xh, double& xl) {
  xh = i128_to_f64_rne(lo, hi);
  uint64_t tl, th;
  double fr;
  trunc_mod128(xh, tl, th, fr);
  const uint64_t rl = lo - tl;
  const uint64_t rh = hi - th - (lo < tl ? 1 : 0);
  xl = i128_to_f64_rne(rl, rh);
}

// u128 product: the fft128 pipeline of src/fft128/mod.rs:1998-2058 fused.
// a, out: N coefficients as (lo, hi) u64 pairs; bhat: 4 arrays of n = N/2 f64.
__global__ void __launch_bounds__(256) u128_product_kernel(const uint64_t* __restrict__ a,
                                                          const double* __restrict__ bhat, long bhat_stride,
                                                          uint64_t* __restrict__ out, long count, int log2n,
                                                          F128Tw tw, double factor) {
  extern __shared__ double sm[];
  const int n = 1 << log2n;
  F128Arrays s{sm, sm + n, sm + 2 * n, sm + 3 * n};
  const int tid = threadIdx.x, nth = blockDim.x;
  for (long prod = blockIdx.x; prod < count; prod += gridDim.x) {
    const uint64_t* ap = a + prod * 4L * n;
    for (int j = tid; j < 2 * n; j += nth) {
      // coefficient j -> re (j < n) or im (j >= n) of point j mod n
      double xh, xl;
      u128_to_f128(__ldcs(ap + 2 * j), __ldcs(ap + 2 * j + 1), xh, xl);
      if (j < n) {
        s.re0[j] = xh;
        s.re1[j] = xl;
      } else {
        s.im0[j - n] = xh;
        s.im1[j - n] = xl;
      }
    }
    __syncthreads();
    f128_stages_smem<true>(s, log2n, log2n, 0, tw, tid, nth);
    const double* bp = bhat + prod * bhat_stride;
    for (int k = tid; k < n; k += nth) {
      f128 pr, pi;
      cplx_mul(f128{s.re0[k], s.re1[k]}, f128{s.im0[k], s.im1[k]}, f128{__ldg(bp + k), __ldg(bp + n + k)},
               f128{__ldg(bp + 2 * n + k), __ldg(bp + 3 * n + k)}, pr, pi);
      s.re0[k] = __dmul_rn(pr.hi, factor);
      s.re1[k] = __dmul_rn(pr.lo, factor);
      s.im0[k] = __dmul_rn(pi.hi, factor);
      s.im1[k] = __dmul_rn(pi.lo, factor);
    }
    __syncthreads();
    f128_stages_smem<false>(s, log2n, log2n, 0, tw, tid, nth);
    uint64_t* op = out + prod * 4L * n;
    for (int j = tid; j < 2 * n; j += nth) {
      uint64_t rl, rh;
      if (j < n) round_half_up_mod128(s.re0[j], s.re1[j], rl, rh);
      else round_half_up_mod128(s.im0[j - n], s.im1[j - n], rl, rh);
      __stcs(op + 2 * j, rl);
      __stcs(op + 2 * j + 1, rh);
    }
    __syncthreads();
  }
}

// One u128 product of N = 2n coefficients (64 <= n <= 1024) per cluster of S = 2^LS
// CTAs, for a few products: the steps of u128_product_kernel on the cluster
// layouts of f128_cluster_kernel.  CTA c folds the coefficients of class c into
// A, runs the wide forward stages, sends its class to the blocks, runs the
// narrow forward stages, the pointwise product (the operand at the block's
// points) and the narrow inverse stages on its block, sends the block to the
// classes, runs the wide inverse stages and rounds class c.  The same operations
// on the same values as the one-CTA kernel, so the results are bit-identical.
template <int LS>
__global__ void __launch_bounds__(256) u128_product_cluster_kernel(const uint64_t* __restrict__ a,
                                                                  const double* __restrict__ bhat, long bhat_stride,
                                                                  uint64_t* __restrict__ out, int log2n, F128Tw tw,
                                                                  double factor) {
  constexpr int S = 1 << LS;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double sm[];
  const int lnp = log2n - LS;
  const int np = 1 << lnp;
  const int n = 1 << log2n;
  const int c = (int)(blockIdx.x & (S - 1));
  const long prod = (long)(blockIdx.x >> LS);
  const int tid = threadIdx.x, nth = blockDim.x;
  const F128Arrays A{sm, sm + np, sm + 2 * np, sm + 3 * np};
  const F128Arrays B{sm + 4 * np, sm + 5 * np, sm + 6 * np, sm + 7 * np};
  double* xs = sm + 8 * np;
  const uint64_t* ap = a + prod * 4L * n;
  auto token = cl.barrier_arrive();  // every CTA runs before a peer's memory is written
  // coefficient p of class c -> re of point p, coefficient p + n -> im of point p
  for (int t = tid; t < 2 * np; t += nth) {
    const int q = t & (np - 1);
    const int j = ((q << LS) + c) + (t >= np ? n : 0);
    double xh, xl;
    u128_to_f128(__ldcs(ap + 2 * j), __ldcs(ap + 2 * j + 1), xh, xl);
    if (t < np) {
      A.re0[q] = xh;
      A.re1[q] = xl;
    } else {
      A.im0[q] = xh;
      A.im1[q] = xl;
    }
  }
  __syncthreads();
  for (int lt = log2n - 1; lt >= LS; --lt) f128_wide_stage<true, LS>(A, xs, log2n, c, lt, tw, tid, nth);
  cl.barrier_wait(std::move(token));
  f128_classes_to_blocks<LS>(cl, A, B, lnp, c, tid, nth);
  cl.sync();  // every block is complete; every CTA is done with its class copy
  for (int lt = LS - 1; lt >= 0; --lt) f128_narrow_stage<true, LS>(B, xs, log2n, c, lt, tw, tid, nth);
  const double* bp = bhat + prod * bhat_stride + ((long)c << lnp);
  for (int q = tid; q < np; q += nth) {
    f128 pr, pi;
    cplx_mul(f128{B.re0[q], B.re1[q]}, f128{B.im0[q], B.im1[q]}, f128{__ldg(bp + q), __ldg(bp + n + q)},
             f128{__ldg(bp + 2 * n + q), __ldg(bp + 3 * n + q)}, pr, pi);
    B.re0[q] = __dmul_rn(pr.hi, factor);
    B.re1[q] = __dmul_rn(pr.lo, factor);
    B.im0[q] = __dmul_rn(pi.hi, factor);
    B.im1[q] = __dmul_rn(pi.lo, factor);
  }
  __syncthreads();
  for (int lt = 0; lt < LS; ++lt) f128_narrow_stage<false, LS>(B, xs, log2n, c, lt, tw, tid, nth);
  f128_blocks_to_classes<LS>(cl, A, B, lnp, c, tid, nth);
  cl.sync();  // every class is complete (no peer memory is touched after this)
  for (int lt = LS; lt <= log2n - 1; ++lt) f128_wide_stage<false, LS>(A, xs, log2n, c, lt, tw, tid, nth);
  uint64_t* op = out + prod * 4L * n;
  for (int t = tid; t < 2 * np; t += nth) {
    const int q = t & (np - 1);
    const int j = ((q << LS) + c) + (t >= np ? n : 0);
    uint64_t rl, rh;
    if (t < np) round_half_up_mod128(A.re0[q], A.re1[q], rl, rh);
    else round_half_up_mod128(A.im0[q], A.im1[q], rl, rh);
    __stcs(op + 2 * j, rl);
    __stcs(op + 2 * j + 1, rh);
  }
}

// Bhat for small digits: f128(b, 0), fold, forward.
__global__ void __launch_bounds__(256) u128_prepare_kernel(const int64_t* __restrict__ b, double* __restrict__ bhat,
                                                          long count, int log2n, F128Tw tw) {
  extern __shared__ double sm[];
  const int n = 1 << log2n;
  F128Arrays s{sm, sm + n, sm + 2 * n, sm + 3 * n};
  const int tid = threadIdx.x, nth = blockDim.x;
  for (long prod = blockIdx.x; prod < count; prod += gridDim.x) {
    const int64_t* bp = b + prod * 2L * n;
    for (int j = tid; j < n; j += nth) {
      s.re0[j] = i64_to_f64_rne(bp[j]);
      s.re1[j] = 0.0;
      s.im0[j] = i64_to_f64_rne(bp[j + n]);
      s.im1[j] = 0.0;
    }
    __syncthreads();
    f128_stages_smem<true>(s, log2n, log2n, 0, tw, tid, nth);
    double* op = bhat + prod * 4L * n;
    for (int k = tid; k < n; k += nth) {
      op[k] = s.re0[k];
      op[n + k] = s.re1[k];
      op[2 * n + k] = s.im0[k];
      op[3 * n + k] = s.im1[k];
    }
    __syncthreads();
  }
}


// ---- u128 products above N = 8192: the same steps as separate kernels around
// the fft128 plan's transform (global stages + shared-memory blocks), on a
// workspace of four arrays of count x n f64 (the plan's batch layout).

// a (N (lo, hi) pairs per product) -> f128 points, as u128_product_kernel does.
__global__ void __launch_bounds__(256) u128_fold_kernel(const uint64_t* __restrict__ a, F128Arrays z, long count,
                                                       int log2n) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  const long total = count << (log2n + 1);
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long p = g >> (log2n + 1), j = g & (2 * n - 1);
    const uint64_t* ap = a + p * 4 * n;
    double xh, xl;
    u128_to_f128(__ldcs(ap + 2 * j), __ldcs(ap + 2 * j + 1), xh, xl);
    if (j < n) {
      z.re0[p * n + j] = xh;
      z.re1[p * n + j] = xl;
    } else {
      z.im0[p * n + j - n] = xh;
      z.im1[p * n + j - n] = xl;
    }
  }
}

// z <- (z * bhat) * factor, the fused kernel's double-double pointwise step.
__global__ void __launch_bounds__(256) u128_pointwise_kernel(F128Arrays z, const double* __restrict__ bhat,
                                                            long bhat_stride, long count, int log2n, double factor) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  const long total = count << log2n;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long p = g >> log2n, k = g & (n - 1);
    const double* bp = bhat + p * bhat_stride;
    f128 pr, pi;
    cplx_mul(f128{z.re0[g], z.re1[g]}, f128{z.im0[g], z.im1[g]}, f128{__ldg(bp + k), __ldg(bp + n + k)},
             f128{__ldg(bp + 2 * n + k), __ldg(bp + 3 * n + k)}, pr, pi);
    z.re0[g] = __dmul_rn(pr.hi, factor);
    z.re1[g] = __dmul_rn(pr.lo, factor);
    z.im0[g] = __dmul_rn(pi.hi, factor);
    z.im1[g] = __dmul_rn(pi.lo, factor);
  }
}

// f128 points -> N (lo, hi) pairs, floor(x + 1/2) mod 2^128.
__global__ void __launch_bounds__(256) u128_round_kernel(F128Arrays z, uint64_t* __restrict__ out, long count,
                                                        int log2n) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  const long total = count << (log2n + 1);
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long p = g >> (log2n + 1), j = g & (2 * n - 1);
    uint64_t rl, rh;
    if (j < n) round_half_up_mod128(z.re0[p * n + j], z.re1[p * n + j], rl, rh);
    else round_half_up_mod128(z.im0[p * n + j - n], z.im1[p * n + j - n], rl, rh);
    __stcs(out + p * 4 * n + 2 * j, rl);
    __stcs(out + p * 4 * n + 2 * j + 1, rh);
  }
}

// digits -> f128(b, 0) points (the operand's fold), and the transformed points
// -> the operand layout (four arrays of n per operand).
__global__ void __launch_bounds__(256) u128_prepare_fold_kernel(const int64_t* __restrict__ b, F128Arrays z,
                                                               long count, int log2n) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  const long total = count << log2n;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long p = g >> log2n, j = g & (n - 1);
    const int64_t* bp = b + p * 2 * n;
    z.re0[g] = i64_to_f64_rne(bp[j]);
    z.re1[g] = 0.0;
    z.im0[g] = i64_to_f64_rne(bp[j + n]);
    z.im1[g] = 0.0;
  }
}
__global__ void __launch_bounds__(256) u128_operand_layout_kernel(F128Arrays z, double* __restrict__ bhat,
                                                                 long count, int log2n) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  const long total = count << log2n;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long p = g >> log2n, k = g & (n - 1);
    double* op = bhat + p * 4 * n;
    op[k] = z.re0[g];
    op[n + k] = z.re1[g];
    op[2 * n + k] = z.im0[g];
    op[3 * n + k] = z.im1[g];
  }
}

}  // namespace cfft

struct cfft_f128_plan {
  size_t n = 0;
  int block_log2 = 0;      // points per shared-memory block as a log2 (0: automatic)
  double* d_tw = nullptr;  // 4 arrays of n
  F128Tw tw() const { return F128Tw{d_tw, d_tw + n, d_tw + 2 * n, d_tw + 3 * n}; }
};

struct cfft_u128_product_plan {
  size_t N = 0;
  cfft_f128_plan f;
};

namespace {

// Raises the fft128 kernels' dynamic shared-memory limit once per device.
std::mutex g_f128_attr_mu;
std::vector<int> g_f128_attr_devices;
cfft_status f128_attrs() {
  int dev = 0;
  CFFT_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_f128_attr_mu);
  for (int d : g_f128_attr_devices)
    if (d == dev) return CFFT_OK;
  const int max_smem = 4 * (1 << kF128SmemLog2) * (int)sizeof(double);
  CFFT_CUDA_TRY(cudaFuncSetAttribute(f128_smem_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  CFFT_CUDA_TRY(cudaFuncSetAttribute(f128_smem_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  CFFT_CUDA_TRY(cudaFuncSetAttribute(u128_product_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  CFFT_CUDA_TRY(cudaFuncSetAttribute(u128_prepare_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  g_f128_attr_devices.push_back(dev);
  return CFFT_OK;
}

cfft_status build_f128(cfft_f128_plan* p, size_t n) {
  cfft_status st = f128_attrs();
  if (st != CFFT_OK) return st;
  p->n = n;
  std::vector<double> tw(4 * n);
  f128_twiddles(n, tw.data(), tw.data() + n, tw.data() + 2 * n, tw.data() + 3 * n);
  return upload(tw.data(), 4 * n, &p->d_tw);
}

// The resident CTAs (13 per SM for N = 1024) stride over the batch.  For
// these small CTAs this measured 5% faster than one CTA per product (0.94 M
// vs 0.89 M products/s at N = 1024, 2048 per launch).
static int product_grid(const void* kernel, int threads, size_t smem, long count) {
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  return (int)std::max<long>(1, std::min<long>(count, (long)sm_count() * std::max(per_sm, 1)));
}


int f128_threads(int log2c) { return std::min(256, std::max(64, (1 << log2c) / 8)); }

// `batch` negacyclic transforms of n points stored back to back in each of
// the four arrays, with the twiddle arrays tw (init_negacyclic_twiddles).
cfft_status run_f128_tw(size_t n, const F128Tw& tw, double* re0, double* re1, double* im0, double* im1, size_t batch,
                        bool fwd, cudaStream_t stream, int block_log2 = 0, bool one_kernel = false) {
  if (!re0 || !re1 || !im0 || !im1) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (batch == 0) return CFFT_OK;
  cfft_status ast = f128_attrs();
  if (ast != CFFT_OK) return ast;
  const int log2n = ilog2(n);
  // a small batch of 64..2048 points: one transform per cluster, two warps per 32
  // butterflies, every CTA on an SM of its own: up to 8 CTAs of 128 points up to 1024
  // points, 16 CTAs (a non-portable cluster size, when such a cluster fits) at 2048.  fwd+inv, one transform: 24.9 us at 64 points (one CTA, a thread per
  // butterfly: 43.6), 42.1 at 512 (75.8), 46.7 at 1024 (85.2), 51.7 at 2048 (93.6 over
  // global stages).  From SMs/2 CTAs on the block path is as fast.  4096 points take
  // the half-butterfly stages below (one forward 51.9 us on a 16-CTA cluster, whose 16
  // SMs' FP64 pipes bind it)
  if (!one_kernel && block_log2 == 0 && log2n >= 6 && log2n <= 11) {
    const int ls = log2n <= 10 ? std::max(0, log2n - 7) : 4;
    static const void* const kfn[2][5] = {
        {(const void*)f128_cluster_kernel<false, 0>, (const void*)f128_cluster_kernel<false, 1>,
         (const void*)f128_cluster_kernel<false, 2>, (const void*)f128_cluster_kernel<false, 3>,
         (const void*)f128_cluster_kernel<false, 4>},
        {(const void*)f128_cluster_kernel<true, 0>, (const void*)f128_cluster_kernel<true, 1>,
         (const void*)f128_cluster_kernel<true, 2>, (const void*)f128_cluster_kernel<true, 3>,
         (const void*)f128_cluster_kernel<true, 4>}};
    const void* fn = kfn[fwd ? 1 : 0][ls];
    const int np = 1 << (log2n - ls);
    const int threads = std::min(256, np);
    const size_t smem = (8 * (size_t)np + 2 * (size_t)threads) * sizeof(double);
    if (((long)batch << ls) <= (long)sm_count() / 2 && (ls <= 3 || cluster_fits(fn, threads, 1 << ls, smem))) {
      const int grid = (int)((long)batch << ls);
      F128Arrays g{re0, re1, im0, im1};
      F128Tw t = tw;
      int ln = log2n;
      void* args[] = {&g, &ln, &t};
      return launch_kernel_cluster(fn, grid, threads, 1 << ls, args, spread_smem(fn, grid, threads, 1 << ls, smem),
                                   stream, true);
    }
  }
  // a small batch of larger transforms (or more transforms than the cluster rule above
  // takes): every stage above 128- or 256-point blocks in global memory, then the
  // blocks in shared memory, one per CTA, all with two warps per 32 butterflies
  // (f128_half_stage_kernel, f128_smem_half_kernel), at most one block per SM
  if (!one_kernel && block_log2 == 0 && log2n >= 8 && ((long)batch << log2n) < (1L << 31)) {
    int log2c = 7;
    while (log2c < 8 && ((long)batch << (log2n - log2c)) > (long)sm_count()) ++log2c;
    if (((long)batch << (log2n - log2c)) <= (long)sm_count()) {
      F128Arrays g{re0, re1, im0, im1};
      F128Tw t = tw;
      int ln = log2n, lc = log2c;
      long total = (long)batch << (log2n - 1);
      const int sgrid = (int)((total + 31) / 32);
      const int bgrid = (int)((long)batch << (log2n - log2c));
      const void* sfn = fwd ? (const void*)f128_half_stage_kernel<true> : (const void*)f128_half_stage_kernel<false>;
      const void* bfn = fwd ? (const void*)f128_smem_half_kernel<true> : (const void*)f128_smem_half_kernel<false>;
      auto stage = [&](int lt) {
        void* args[] = {&g, &ln, &lt, &total, &t};
        return launch_kernel(sfn, sgrid, 64, args, 0, stream, true);
      };
      void* bargs[] = {&g, &ln, &lc, &t};
      cfft_status st = CFFT_OK;
      if (fwd) {
        for (int lt = log2n - 1; lt >= log2c && st == CFFT_OK; --lt) st = stage(lt);
        if (st == CFFT_OK) st = launch_kernel(bfn, bgrid, 1 << log2c, bargs, 0, stream, true);
      } else {
        st = launch_kernel(bfn, bgrid, 1 << log2c, bargs, 0, stream, true);
        for (int lt = log2c; lt <= log2n - 1 && st == CFFT_OK; ++lt) st = stage(lt);
      }
      return st;
    }
  }
  int log2c = std::min(log2n, block_log2 > 0 ? block_log2 : kF128SmemLog2);
  // small batches: smaller shared-memory blocks after more global stages, so that
  // one transform spreads over several SMs (same butterflies, same results)
  const bool few = ((long)batch << (log2n - log2c)) < (long)sm_count() / 2;
  // large batches: 512-point blocks (more CTAs per SM) measured 1-3% faster than
  // 4096 (fwd+inv, 2^22 points per call, n = 1024..16384)
  if (block_log2 == 0 && !few && !one_kernel) log2c = std::min(log2c, kF128BlockLog2Auto);
  while (!one_kernel && log2c > 8 && ((long)batch << (log2n - log2c)) < (long)sm_count() / 2) --log2c;
  F128Arrays g{re0, re1, im0, im1};
  const long nblocks = (long)batch << (log2n - log2c);
  // few blocks: a thread per butterfly of a stage (latency); many: fewer threads, more CTAs per SM
  int threads = few ? std::min(256, 1 << (log2c - 1)) : f128_threads(log2c);
  // whole transforms of fewer than 128 points: 128 points per CTA iteration, 64 threads,
  // one butterfly per thread and stage (n = 32 alone would fill half a warp)
  int log2t = 0;
  if (log2c == log2n && log2c < 7) {
    log2t = 7 - log2c;
    threads = 64;
  }
  const size_t smem = (size_t)4 * (size_t(1) << (log2c + log2t)) * sizeof(double);
  const int grid = product_grid(fwd ? (const void*)f128_smem_kernel<true> : (const void*)f128_smem_kernel<false>,
                                threads, smem, (nblocks + (1L << log2t) - 1) >> log2t);
  const long total = (long)batch << (log2n - 1);
  // global stages: 256-thread CTAs; a stage of fewer butterflies than one such CTA per SM
  // takes 128-thread CTAs, so that its warps land on twice as many SM sub-partitions (a
  // warp issues FP64 on one sub-partition, and one butterfly is ~100 dependent FP64 steps)
  const int sthreads = total < 256L * sm_count() ? 128 : 256;
  const int sgrid = (int)std::min<long>((total + sthreads - 1) / sthreads, (long)sm_count() * 16);
  // programmatic dependent launches: each kernel is launched as the previous one's CTAs exit
  F128Tw t = tw;
  long tot = total, nb = nblocks;
  int ln = log2n, lc = log2c;
  auto stage = [&](int lt) {
    void* args[] = {&g, &ln, &lt, &tot, &t};
    return launch_kernel(fwd ? (const void*)f128_stage_kernel<true> : (const void*)f128_stage_kernel<false>, sgrid,
                         sthreads, args, 0, stream, true);
  };
  void* sargs[] = {&g, &ln, &lc, &nb, &t, &log2t};
  const void* sfn = fwd ? (const void*)f128_smem_kernel<true> : (const void*)f128_smem_kernel<false>;
  cfft_status st = CFFT_OK;
  if (fwd) {
    for (int lt = log2n - 1; lt >= log2c && st == CFFT_OK; --lt) st = stage(lt);
    if (st == CFFT_OK) st = launch_kernel(sfn, grid, threads, sargs, smem, stream, true);
  } else {
    st = launch_kernel(sfn, grid, threads, sargs, smem, stream, true);
    for (int lt = log2c; lt <= log2n - 1 && st == CFFT_OK; ++lt) st = stage(lt);
  }
  return st;
}

int elementwise_grid(long total) {
  return (int)std::max<long>(1, std::min<long>((total + 255) / 256, (long)sm_count() * 16));
}

// Four arrays of count x n f64 from the stream-ordered allocator (no device
// synchronisation; calls on different streams get different blocks).
cfft_status workspace_alloc(size_t count, size_t n, cudaStream_t s, F128Arrays* z) {
  void* ptr = nullptr;
  const size_t per = count * n;
  if (cudaMallocAsync(&ptr, 4 * per * sizeof(double), s) != cudaSuccess)
    return fail(CFFT_ERR_OUT_OF_MEMORY, "u128 product workspace");
  double* d = (double*)ptr;
  *z = F128Arrays{d, d + per, d + 2 * per, d + 3 * per};
  return CFFT_OK;
}

cfft_status run_f128(const cfft_f128_plan* p, double* re0, double* re1, double* im0, double* im1, size_t batch,
                     bool fwd, cudaStream_t stream) {
  if (!p) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_f128_tw(p->n, p->tw(), re0, re1, im0, im1, batch, fwd, stream, p->block_log2);
}

cfft_status run_f128_host(const cfft_f128_plan* p, double* re0, double* re1, double* im0, double* im1, size_t batch,
                          bool fwd) {
  if (!p || !re0 || !re1 || !im0 || !im1) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  const size_t bytes = batch * p->n * sizeof(double);
  void* d;
  cudaStream_t s;
  // page-locked arrays and a transform that one shared-memory block holds: one
  // kernel works on the caller's memory in place, across the host link
  if (ilog2(p->n) <= kF128SmemLog2 && batch > 0) {
    double* m[4] = {(double*)mapped_host_range(re0, bytes), (double*)mapped_host_range(re1, bytes),
                    (double*)mapped_host_range(im0, bytes), (double*)mapped_host_range(im1, bytes)};
    if (m[0] && m[1] && m[2] && m[3]) {
      cfft_status st = host_staging(0, &d, &s);
      if (st != CFFT_OK) return st;
      st = run_f128_tw(p->n, p->tw(), m[0], m[1], m[2], m[3], batch, fwd, s, ilog2(p->n), true);
      if (st != CFFT_OK) return st;
      CFFT_CUDA_TRY(cudaStreamSynchronize(s));
      return CFFT_OK;
    }
  }
  double* hh[4] = {re0, re1, im0, im1};
  // pageable arrays of up to 4 MiB in all: CPU copies into the thread's page-locked
  // bounce buffer and one DMA copy each way (a pageable cudaMemcpy costs ~10 us of
  // driver time, and there would be eight), with the device path in between, which
  // spreads a small batch over many SMs
  if (batch > 0 && 4 * bytes <= kHostBounceMax) {
    void *hb = nullptr, *db = nullptr;
    cfft_status st = host_bounce(4 * bytes, &hb, &db);
    if (st != CFFT_OK) return st;
    st = host_staging(4 * bytes, &d, &s);
    if (st != CFFT_OK) return st;
    for (int i = 0; i < 4; ++i) std::memcpy((char*)hb + i * bytes, hh[i], bytes);
    CFFT_CUDA_TRY(cudaMemcpyAsync(d, hb, 4 * bytes, cudaMemcpyHostToDevice, s));
    double* m[4];
    for (int i = 0; i < 4; ++i) m[i] = (double*)((char*)d + i * bytes);
    st = run_f128(p, m[0], m[1], m[2], m[3], batch, fwd, s);
    if (st != CFFT_OK) return st;
    CFFT_CUDA_TRY(cudaMemcpyAsync(hb, d, 4 * bytes, cudaMemcpyDeviceToHost, s));
    CFFT_CUDA_TRY(cudaStreamSynchronize(s));
    for (int i = 0; i < 4; ++i) std::memcpy(hh[i], (char*)hb + i * bytes, bytes);
    return CFFT_OK;
  }
  cfft_status st = host_staging(4 * bytes, &d, &s);
  if (st != CFFT_OK) return st;
  double* dd[4];
  for (int i = 0; i < 4; ++i) {
    dd[i] = (double*)((char*)d + i * bytes);
    CFFT_CUDA_TRY(cudaMemcpyAsync(dd[i], hh[i], bytes, cudaMemcpyHostToDevice, s));
  }
  st = run_f128(p, dd[0], dd[1], dd[2], dd[3], batch, fwd, s);
  if (st != CFFT_OK) return st;
  for (int i = 0; i < 4; ++i) CFFT_CUDA_TRY(cudaMemcpyAsync(hh[i], dd[i], bytes, cudaMemcpyDeviceToHost, s));
  CFFT_CUDA_TRY(cudaStreamSynchronize(s));
  return CFFT_OK;
}

}  // namespace

extern "C" {

cfft_status cfft_f128_plan_create(size_t n, cfft_f128_plan** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!is_pow2(n) || n < 32) return fail(CFFT_ERR_INVALID_SIZE, "fft128 plan: n must be a power of two >= 32");
  if (ilog2(n) > kF128MaxLog2) return fail(CFFT_ERR_INVALID_SIZE, "fft128 plan: n must be at most 2^24");
  auto* p = new cfft_f128_plan();
  cfft_status st = build_f128(p, n);
  if (st != CFFT_OK) {
    if (p->d_tw) cudaFree(p->d_tw);
    delete p;
    return st;
  }
  *out = p;
  return CFFT_OK;
}

void cfft_f128_plan_destroy(cfft_f128_plan* plan) {
  if (!plan) return;
  if (plan->d_tw) cudaFree(plan->d_tw);
  delete plan;
}
size_t cfft_f128_fft_size(const cfft_f128_plan* plan) { return plan ? plan->n : 0; }

cfft_status cfft_f128_set_block_points(cfft_f128_plan* plan, size_t points) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  if (points != 0 && (!is_pow2(points) || points < 256 || ilog2(points) > kF128SmemLog2))
    return fail(CFFT_ERR_INVALID_ARGUMENT, "block points must be 0 or a power of two in [256, 4096]");
  plan->block_log2 = points == 0 ? 0 : ilog2(points);
  return CFFT_OK;
}
size_t cfft_f128_block_points(const cfft_f128_plan* plan) {
  return plan && plan->block_log2 > 0 ? size_t(1) << plan->block_log2 : 0;
}

cfft_status cfft_f128_fwd(const cfft_f128_plan* p, double* re0, double* re1, double* im0, double* im1, size_t batch,
                          void* stream) {
  return run_f128(p, re0, re1, im0, im1, batch, true, (cudaStream_t)stream);
}
cfft_status cfft_f128_inv(const cfft_f128_plan* p, double* re0, double* re1, double* im0, double* im1, size_t batch,
                          void* stream) {
  return run_f128(p, re0, re1, im0, im1, batch, false, (cudaStream_t)stream);
}
cfft_status cfft_f128_fwd_host(const cfft_f128_plan* p, double* re0, double* re1, double* im0, double* im1,
                               size_t batch) {
  return run_f128_host(p, re0, re1, im0, im1, batch, true);
}
cfft_status cfft_f128_inv_host(const cfft_f128_plan* p, double* re0, double* re1, double* im0, double* im1,
                               size_t batch) {
  return run_f128_host(p, re0, re1, im0, im1, batch, false);
}

cfft_status cfft_f128_init_negacyclic_twiddles(size_t n, double* re0, double* re1, double* im0, double* im1) {
  if (!re0 || !re1 || !im0 || !im1) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (!is_pow2(n) || ilog2(n) > kF128MaxLog2) return fail(CFFT_ERR_INVALID_SIZE, "n must be a power of two <= 2^24");
  if (n < 2) return CFFT_OK;
  std::vector<double> tw(4 * n);
  f128_twiddles(n, tw.data(), tw.data() + n, tw.data() + 2 * n, tw.data() + 3 * n);
  double* dst[4] = {re0, re1, im0, im1};
  for (int k = 0; k < 4; ++k)  // positions 1..n-1, as the reference; position 0 is left as it is
    std::copy(tw.begin() + (long)k * (long)n + 1, tw.begin() + (long)(k + 1) * (long)n, dst[k] + 1);
  return CFFT_OK;
}

static cfft_status raw_f128(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                            const double* t0, const double* t1, const double* t2, const double* t3, bool fwd,
                            void* stream) {
  if (!t0 || !t1 || !t2 || !t3) return fail(CFFT_ERR_INVALID_ARGUMENT, "null twiddle array");
  if (!is_pow2(n) || n < 2 || ilog2(n) > kF128MaxLog2)
    return fail(CFFT_ERR_INVALID_SIZE, "n must be a power of two in [2, 2^24]");
  return run_f128_tw(n, F128Tw{t0, t1, t2, t3}, re0, re1, im0, im1, batch, fwd, (cudaStream_t)stream);
}
cfft_status cfft_f128_negacyclic_fwd(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                     const double* twid_re0, const double* twid_re1, const double* twid_im0,
                                     const double* twid_im1, void* stream) {
  return raw_f128(n, batch, re0, re1, im0, im1, twid_re0, twid_re1, twid_im0, twid_im1, true, stream);
}
cfft_status cfft_f128_negacyclic_inv(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                     const double* twid_re0, const double* twid_re1, const double* twid_im0,
                                     const double* twid_im1, void* stream) {
  return raw_f128(n, batch, re0, re1, im0, im1, twid_re0, twid_re1, twid_im0, twid_im1, false, stream);
}

// The same free functions on host slices (the reference's signatures take
// &mut [f64] / &[f64]): data and twiddles are staged through device memory.
static cfft_status raw_f128_host(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                 const double* t0, const double* t1, const double* t2, const double* t3, bool fwd) {
  if (!re0 || !re1 || !im0 || !im1 || !t0 || !t1 || !t2 || !t3) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (!is_pow2(n) || n < 2 || ilog2(n) > kF128MaxLog2)
    return fail(CFFT_ERR_INVALID_SIZE, "n must be a power of two in [2, 2^24]");
  if (batch == 0) return CFFT_OK;
  const size_t bytes = batch * n * sizeof(double), tw_bytes = n * sizeof(double);
  void* d;
  cudaStream_t s;
  cfft_status st = host_staging(4 * bytes + 4 * tw_bytes, &d, &s);
  if (st != CFFT_OK) return st;
  double* hh[4] = {re0, re1, im0, im1};
  const double* th[4] = {t0, t1, t2, t3};
  double* dd[4];
  double* dt[4];
  for (int i = 0; i < 4; ++i) {
    dd[i] = (double*)((char*)d + i * bytes);
    dt[i] = (double*)((char*)d + 4 * bytes + i * tw_bytes);
    CFFT_CUDA_TRY(cudaMemcpyAsync(dd[i], hh[i], bytes, cudaMemcpyHostToDevice, s));
    CFFT_CUDA_TRY(cudaMemcpyAsync(dt[i], th[i], tw_bytes, cudaMemcpyHostToDevice, s));
  }
  st = run_f128_tw(n, F128Tw{dt[0], dt[1], dt[2], dt[3]}, dd[0], dd[1], dd[2], dd[3], batch, fwd, s);
  if (st != CFFT_OK) return st;
  for (int i = 0; i < 4; ++i) CFFT_CUDA_TRY(cudaMemcpyAsync(hh[i], dd[i], bytes, cudaMemcpyDeviceToHost, s));
  CFFT_CUDA_TRY(cudaStreamSynchronize(s));
  return CFFT_OK;
}
cfft_status cfft_f128_negacyclic_fwd_host(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                          const double* twid_re0, const double* twid_re1, const double* twid_im0,
                                          const double* twid_im1) {
  return raw_f128_host(n, batch, re0, re1, im0, im1, twid_re0, twid_re1, twid_im0, twid_im1, true);
}
cfft_status cfft_f128_negacyclic_inv_host(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                          const double* twid_re0, const double* twid_re1, const double* twid_im0,
                                          const double* twid_im1) {
  return raw_f128_host(n, batch, re0, re1, im0, im1, twid_re0, twid_re1, twid_im0, twid_im1, false);
}

cfft_status cfft_u128_product_plan_create(size_t N, cfft_u128_product_plan** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!is_pow2(N) || N < 64 || ilog2(N) > kF128MaxLog2 + 1)
    return fail(CFFT_ERR_INVALID_SIZE, "u128 product: N must be a power of two in [64, 2^25]");
  auto* p = new cfft_u128_product_plan();
  p->N = N;
  cfft_status st = build_f128(&p->f, N / 2);
  if (st != CFFT_OK) {
    if (p->f.d_tw) cudaFree(p->f.d_tw);
    delete p;
    return st;
  }
  *out = p;
  return CFFT_OK;
}

void cfft_u128_product_plan_destroy(cfft_u128_product_plan* plan) {
  if (!plan) return;
  if (plan->f.d_tw) cudaFree(plan->f.d_tw);
  delete plan;
}
size_t cfft_u128_product_poly_size(const cfft_u128_product_plan* plan) { return plan ? plan->N : 0; }
cfft_f128_plan* cfft_u128_product_fft(cfft_u128_product_plan* plan) { return plan ? &plan->f : nullptr; }

cfft_status cfft_u128_prepare_operand(const cfft_u128_product_plan* p, const int64_t* b, double* bhat4, size_t count,
                                      void* stream) {
  if (!p || !b || !bhat4) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (count == 0) return CFFT_OK;
  if (ilog2(p->f.n) > kF128SmemLog2) {  // fold, the plan's forward transform, operand layout
    cudaStream_t s = (cudaStream_t)stream;
    const int log2n = ilog2(p->f.n);
    F128Arrays z;
    cfft_status st = workspace_alloc(count, p->f.n, s, &z);
    if (st != CFFT_OK) return st;
    const long total = (long)count << log2n;
    CFFT_CUDA_TRY(launch_dependent(u128_prepare_fold_kernel, elementwise_grid(total), 256, 0, s, b, z, (long)count,
                                   log2n));
    st = run_f128_tw(p->f.n, p->f.tw(), z.re0, z.re1, z.im0, z.im1, count, true, s, p->f.block_log2);
    if (st == CFFT_OK) {
      st = launch_dependent(u128_operand_layout_kernel, elementwise_grid(total), 256, 0, s, z, bhat4, (long)count,
                            log2n) == cudaSuccess
               ? CFFT_OK
               : fail(CFFT_ERR_CUDA, "operand layout launch");
    }
    cudaFreeAsync(z.re0, s);
    return st;
  }
  const int log2n = ilog2(p->f.n);
  const int threads = f128_threads(log2n);
  const size_t smem = 4 * p->f.n * sizeof(double);
  const int grid = product_grid((const void*)u128_prepare_kernel, threads, smem, (long)count);
  u128_prepare_kernel<<<grid, threads, smem, (cudaStream_t)stream>>>(b, bhat4, (long)count, log2n, p->f.tw());
  CFFT_CHECK_LAUNCH();
  return CFFT_OK;
}

cfft_status cfft_u128_product(const cfft_u128_product_plan* p, const uint64_t* a, const double* bhat4,
                              size_t bhat_stride, uint64_t* out, size_t count, void* stream) {
  if (!p || !a || !bhat4 || !out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (bhat_stride != 0 && bhat_stride != 2 * p->N)
    return fail(CFFT_ERR_INVALID_ARGUMENT, "bhat_stride must be 0 or 2N");
  if (count == 0) return CFFT_OK;
  const bool few = (long)count < (long)sm_count() / 2;
  // A few products of N = 128..4096: one product per cluster of up to 8 CTAs of 128
  // points, 16 CTAs at N = 4096 (u128_product_cluster_kernel), two warps per 32
  // butterflies.  N = 8192 takes the five launches, whose transforms run the
  // half-butterfly stages over more SMs
  {
    const int log2n = ilog2(p->f.n);
    const int ls = log2n <= 10 ? std::max(0, log2n - 7) : 4;
    static const void* const kfn[5] = {
        (const void*)u128_product_cluster_kernel<0>, (const void*)u128_product_cluster_kernel<1>,
        (const void*)u128_product_cluster_kernel<2>, (const void*)u128_product_cluster_kernel<3>,
        (const void*)u128_product_cluster_kernel<4>};
    const void* fn = kfn[ls];
    const int np = 1 << (log2n - ls);
    const int threads = std::min(256, np);
    const size_t smem = (8 * (size_t)np + 2 * (size_t)threads) * sizeof(double);
    if (log2n >= 6 && log2n <= 11 && ((long)count << ls) <= (long)sm_count() / 2 &&
        (ls <= 3 || cluster_fits(fn, threads, 1 << ls, smem))) {
      const int grid = (int)((long)count << ls);
      long stride = (long)bhat_stride;
      int ln = log2n;
      F128Tw t = p->f.tw();
      double factor = 2.0 / (double)p->N;
      void* args[] = {(void*)&a, (void*)&bhat4, &stride, (void*)&out, &ln, &t, &factor};
      return launch_kernel_cluster(fn, grid, threads, 1 << ls, args, spread_smem(fn, grid, threads, 1 << ls, smem),
                                   (cudaStream_t)stream);
    }
  }
  // Above N = 8192, and for a few products of N >= 1024 (their transforms then spread
  // over many SMs instead of one CTA each): fold, forward, pointwise, inverse, round
  // as five launches around the plan's transform.  Bit-identical to the fused kernel.
  if (ilog2(p->f.n) > kF128SmemLog2 || (few && p->f.n >= 512)) {
    cudaStream_t s = (cudaStream_t)stream;
    const int log2n = ilog2(p->f.n);
    F128Arrays z;
    cfft_status st = workspace_alloc(count, p->f.n, s, &z);
    if (st != CFFT_OK) return st;
    const long total = (long)count << log2n;
    CFFT_CUDA_TRY(launch_dependent(u128_fold_kernel, elementwise_grid(2 * total), 256, 0, s, a, z, (long)count, log2n));
    st = run_f128_tw(p->f.n, p->f.tw(), z.re0, z.re1, z.im0, z.im1, count, true, s, p->f.block_log2);
    if (st == CFFT_OK) {
      st = launch_dependent(u128_pointwise_kernel, elementwise_grid(total), 256, 0, s, z, bhat4, (long)bhat_stride,
                            (long)count, log2n, 2.0 / (double)p->N) == cudaSuccess
               ? CFFT_OK
               : fail(CFFT_ERR_CUDA, "pointwise launch");
    }
    if (st == CFFT_OK)
      st = run_f128_tw(p->f.n, p->f.tw(), z.re0, z.re1, z.im0, z.im1, count, false, s, p->f.block_log2);
    if (st == CFFT_OK) {
      st = launch_dependent(u128_round_kernel, elementwise_grid(2 * total), 256, 0, s, z, out, (long)count, log2n) ==
                   cudaSuccess
               ? CFFT_OK
               : fail(CFFT_ERR_CUDA, "round launch");
    }
    cudaFreeAsync(z.re0, s);
    return st;
  }
  const int log2n = ilog2(p->f.n);
  // few products: a thread per butterfly (latency); many: fewer threads, more CTAs per SM
  const int threads = few ? std::min(256, 1 << (log2n - 1)) : f128_threads(log2n);
  const size_t smem = 4 * p->f.n * sizeof(double);
  const int grid = product_grid((const void*)u128_product_kernel, threads, smem, (long)count);
  u128_product_kernel<<<grid, threads, smem, (cudaStream_t)stream>>>(
      a, bhat4, (long)bhat_stride, out, (long)count, log2n, p->f.tw(), 2.0 / (double)p->N);
  CFFT_CHECK_LAUNCH();
  return CFFT_OK;
}

cfft_status cfft_u128_product_host(const cfft_u128_product_plan* p, const uint64_t* a, const double* bhat4,
                                   size_t bhat_stride, uint64_t* out, size_t count) {
  if (!p || !a || !bhat4 || !out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (bhat_stride != 0 && bhat_stride != 2 * p->N)
    return fail(CFFT_ERR_INVALID_ARGUMENT, "bhat_stride must be 0 or 2N");
  if (count == 0) return CFFT_OK;
  // about 16 chunks on 4 streams, each at least two CTAs per SM
  constexpr int kSlots = 4;
  const size_t poly_bytes = p->N * 2 * sizeof(uint64_t);
  const size_t chunk = std::min(count, std::max((size_t)sm_count() * 2, (count + 15) / 16));
  // page-locked `out`: the kernels store the results there themselves (no copy out)
  uint64_t* mapped_out = (uint64_t*)mapped_host_range(out, count * poly_bytes);
  PipeSlot slot[kSlots];
  cfft_status st = host_pipeline(kSlots, 2 * chunk * poly_bytes, slot);
  if (st != CFFT_OK) return st;
  size_t i = 0;
  for (size_t first = 0; first < count; first += chunk, ++i) {
    const size_t c = std::min(chunk, count - first);
    const PipeSlot& sl = slot[i % kSlots];
    uint64_t* da = (uint64_t*)sl.dev;
    uint64_t* dout = mapped_out ? mapped_out + first * 2 * p->N : da + chunk * 2 * p->N;
    CFFT_CUDA_TRY(cudaMemcpyAsync(da, a + first * 2 * p->N, c * poly_bytes, cudaMemcpyHostToDevice, sl.stream));
    const double* bh = bhat4 + (bhat_stride ? first * bhat_stride : 0);
    st = cfft_u128_product(p, da, bh, bhat_stride, dout, c, sl.stream);
    if (st != CFFT_OK) return st;
    if (!mapped_out)
      CFFT_CUDA_TRY(cudaMemcpyAsync(out + first * 2 * p->N, dout, c * poly_bytes, cudaMemcpyDeviceToHost, sl.stream));
  }
  for (int k = 0; k < kSlots; ++k) CFFT_CUDA_TRY(cudaStreamSynchronize(slot[k].stream));
  return CFFT_OK;
}

}  // extern "C"
