// c64_kernels.cuh -- kernel templates of the c64 transforms and the u64 product.
//
// Each kernel is instantiated per (ordered base algorithm, integer-add level)
// so that it carries exactly one algorithm's code; the instantiations live in
// the kinst_*.cu translation units (compiled in parallel) and are reached
// through the pointer tables declared at the end of this file.
#pragma once
#include "stockham.cuh"

namespace cfft {

// Sub-transforms of 2^log2n_{d0} points, `tpc` per CTA: load to shared memory,
// run the unordered transform from level d0 (ordered plans have no levels),
// store back.
template <int ALGO, int E, bool FWD>
__global__ void __launch_bounds__(256) c64_smem_kernel(double2* data, int count, int tpc, DevLevels L, int d0,
                                                       const double2* __restrict__ w) {
  extern __shared__ double2 smem[];
  grid_dependency_wait();
  const int log2sub = L.log2n[d0];
  const long first = (long)blockIdx.x * tpc;
  const int nch = (int)min((long)tpc, (long)count - first);
  double2* x = smem;
  double2* y = smem + ((long)tpc << log2sub);
  double2* g = data + (first << log2sub);
  const int npts = nch << log2sub;
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int i = tid; i < npts; i += nth) x[i] = g[i];
  __syncthreads();
  const double2* r = unordered_smem<FWD, E, ALGO>(L, d0, nch, x, y, w, tid, nth);
  for (int i = tid; i < npts; i += nth) g[i] = r[i];
}

// Fused negacyclic u64 product (see product_u64.cu for the pipeline): one
// product per CTA at a time, grid-stride over the batch.
template <int ALGO, int E, int THREADS>
__global__ void __launch_bounds__(THREADS) u64_product_kernel(const uint64_t* __restrict__ a,
                                                             const double2* __restrict__ bhat, long bhat_stride,
                                                             uint64_t* __restrict__ out, long count, DevLevels L,
                                                             const double2* __restrict__ w,
                                                             const double2* __restrict__ winv,
                                                             const double2* __restrict__ tw,
                                                             const double2* __restrict__ itw, int log2p) {
  // 2^log2p products per CTA iteration, back to back in shared memory (small N: a pass's
  // butterflies then fill whole warps; the products stay independent, so the bits do not
  // depend on the packing)
  extern __shared__ double2 smem[];
  const int log2n = L.log2n[0];
  const int n = 1 << log2n;
  double2* x = smem;
  double2* y = smem + ((long)n << log2p);
  const int tid = threadIdx.x;
  for (long first = (long)blockIdx.x << log2p; first < count; first += (long)gridDim.x << log2p) {
    const int np = (int)min((long)1 << log2p, count - first);
    const int pts = np << log2n;
    for (int j = tid; j < pts; j += THREADS) {
      const int jj = j & (n - 1);
      const uint64_t* ap = a + ((first + (j >> log2n)) << (log2n + 1));
      const c64 v{i64_to_f64_rne((int64_t)__ldcs(ap + jj)), i64_to_f64_rne((int64_t)__ldcs(ap + jj + n))};
      st(x + j, cmul(ldg(tw + jj), v));
    }
    __syncthreads();
    double2* r = unordered_smem<true, E, ALGO>(L, 0, np, x, y, w, tid, THREADS);
    for (int k = tid; k < pts; k += THREADS) {
      const double2* bp = bhat + (first + (k >> log2n)) * bhat_stride;
      st(r + k, cmul(ldg(bp + (k & (n - 1))), ld(r + k)));
    }
    __syncthreads();
    double2* o = (r == x) ? y : x;
    double2* s = unordered_smem<false, E, ALGO>(L, 0, np, r, o, winv, tid, THREADS);
    for (int j = tid; j < pts; j += THREADS) {
      const int jj = j & (n - 1);
      uint64_t* op = out + ((first + (j >> log2n)) << (log2n + 1));
      const c64 t = cmul(ldg(itw + jj), ld(s + j));
      __stcs(op + jj, round_half_up_mod64(t.re));
      __stcs(op + jj + n, round_half_up_mod64(t.im));
    }
    __syncthreads();
  }
}

// Sum of `terms` products accumulated in the Fourier domain, one inverse per
// group (the TFHE external-product shape): per group, every term is folded,
// twisted and transformed in shared memory, multiplied by its operand and added
// into an accumulator in term order; the accumulator is inverted, untwisted
// and rounded once.  ACC = 0: the accumulator is a third shared buffer (3 x N/2
// c64).  ACC > 0 (N/2 <= ACC x THREADS): each thread keeps the accumulator
// entries k = tid + j x THREADS it multiplies in registers, so shared memory
// is the 2 x N/2 ping-pong pair and more CTAs fit on an SM; the additions and
// their order are the same.
template <int ALGO, int THREADS, int ACC>
__global__ void __launch_bounds__(THREADS) u64_product_sum_kernel(const uint64_t* __restrict__ a,
                                                                 const double2* __restrict__ bhat, int terms,
                                                                 uint64_t* __restrict__ out, long count, DevLevels L,
                                                                 const double2* __restrict__ w,
                                                                 const double2* __restrict__ winv,
                                                                 const double2* __restrict__ tw,
                                                                 const double2* __restrict__ itw) {
  extern __shared__ double2 smem[];
  const int log2n = L.log2n[0];
  const int n = 1 << log2n;
  double2* x = smem;
  double2* y = smem + n;
  double2* acc = smem + 2 * n;  // ACC == 0 only
  c64 racc[ACC > 0 ? ACC : 1];
  const int tid = threadIdx.x;
  for (long g = blockIdx.x; g < count; g += gridDim.x) {
    for (int t = 0; t < terms; ++t) {
      const long term = g * terms + t;
      const uint64_t* ap = a + (term << (log2n + 1));
      for (int j = tid; j < n; j += THREADS) {
        const c64 v{i64_to_f64_rne((int64_t)__ldcs(ap + j)), i64_to_f64_rne((int64_t)__ldcs(ap + j + n))};
        st(x + j, cmul(ldg(tw + j), v));
      }
      __syncthreads();
      const double2* r = unordered_smem<true, 0, ALGO>(L, 0, 1, x, y, w, tid, THREADS);
      const double2* bp = bhat + (term << log2n);
      if (ACC > 0) {
#pragma unroll
        for (int j = 0; j < (ACC > 0 ? ACC : 1); ++j) {
          const int k = tid + j * THREADS;
          if (k < n) {
            const c64 p = cmul(ldg(bp + k), ld(r + k));
            racc[j] = t == 0 ? p : cadd(racc[j], p);
          }
        }
      } else {
        for (int k = tid; k < n; k += THREADS) {
          const c64 p = cmul(ldg(bp + k), ld(r + k));
          st(acc + k, t == 0 ? p : cadd(ld(acc + k), p));
        }
      }
      __syncthreads();
    }
    double2* src = acc;
    if (ACC > 0) {
#pragma unroll
      for (int j = 0; j < (ACC > 0 ? ACC : 1); ++j) {
        const int k = tid + j * THREADS;
        if (k < n) st(y + k, racc[j]);
      }
      __syncthreads();
      src = y;
    }
    const double2* s = unordered_smem<false, 0, ALGO>(L, 0, 1, src, x, winv, tid, THREADS);
    uint64_t* op = out + (g << (log2n + 1));
    for (int j = tid; j < n; j += THREADS) {
      const c64 v = cmul(ldg(itw + j), ld(s + j));
      __stcs(op + j, round_half_up_mod64(v.re));
      __stcs(op + j + n, round_half_up_mod64(v.im));
    }
    __syncthreads();
  }
}

// Accumulator entries per thread in the register variant of the sum kernel:
// covers N/2 <= 8 x 128 = 1024 (N <= 2048).
constexpr int kSumRegAcc = 8;

// Bhat = fwd(tau^j * (b_j + i b_{j+N/2})) for small signed digits b.
template <int ALGO, int THREADS>
__global__ void __launch_bounds__(THREADS) u64_prepare_kernel(const int64_t* __restrict__ b,
                                                             double2* __restrict__ bhat, long count, DevLevels L,
                                                             const double2* __restrict__ w,
                                                             const double2* __restrict__ tw) {
  extern __shared__ double2 smem[];
  const int log2n = L.log2n[0];
  const int n = 1 << log2n;
  double2* x = smem;
  double2* y = smem + n;
  const int tid = threadIdx.x;
  for (long prod = blockIdx.x; prod < count; prod += gridDim.x) {
    const int64_t* bp = b + (prod << (log2n + 1));
    for (int j = tid; j < n; j += THREADS) {
      const c64 v{i64_to_f64_rne(bp[j]), i64_to_f64_rne(bp[j + n])};
      st(x + j, cmul(ldg(tw + j), v));
    }
    __syncthreads();
    const double2* r = unordered_smem<true, 0, ALGO>(L, 0, 1, x, y, w, tid, THREADS);
    double2* op = bhat + (prod << log2n);
    for (int k = tid; k < n; k += THREADS) op[k] = r[k];
    __syncthreads();
  }
}

constexpr int kProdThreads = 128;

// Kernel-pointer tables (nullptr when the combination is not instantiated).
const void* c64_kernel_e0(int algo, bool fwd);
// one transform over 2^ls CTAs (split.cuh); mode 0 no outer levels, 1 with levels
const void* c64_split_kernel_ptr(int algo, bool fwd, int ls, int mode);
const void* c64_kernel_emu(int algo, int e, bool fwd);
const void* u64_product_kernel_e0(int algo);
const void* u64_product_kernel_emu(int algo, int e);
const void* u64_prepare_kernel_ptr(int algo);
const void* u64_product_sum_kernel_ptr(int algo, bool reg_acc);

inline const void* c64_kernel(int algo, int e, bool fwd) {
  const int lvl = emu_level_for(algo, e);
  return lvl == 0 ? c64_kernel_e0(algo, fwd) : c64_kernel_emu(algo, lvl, fwd);
}
inline const void* u64_product_kernel_ptr(int algo, int e) {
  const int lvl = emu_level_for(algo, e);
  return lvl == 0 ? u64_product_kernel_e0(algo) : u64_product_kernel_emu(algo, lvl);
}

}  // namespace cfft
