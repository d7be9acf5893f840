// product_u64.cu -- fused negacyclic u64 polynomial product on unordered::Plan.
//
// One CTA computes one product at a time (grid-stride over the batch): it
// reads N u64 coefficients and N/2 resident Fourier coefficients, writes N u64
// results, and keeps every intermediate in shared memory, so a product costs
// exactly 48 KiB of HBM traffic at N = 2048 (24 bytes per coefficient).
//
// Pipeline (the way the reference's caller uses unordered::Plan; the crate
// itself has no product code):
//   z_j = tau^j * (a_j + i a_{j+N/2}),  tau = exp(i pi / N),  a read as i64
//   Z = fwd(z)                      unordered forward, permuted order
//   P_k = Bhat_k * Z_k              Bhat = fwd of the twisted operand, resident
//   p = inv(P)                      unordered inverse, standard order
//   t_j = (conj(tau^j) / (N/2)) * p_j
//   c_j = floor(Re t_j + 1/2) mod 2^64,  c_{j+N/2} = floor(Im t_j + 1/2) mod 2^64
// Every complex product is the reference's FMA form (cmul); conversions are
// exact integer-pipe routines, so the result is bit-identical to the oracle's
// CPU restatement of the same pipeline.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cfft_internal.h"
#include "runtime.h"
#include "c64_kernels.cuh"
#include "split_product.cuh"
#include "tune_cache.h"

using namespace cfft;

struct cfft_u64_product_plan {
  size_t N = 0, n = 0, base_n = 0;
  cfft_unordered_plan* fft = nullptr;  // the plan's transform, for the unfused entry points
  int base_algo = 0;
  LevelDesc lv{};
  DevLevels dlv{};
  double2 *d_w = nullptr, *d_winv = nullptr, *d_tw = nullptr, *d_itw = nullptr;
  int emu = 0;  // eighths of the butterfly additions issued on the integer pipe
  int cluster = 0;  // CTAs per product: 0 automatic, 1 one CTA, 2/4/8 a cluster of that size
};

namespace cfft {
// The product pipeline's elementwise steps as separate kernels (the unfused path).
__global__ void fold_twist_kernel(const uint64_t* __restrict__ a, double2* __restrict__ z, long total, int log2n,
                                  const double2* __restrict__ tw) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long p = g >> log2n, j = g & (n - 1);
    const uint64_t* ap = a + (p << (log2n + 1));
    const c64 v{i64_to_f64_rne((int64_t)ap[j]), i64_to_f64_rne((int64_t)ap[j + n])};
    st(z + g, cmul(ldg(tw + j), v));
  }
}
__global__ void pointwise_kernel(const double2* __restrict__ bhat, long bhat_stride, double2* __restrict__ z,
                                 long total, int log2n) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long p = g >> log2n, k = g & (n - 1);
    st(z + g, cmul(ldg(bhat + p * bhat_stride + k), ld(z + g)));
  }
}
// acc[g] = sum over t of bhat[g, t] * z[g, t] (terms back to back per group),
// the first product assigned and the others added in term order, as the fused
// sum kernels do.
__global__ void fourier_sum_kernel(const double2* __restrict__ bhat, const double2* __restrict__ z,
                                   double2* __restrict__ acc, int terms, long total, int log2n) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long grp = g >> log2n, k = g & (n - 1);
    const long base = ((grp * terms) << log2n) + k;
    c64 s = cmul(ldg(bhat + base), ld(z + base));
    for (int t = 1; t < terms; ++t) {
      const long o = base + ((long)t << log2n);
      s = cadd(s, cmul(ldg(bhat + o), ld(z + o)));
    }
    st(acc + g, s);
  }
}
// digits of the monomial X^degree mod (X^N + 1): one coefficient +-1 (X^N = -1)
__global__ void monomial_digits_kernel(int64_t* __restrict__ b, long N, unsigned long long degree) {
  grid_dependency_wait();
  const long pos = (long)(degree % (unsigned long long)N);
  const int64_t sign = ((degree / (unsigned long long)N) & 1) ? -1 : 1;
  for (long j = (long)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (long)gridDim.x * blockDim.x)
    b[j] = j == pos ? sign : 0;
}
__global__ void untwist_round_kernel(const double2* __restrict__ z, uint64_t* __restrict__ out, long total, int log2n,
                                     const double2* __restrict__ itw) {
  grid_dependency_wait();
  const long n = 1L << log2n;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long p = g >> log2n, j = g & (n - 1);
    const c64 t = cmul(ldg(itw + j), ld(z + g));
    uint64_t* op = out + (p << (log2n + 1));
    op[j] = round_half_up_mod64(t.re);
    op[j + n] = round_half_up_mod64(t.im);
  }
}
}  // namespace cfft

namespace {

int ew_grid(long total) { return (int)std::max<long>(1, std::min<long>((total + 255) / 256, (long)sm_count() * 16)); }

void free_u64(cfft_u64_product_plan* p) {
  if (p->fft) cfft_unordered_plan_destroy(p->fft);
  if (p->d_w) cudaFree(p->d_w);
  if (p->d_winv) cudaFree(p->d_winv);
  if (p->d_tw) cudaFree(p->d_tw);
  if (p->d_itw) cudaFree(p->d_itw);
}

DevLevels dev_levels(const LevelDesc& l) {
  DevLevels d;
  std::memset(&d, 0, sizeof(d));
  d.nlevels = l.nlevels;
  for (int i = 0; i <= kMaxLevels; ++i) {
    d.log2n[i] = l.log2n[i];
    d.w_off[i] = l.w_off[i];
  }
  for (int i = 0; i < kMaxLevels; ++i) {
    d.log2r[i] = l.log2r[i];
    d.winv_off[i] = l.winv_off[i];
  }
  return d;
}

// One CTA per product (the block scheduler hands the next product to the
// first SM with room, which balances the SMs to within one product) up to a
// large count; beyond it a grid of the resident CTAs strides over the batch.
int grid_for(const void* kernel, int threads, size_t smem, long count) {
  if (count <= (1L << 20)) return (int)std::max<long>(1, count);
  return (int)((long)sm_count() * max_blocks_per_sm(kernel, threads, smem));
}

// Sums of products too large for a cluster (N > 65536), unfused: fold and twist
// every term, the plan's forward transforms, the Fourier-domain sum per group,
// one inverse per group, untwist and round.  Groups run in chunks whose
// workspace (terms + 1 transforms per group) stays within 1 GiB.
cfft_status product_sum_unfused(const cfft_u64_product_plan* plan, const uint64_t* a, const double* bhat,
                                size_t terms, uint64_t* out, size_t count, cudaStream_t s) {
  const size_t n = plan->n, per_group = (terms + 1) * n * sizeof(double2);
  const size_t chunk = std::min(count, std::max<size_t>(1, (size_t(1) << 30) / per_group));
  void* ws = nullptr;
  if (cudaMallocAsync(&ws, chunk * per_group, s) != cudaSuccess)
    return fail(CFFT_ERR_OUT_OF_MEMORY, "product sum workspace");
  double2* z = (double2*)ws;
  double2* acc = z + chunk * terms * n;
  cfft_status st = CFFT_OK;
  for (size_t g0 = 0; g0 < count && st == CFFT_OK; g0 += chunk) {
    const size_t g = std::min(chunk, count - g0);
    st = cfft_u64_fold_twist(plan, a + g0 * terms * plan->N, (double*)z, g * terms, s);
    if (st == CFFT_OK) st = cfft_unordered_fwd(plan->fft, (double*)z, g * terms, s);
    if (st == CFFT_OK) {
      const long total = (long)(g * n);
      st = launch_dependent(fourier_sum_kernel, ew_grid(total), 256, 0, s, (const double2*)bhat + g0 * terms * n, z,
                            acc, (int)terms, total, ilog2(n)) == cudaSuccess
               ? CFFT_OK
               : fail(CFFT_ERR_CUDA, "fourier_sum_kernel launch");
    }
    if (st == CFFT_OK) st = cfft_unordered_inv(plan->fft, (double*)acc, g, s);
    if (st == CFFT_OK) st = cfft_u64_untwist_round(plan, (const double*)acc, out + g0 * plan->N, g, s);
  }
  cudaFreeAsync(ws, s);
  return st;
}

cfft_status launch_product(const cfft_u64_product_plan* plan, const uint64_t* a, const double* bhat,
                           size_t bhat_stride, uint64_t* out, size_t count, cudaStream_t stream) {
  const void* fn = u64_product_kernel_ptr(plan->base_algo, plan->emu);
  // N <= 128: 512 points per CTA iteration (one product of n = 32 would give a radix-4
  // pass 8 butterflies, a quarter warp: 122 vs 375 M products/s possible at N = 64)
  int log2p = 0;
  while ((plan->n << log2p) < 512 && plan->n <= 64) ++log2p;
  const size_t smem = 2 * (plan->n << log2p) * sizeof(double2);
  const int grid = grid_for(fn, kProdThreads, smem, ((long)count + (1L << log2p) - 1) >> log2p);
  DevLevels L = plan->dlv;
  long stride = (long)bhat_stride, cnt = (long)count;
  const double2* bh = (const double2*)bhat;
  void* args[] = {(void*)&a, (void*)&bh, &stride, (void*)&out, &cnt, &L, (void*)&plan->d_w, (void*)&plan->d_winv,
                  (void*)&plan->d_tw, (void*)&plan->d_itw, &log2p};
  return launch_kernel(fn, grid, kProdThreads, args, smem, stream);
}

// CTAs per product as a log2 (0: one CTA).  A product whose N/2-point
// transform exceeds one CTA's shared memory (N > 8192) always runs on a
// cluster, S = 2^ls with S <= level 0's radix, S <= 8 and n/S <= 4096 points
// per CTA (so N <= 65536); its default S gives each CTA 1024 points (the base
// size) where possible.  Smaller products use a cluster when the batch is too
// small to give every SM a product, or as the plan forces.
int product_split_log2(const cfft_u64_product_plan* p, size_t count, bool* ok) {
  *ok = true;
  const int log2n = ilog2(p->n);
  const int max_ls = p->lv.nlevels >= 1 ? std::min(3, p->lv.log2r[0]) : 0;
  const int min_ls = std::max(0, log2n - kSmemLog2Max);
  if (min_ls > max_ls) {
    *ok = false;
    return 0;
  }
  if (p->cluster >= 2) return std::max(min_ls, std::min(max_ls, ilog2((size_t)p->cluster)));
  if (min_ls > 0) return std::max(min_ls, std::min(max_ls, log2n - 10));
  if (p->cluster == 1 || max_ls == 0) return 0;
  // N = 8192: two CTAs of 2048 points (1.43 M products/s) beat one CTA of 4096,
  // which leaves one CTA per SM (1.12 M/s, 4864 products per launch)
  int ls = std::min(max_ls, std::max(0, log2n - kBlockLog2Auto));
  while (ls < max_ls && (count << ls) < (size_t)sm_count()) ++ls;
  return ls;
}

cfft_status launch_split_product(const cfft_u64_product_plan* plan, int ls, const uint64_t* a, const double* bhat,
                                 size_t bhat_stride, uint64_t* out, size_t count, cudaStream_t stream,
                                 const cfft_product_item* items = nullptr, int terms = 1) {
  const size_t part = plan->n >> ls;
  const bool big = part > 2048;  // 4096 points per CTA: one CTA per SM, 512 threads
  const void* fn = u64_product_split_ptr(plan->base_algo, ls, big);
  const size_t smem = 2 * (plan->n >> ls) * sizeof(double2);
  if ((count << ls) > 0x7fffffffUL) return fail(CFFT_ERR_INVALID_SIZE, "batch too large");
  DevLevels L = plan->dlv;
  long stride = (long)bhat_stride;
  const double2* bh = (const double2*)bhat;
  void* args[] = {(void*)&a, (void*)&bh, &stride, (void*)&out, &terms, (void*)&items, &L, (void*)&plan->d_w,
                  (void*)&plan->d_winv, (void*)&plan->d_tw, (void*)&plan->d_itw};
  // 128 threads (several CTAs per SM) for parts up to 1024 points, 256 for 2048
  // (shared memory allows 3 CTAs per SM), 512 for 4096 (one CTA per SM)
  const int threads = part <= 1024 ? 128 : (part <= 2048 ? kSplitProdThreads : kSplitProdThreadsBig);
  const int grid = (int)(count << ls);
  return launch_kernel_cluster(fn, grid, threads, 1 << ls, args, spread_smem(fn, grid, threads, 1 << ls, smem),
                               stream);
}

// CTAs per product as a log2 for plans without an outer level (n = base_n;
// u64_product_split0_kernel): S <= the base radix R and S <= 8, with at least
// 64 points per CTA.  `fast` also keeps at least 32 butterflies in each of a
// class's passes (64 for DIT, one thread per butterfly): with fewer, a lone
// product measured slower than on fewer CTAs (N = 2048, Dif8: 23.4 us on 8
// CTAs, 16.0 on 4; Dif16: 36.8 on 8, 25.0 on 2; Dit16 on 2: 45.9 against
// 39.8 for the five launches).  0 when the plan has levels or no S >= 2 fits.
int split0_log2(const cfft_u64_product_plan* p, bool fast = true) {
  if (p->lv.nlevels != 0) return 0;
  const int lr = p->base_algo / 2 + 1;
  const int log2n = ilog2(p->n);
  const int min_lb = !fast ? 0 : ((p->base_algo & 1) ? 6 : 5);
  int ls = std::min(3, lr);
  while (ls > 0 && (log2n - ls < 6 || log2n - ls - lr < min_lb)) --ls;
  return ls;
}

cfft_status launch_split0_product(const cfft_u64_product_plan* plan, int ls, const uint64_t* a, const double* bhat,
                                  size_t bhat_stride, uint64_t* out, size_t count, cudaStream_t stream,
                                  const cfft_product_item* items = nullptr, int terms = 1) {
  const int algo = plan->base_algo;
  const void* fn = u64_product_split0_ptr(algo, ls, terms > 1);
  if (!fn) return fail(CFFT_ERR_INVALID_SIZE, "no cluster product kernel for this base and cluster size");
  if ((count << ls) > 0x7fffffffUL) return fail(CFFT_ERR_INVALID_SIZE, "batch too large");
  const size_t part = plan->n >> ls;
  const size_t radix = size_t(2) << (algo / 2);
  // DIF: two threads per butterfly of a pass (half butterflies), DIT: one; at
  // least a thread per two points for the elementwise steps (radix 16 has few
  // butterflies per pass)
  const size_t pass_threads = ((algo & 1) ? 1 : 2) * part / radix;
  const int threads = (int)std::min<size_t>(256, std::max<size_t>(32, std::max(pass_threads, part / 2)));
  const size_t smem = 3 * part * sizeof(double2);
  const int grid = (int)(count << ls);
  DevLevels L = plan->dlv;
  long stride = (long)bhat_stride;
  const double2* bh = (const double2*)bhat;
  void* args[] = {(void*)&a, (void*)&bh, &stride, (void*)&out, &terms, (void*)&items, &L, (void*)&plan->d_w,
                  (void*)&plan->d_winv, (void*)&plan->d_tw, (void*)&plan->d_itw};
  // a few products: every CTA on an SM of its own
  return launch_kernel_cluster(fn, grid, threads, 1 << ls, args, spread_smem(fn, grid, threads, 1 << ls, smem),
                               stream);
}

// Launch shape of u64_product_split2_kernel with 2^ls1 classes: threads per CTA
// and shared memory (three buffers of the CTA's part of the base).
void split2_launch_shape(const cfft_u64_product_plan* p, int ls1, int* threads, size_t* smem) {
  const size_t part = p->base_n >> ls1;
  const size_t radix = size_t(2) << (p->base_algo / 2);
  *threads = (int)std::min<size_t>(256, std::max<size_t>(32, std::max(2 * part / radix, part / 2)));
  *smem = 3 * part * sizeof(double2);
}

// The shape of u64_product_split2_kernel for a plan, as log2s: one outer level
// of radix R0 = 2^ls0 <= 8 over a DIF base of m points and S1 = 2^ls1 >= 2
// classes of the base, with S1 <= R, at least 64 points per CTA and at least 32
// butterflies in each of a class's passes (as split0_log2).  R0 * S1 is at most
// 16 where the `count` products' (or sums') 16-CTA clusters (a non-portable size)
// are resident at once with one CTA per SM; else at most 8.  Not for a radix-2 base under a radix-4 level: N = 4096
// on Dif2/512 measured slower than the five launches from 16 products (29.7
// against 24.9 us).  false when the plan has another shape.
bool split2_shape(const cfft_u64_product_plan* p, size_t count, int* ls0, int* ls1, bool sum = false,
                  bool allow16 = true) {
  if (p->lv.nlevels != 1 || (p->base_algo & 1) || p->lv.log2r[0] > 3) return false;
  const int lr = p->base_algo / 2 + 1;
  if (lr == 1 && p->lv.log2r[0] > 1) return false;
  const int log2m = ilog2(p->base_n);
  const int l0 = p->lv.log2r[0];
  for (int max_ls = allow16 && (count << 4) <= (size_t)sm_count() ? 4 : 3; max_ls >= 3; --max_ls) {
    int l1 = std::min(max_ls - l0, lr);
    while (l1 > 0 && (log2m - l1 < 6 || log2m - l1 - lr < 5)) --l1;
    if (l1 < 1) return false;
    const void* fn = u64_product_split2_ptr(p->base_algo, l0, l1, sum);
    if (!fn) continue;
    if (l0 + l1 > 3) {  // every product's 16-CTA cluster resident at once, one CTA per SM
      int threads = 0;
      size_t smem = 0;
      split2_launch_shape(p, l1, &threads, &smem);
      if ((long)count > (long)spread_clusters(fn, threads, 16)) continue;
    }
    *ls0 = l0;
    *ls1 = l1;
    return true;
  }
  return false;
}

cfft_status launch_split2_product(const cfft_u64_product_plan* plan, int ls0, int ls1, const uint64_t* a,
                                  const double* bhat, size_t bhat_stride, uint64_t* out, size_t count,
                                  cudaStream_t stream, const cfft_product_item* items = nullptr, int terms = 1) {
  const void* fn = u64_product_split2_ptr(plan->base_algo, ls0, ls1, terms > 1);
  if (!fn) return fail(CFFT_ERR_INVALID_SIZE, "no one-level cluster product kernel for this shape");
  const int ls = ls0 + ls1;
  if ((count << ls) > 0x7fffffffUL) return fail(CFFT_ERR_INVALID_SIZE, "batch too large");
  int threads = 0;
  size_t smem = 0;
  split2_launch_shape(plan, ls1, &threads, &smem);
  const int grid = (int)(count << ls);
  DevLevels L = plan->dlv;
  long stride = (long)bhat_stride;
  const double2* bh = (const double2*)bhat;
  void* args[] = {(void*)&a, (void*)&bh, &stride, (void*)&out, &terms, (void*)&items, &L, (void*)&plan->d_w,
                  (void*)&plan->d_winv, (void*)&plan->d_tw, (void*)&plan->d_itw};
  return launch_kernel_cluster(fn, grid, threads, 1 << ls, args, spread_smem(fn, grid, threads, 1 << ls, smem),
                               stream);
}

}  // namespace

// Products given as device items (all of the plan's N) on the largest cluster
// the plan allows, for latency: the serving loop's large products.
bool cfft::u64_product_splittable(const cfft_u64_product_plan* plan) {
  if (plan->lv.nlevels == 0) return split0_log2(plan) >= 1;
  const int max_ls = std::min(3, plan->lv.log2r[0]);
  const int min_ls = std::max(0, ilog2(plan->n) - kSmemLog2Max);
  return max_ls >= 1 && min_ls <= max_ls;
}

cfft_status cfft::u64_product_split_items(const cfft_u64_product_plan* plan, const cfft_product_item* items,
                                          size_t count, void* stream) {
  if (!u64_product_splittable(plan)) return fail(CFFT_ERR_INVALID_SIZE, "product size cannot be split over a cluster");
  if (count == 0) return CFFT_OK;
  if (plan->lv.nlevels == 0)
    return launch_split0_product(plan, split0_log2(plan), nullptr, nullptr, 0, nullptr, count, (cudaStream_t)stream,
                                 items);
  // At most 8 CTAs per product here: the serving loop and the work queue keep several
  // launches in flight, and a 16-CTA cluster waits for 16 free SMs of one GPC
  int ls0 = 0, ls1 = 0;
  if (split2_shape(plan, count, &ls0, &ls1, false, false))
    return launch_split2_product(plan, ls0, ls1, nullptr, nullptr, 0, nullptr, count, (cudaStream_t)stream, items);
  const int max_ls = std::min(3, plan->lv.log2r[0]);
  return launch_split_product(plan, max_ls, nullptr, nullptr, 0, nullptr, count, (cudaStream_t)stream, items);
}

void cfft::u64_product_tables(const cfft_u64_product_plan* p, const void** w, const void** winv, const void** tw,
                              const void** itw) {
  *w = p->d_w;
  *winv = p->d_winv;
  *tw = p->d_tw;
  *itw = p->d_itw;
}

extern "C" {

cfft_status cfft_u64_fold_twist(const cfft_u64_product_plan* plan, const uint64_t* a, double* z, size_t count,
                                void* stream) {
  if (!plan || !a || !z) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (count == 0) return CFFT_OK;
  const long total = (long)(count * plan->n);
  CFFT_CUDA_TRY(launch_dependent(fold_twist_kernel, ew_grid(total), 256, 0, (cudaStream_t)stream, a, (double2*)z,
                                 total, ilog2(plan->n), (const double2*)plan->d_tw));
  return CFFT_OK;
}

cfft_status cfft_c64_pointwise(const double* bhat, size_t bhat_stride, double* z, size_t n, size_t count,
                               void* stream) {
  if (!bhat || !z) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (!is_pow2(n)) return fail(CFFT_ERR_INVALID_SIZE, "n must be a power of two");
  if (count == 0) return CFFT_OK;
  const long total = (long)(count * n);
  CFFT_CUDA_TRY(launch_dependent(pointwise_kernel, ew_grid(total), 256, 0, (cudaStream_t)stream, (const double2*)bhat,
                                 (long)bhat_stride, (double2*)z, total, ilog2(n)));
  return CFFT_OK;
}

cfft_status cfft_u64_untwist_round(const cfft_u64_product_plan* plan, const double* z, uint64_t* out, size_t count,
                                   void* stream) {
  if (!plan || !z || !out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (count == 0) return CFFT_OK;
  const long total = (long)(count * plan->n);
  CFFT_CUDA_TRY(launch_dependent(untwist_round_kernel, ew_grid(total), 256, 0, (cudaStream_t)stream,
                                 (const double2*)z, out, total, ilog2(plan->n), (const double2*)plan->d_itw));
  return CFFT_OK;
}

cfft_status cfft_u64_fourier_mul_monomial(const cfft_u64_product_plan* plan, unsigned long long degree, double* z,
                                          size_t count, void* stream) {
  if (!plan || !z) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (count == 0) return CFFT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  // the monomial's digits, its operand (the plan's own preparation), then the pointwise
  // product with every polynomial: the same bits as preparing X^degree and multiplying
  void* ws = nullptr;
  const size_t digit_bytes = plan->N * sizeof(int64_t);
  if (cudaMallocAsync(&ws, digit_bytes + plan->n * sizeof(double2), s) != cudaSuccess)
    return fail(CFFT_ERR_OUT_OF_MEMORY, "monomial workspace");
  int64_t* digits = (int64_t*)ws;
  double* mono = (double*)((char*)ws + digit_bytes);
  cfft_status st = launch_dependent(monomial_digits_kernel, ew_grid((long)plan->N), 256, 0, s, digits, (long)plan->N,
                                    degree) == cudaSuccess
                       ? CFFT_OK
                       : fail(CFFT_ERR_CUDA, "monomial digits launch");
  if (st == CFFT_OK) st = cfft_u64_prepare_operand(plan, digits, mono, 1, stream);
  if (st == CFFT_OK) st = cfft_c64_pointwise(mono, 0, z, plan->n, count, stream);
  cudaFreeAsync(ws, s);
  return st;
}

cfft_status cfft_u64_product_sum(const cfft_u64_product_plan* plan, const uint64_t* a, const double* bhat,
                                 size_t terms, uint64_t* out, size_t count, void* stream) {
  if (!plan || !a || !bhat || !out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (terms == 0 || terms > 0x7fffffff) return fail(CFFT_ERR_INVALID_ARGUMENT, "terms must be at least 1");
  // a few outputs of a plan with one outer level of radix 2 or 4 over a DIF base: one
  // cluster of level-0 slices times base classes per output, as the products
  int l0 = 0, l1 = 0;
  if (count > 0 && (long)count < (long)sm_count() / 2 && plan->cluster == 0 &&
      split2_shape(plan, count, &l0, &l1, terms > 1))
    return launch_split2_product(plan, l0, l1, a, bhat, plan->n, out, count, (cudaStream_t)stream, nullptr,
                                 (int)terms);
  if (plan->N > (size_t(2) << kBlockLog2Auto)) {  // one output per thread-block cluster (N = 8192: by default)
    bool ok = true;
    const int ls = product_split_log2(plan, count, &ok);
    if (count == 0) return CFFT_OK;
    // from N = 32768 the unfused sum, as the products take five launches there
    if (!ok || (plan->N >= 32768 && plan->cluster == 0))
      return product_sum_unfused(plan, a, bhat, terms, out, count, (cudaStream_t)stream);
    if (ls > 0)
      return launch_split_product(plan, ls, a, bhat, plan->n, out, count, (cudaStream_t)stream, nullptr,
                                  (int)terms);
  }
  if (count == 0) return CFFT_OK;
  // a few outputs of a plan without an outer level on a DIF base (the external
  // product of a blind-rotation step): one cluster per output, as the products
  const int ls0 = split0_log2(plan);
  if (ls0 >= 1 && !(plan->base_algo & 1) && (long)count < (long)sm_count() / 2 && plan->cluster == 0 &&
      (plan->n >> ls0) <= (size_t)kSplit0Acc * 256)
    return launch_split0_product(plan, ls0, a, bhat, plan->n, out, count, (cudaStream_t)stream, nullptr, (int)terms);
  const bool reg_acc = plan->n <= (size_t)(kSumRegAcc * kProdThreads);
  const void* fn = u64_product_sum_kernel_ptr(plan->base_algo, reg_acc);
  const size_t smem = (reg_acc ? 2 : 3) * plan->n * sizeof(double2);
  const int grid = grid_for(fn, kProdThreads, smem, (long)count);
  DevLevels L = plan->dlv;
  long cnt = (long)count;
  int tr = (int)terms;
  const double2* bh = (const double2*)bhat;
  void* args[] = {(void*)&a, (void*)&bh, &tr, (void*)&out, &cnt, &L, (void*)&plan->d_w, (void*)&plan->d_winv,
                  (void*)&plan->d_tw, (void*)&plan->d_itw};
  return launch_kernel(fn, grid, kProdThreads, args, smem, (cudaStream_t)stream);
}

cfft_unordered_plan* cfft_u64_product_fft(const cfft_u64_product_plan* plan) { return plan ? plan->fft : nullptr; }

cfft_status cfft_u64_product_set_cluster_size(cfft_u64_product_plan* plan, int ctas) {
  if (!plan || !(ctas == 0 || ctas == 1 || ctas == 2 || ctas == 4 || ctas == 8))
    return fail(CFFT_ERR_INVALID_ARGUMENT, "cluster size must be 0 (automatic), 1, 2, 4 or 8");
  plan->cluster = ctas;
  return CFFT_OK;
}

cfft_status cfft_u64_product_set_int_adds(cfft_u64_product_plan* plan, int eighths) {
  if (!plan || eighths < 0 || eighths > 8) return fail(CFFT_ERR_INVALID_ARGUMENT, "eighths must be in 0..8");
  plan->emu = eighths;
  return CFFT_OK;
}
int cfft_u64_product_int_adds(const cfft_u64_product_plan* plan) {
  return plan ? emu_level_for(plan->base_algo, plan->emu) : -1;
}

cfft_status cfft_u64_product_plan_create(size_t N, cfft_algo base_algo, size_t base_n, cfft_u64_product_plan** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!is_pow2(N) || N < 64 || ilog2(N) > kUnorderedMaxLog2 + 1)
    return fail(CFFT_ERR_INVALID_SIZE, "u64 product: N must be a power of two in [64, 2^29]");
  const size_t n = N / 2;
  if (!is_pow2(base_n) || base_n > n || (base_n != n && base_n < 32) || ilog2(base_n) > 10)
    return fail(CFFT_ERR_INVALID_ARGUMENT, "u64 product: invalid base_n");
  if (base_algo < 0 || base_algo > 7) return fail(CFFT_ERR_INVALID_ARGUMENT, "unknown FftAlgo");
  cfft_status st = CFFT_OK;
  auto* p = new cfft_u64_product_plan();
  p->N = N;
  p->n = n;
  p->base_n = base_n;
  p->base_algo = base_algo;
  p->lv = make_levels(n, base_n);
  p->dlv = dev_levels(p->lv);
  std::vector<c64h> w(n + base_n), wi(n + base_n), tw(n), itw(n);
  unordered_twiddles(n, base_n, algo_radix(base_algo), w.data(), wi.data());
  product_twist_tables(N, tw.data(), itw.data());
  st = upload((const double2*)w.data(), n + base_n, &p->d_w);
  if (st == CFFT_OK) st = cfft_unordered_plan_create(n, base_algo, base_n, &p->fft);
  if (st == CFFT_OK) st = upload((const double2*)wi.data(), n + base_n, &p->d_winv);
  if (st == CFFT_OK) st = upload((const double2*)tw.data(), n, &p->d_tw);
  if (st == CFFT_OK) st = upload((const double2*)itw.data(), n, &p->d_itw);
  if (st != CFFT_OK) {
    free_u64(p);
    delete p;
    return st;
  }
  *out = p;
  return CFFT_OK;
}

void cfft_u64_product_plan_destroy(cfft_u64_product_plan* plan) {
  if (!plan) return;
  free_u64(plan);
  delete plan;
}

size_t cfft_u64_product_poly_size(const cfft_u64_product_plan* plan) { return plan ? plan->N : 0; }
void cfft_u64_product_algo(const cfft_u64_product_plan* plan, cfft_algo* base_algo, size_t* base_n) {
  if (!plan) return;
  if (base_algo) *base_algo = (cfft_algo)plan->base_algo;
  if (base_n) *base_n = plan->base_n;
}

cfft_status cfft_u64_prepare_operand(const cfft_u64_product_plan* plan, const int64_t* b, double* bhat, size_t count,
                                     void* stream) {
  if (!plan || !b || !bhat) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (count == 0) return CFFT_OK;
  if (plan->N > (size_t(2) << kSmemLog2Max)) {  // unfused: fold and twist, then the plan's forward FFT
    cfft_status st = cfft_u64_fold_twist(plan, (const uint64_t*)b, bhat, count, stream);
    if (st != CFFT_OK) return st;
    return cfft_unordered_fwd(plan->fft, bhat, count, stream);
  }
  const size_t smem = 2 * plan->n * sizeof(double2);
  const void* fn = u64_prepare_kernel_ptr(plan->base_algo);
  const int grid = grid_for(fn, kProdThreads, smem, (long)count);
  DevLevels L = plan->dlv;
  long cnt = (long)count;
  double2* bh = (double2*)bhat;
  void* args[] = {(void*)&b, &bh, &cnt, &L, (void*)&plan->d_w, (void*)&plan->d_tw};
  return launch_kernel(fn, grid, kProdThreads, args, smem, (cudaStream_t)stream);
}

cfft_status cfft_u64_product(const cfft_u64_product_plan* plan, const uint64_t* a, const double* bhat,
                             size_t bhat_stride, uint64_t* out, size_t count, void* stream) {
  if (!plan || !a || !bhat || !out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (bhat_stride != 0 && bhat_stride != plan->n)
    return fail(CFFT_ERR_INVALID_ARGUMENT, "bhat_stride must be 0 or N/2");
  bool ok = true;
  const int ls = product_split_log2(plan, count, &ok);
  if (count == 0) return CFFT_OK;
  // The five-launch path on a workspace from the stream-ordered allocator: N > 65536
  // (no cluster holds it), and N >= 32768 at every batch, where it measured faster
  // than one cluster per product (Dif8/512, CUDA events: one product 30.5 vs 74.4 us
  // at 32768, 35.8 vs 142 at 65536; 38 products 134 vs 212 and 274 vs 423; large
  // batches 304 vs 280 k products/s at 32768, 129 vs 102 k at 65536)
  const bool many = (long)count >= (long)sm_count() / 2 && plan->cluster == 0;
  // A few products whose transform has no outer level (n = base_n): one cluster per
  // product on the base's residue classes (u64_product_split0_kernel), as does a plan
  // forced to a cluster size.  Device time per call at N = 2048, Dif4, 4
  // CTAs: 11.7 us for one product (one CTA: 32.2, the five launches: 13.7), 16.7 for
  // 38 (one CTA: 34.9, five launches: 19.4)
  if (plan->cluster >= 2 && split0_log2(plan, false) >= 1)
    return launch_split0_product(plan, std::min(split0_log2(plan, false), ilog2((size_t)plan->cluster)), a, bhat,
                                 bhat_stride, out, count, (cudaStream_t)stream);
  // Base radix >= 4: up to one product per SM (N = 2048, 152 products: 25.5 us on Dif4
  // clusters, 33.9 on one CTA each; Dif8 28.9 against 35.0); radix 2 lost there (Dif2,
  // N = 1024, 152 products: 24.9 against 20.5 us) and keeps the SMs/2 limit.
  const long split0_max = (plan->base_algo >= 2) ? (long)sm_count() : (long)sm_count() / 2 - 1;
  if (plan->cluster == 0 && plan->N >= 512 && (long)count <= split0_max && split0_log2(plan) >= 1)
    return launch_split0_product(plan, split0_log2(plan), a, bhat, bhat_stride, out, count, (cudaStream_t)stream);
  // Likewise a plan with one outer level of radix 2, 4 or 8 over a DIF base: level 0's
  // slices times classes of the base (u64_product_split2_kernel).  One product, Dif4
  // on 1024 points: 13.7 us at N = 4096 (five launches 32.1), 20.9 at 8192 (34.2);
  // 38 products: 23.3 (33.5) and 44.7 (58.8)
  int ls0 = 0, ls1 = 0;
  if (plan->cluster == 0 && !many && split2_shape(plan, count, &ls0, &ls1))
    return launch_split2_product(plan, ls0, ls1, a, bhat, bhat_stride, out, count, (cudaStream_t)stream);
  // otherwise (no cluster kernel for the base) the five launches, whose transforms
  // split over 2-8 CTAs each
  const bool few_unsplit = ls == 0 && plan->cluster == 0 && plan->N >= 2048 && !many;
  // Fewer than SMs/4 products of N = 4096 or 8192 as well (one product: 34 vs 37 us at
  // 4096, 37 vs 39 us at 8192; from SMs/4 products of N = 8192 the cluster kernel is faster)
  const bool few_mid = plan->cluster == 0 && plan->N >= 4096 && plan->N <= 8192 &&
                       (long)count < (long)sm_count() / 4;
  if (!ok || (plan->N >= 32768 && plan->cluster == 0) || few_unsplit || few_mid) {
    cudaStream_t s = (cudaStream_t)stream;
    void* z = nullptr;
    if (cudaMallocAsync(&z, count * plan->n * sizeof(double2), s) != cudaSuccess)
      return fail(CFFT_ERR_OUT_OF_MEMORY, "u64 product workspace");
    cfft_status st = cfft_u64_fold_twist(plan, a, (double*)z, count, stream);
    if (st == CFFT_OK) st = cfft_unordered_fwd(plan->fft, (double*)z, count, stream);
    if (st == CFFT_OK) st = cfft_c64_pointwise(bhat, bhat_stride, (double*)z, plan->n, count, stream);
    if (st == CFFT_OK) st = cfft_unordered_inv(plan->fft, (double*)z, count, stream);
    if (st == CFFT_OK) st = cfft_u64_untwist_round(plan, (const double*)z, out, count, stream);
    cudaFreeAsync(z, s);
    return st;
  }
  if (ls > 0) return launch_split_product(plan, ls, a, bhat, bhat_stride, out, count, (cudaStream_t)stream);
  return launch_product(plan, a, bhat, bhat_stride, out, count, (cudaStream_t)stream);

}

// Method::Measure for the product: every (base_algo, base_n) the reference's
// unordered measurement considers for n = N/2 (src/unordered.rs:553-640: the
// ordered algorithms at n when n <= 256, else bases 512 and 1024), timed on
// the fused product kernel itself over a batch that fills every SM.  Several
// candidates run at the FP64 roof within noise of each other; among those
// within 2% of the fastest a DIF base is taken, whose few-product cluster
// kernels are the faster ones (one N = 4096 product: 13.7 us on Dif4/1024, 31
// us on the five launches that DIT bases take).
cfft_status cfft_u64_product_plan_create_measure(size_t N, double seconds, cfft_u64_product_plan** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!is_pow2(N) || N < 64 || ilog2(N) > kUnorderedMaxLog2 + 1)
    return fail(CFFT_ERR_INVALID_SIZE, "u64 product: N must be a power of two in [64, 2^29]");
  const size_t n = N / 2;
  TuneVal tv;
  if (tune_lookup(2, N, &tv)) {  // measured before on this GPU model
    cfft_status st = cfft_u64_product_plan_create(N, (cfft_algo)tv.algo, tv.base_n, out);
    if (st == CFFT_OK) (*out)->emu = tv.emu;
    return st;
  }
  std::vector<size_t> bases;
  if (n <= 256) bases.push_back(n);
  else
    for (size_t b : {size_t(512), size_t(1024)})
      if (b <= n) bases.push_back(b);
  // eight products per SM up to N = 8192, the same number of CTAs for larger N,
  // within 2 GiB of operands, results and workspace (32 N bytes per product)
  const size_t per_sm = std::max<size_t>(1, 8 * 8192 / std::max<size_t>(N, 8192));
  const size_t count = std::max<size_t>(1, std::min((size_t)sm_count() * per_sm, (size_t(1) << 31) / (32 * N)));
  uint64_t *da = nullptr, *dout = nullptr;
  double* dbhat = nullptr;
  CFFT_CUDA_TRY(cudaMalloc(&da, count * N * sizeof(uint64_t)));
  CFFT_CUDA_TRY(cudaMalloc(&dout, count * N * sizeof(uint64_t)));
  CFFT_CUDA_TRY(cudaMalloc(&dbhat, count * n * sizeof(double2)));
  CFFT_CUDA_TRY(cudaMemset(da, 0, count * N * sizeof(uint64_t)));
  CFFT_CUDA_TRY(cudaMemset(dbhat, 0, count * n * sizeof(double2)));
  cudaStream_t s;
  CFFT_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e30;
  int best_algo = 0;
  size_t best_base = bases.front();
  struct Timed {
    int algo;
    size_t base;
    double ms;
  };
  std::vector<Timed> timed;
  cfft_status st = CFFT_OK;
  for (size_t base : bases) {
    for (int algo = 0; algo < 8 && st == CFFT_OK; ++algo) {
      cfft_u64_product_plan* p = nullptr;
      st = cfft_u64_product_plan_create(N, (cfft_algo)algo, base, &p);
      if (st != CFFT_OK) break;
      cfft_u64_product(p, da, dbhat, n, dout, count, s);  // warm-up
      int reps = 1;
      double per = 0;
      for (;;) {
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps; ++r) cfft_u64_product(p, da, dbhat, n, dout, count, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        per = ms / reps;
        if (ms * 1e-3 >= std::max(seconds, 1e-3) || reps >= 4096) break;
        reps *= 2;
      }
      if (per < best) {
        best = per;
        best_algo = algo;
        best_base = base;
      }
      timed.push_back(Timed{algo, base, per});
      cfft_u64_product_plan_destroy(p);
    }
  }
  if (best_algo & 1) {  // a DIT winner: the fastest DIF base within 2%, if any
    double dif_best = 1e30;
    for (const Timed& t : timed)
      if (!(t.algo & 1) && t.ms <= best * 1.02 && t.ms < dif_best) {
        dif_best = t.ms;
        best_algo = t.algo;
        best_base = t.base;
      }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(da);
  cudaFree(dout);
  cudaFree(dbhat);
  if (st != CFFT_OK) return st;
  st = cfft_u64_product_plan_create(N, (cfft_algo)best_algo, best_base, out);
  if (st != CFFT_OK) return st;
  // integer-pipe share of the additions for the winning algorithm
  CFFT_CUDA_TRY(cudaMalloc(&da, count * N * sizeof(uint64_t)));
  CFFT_CUDA_TRY(cudaMalloc(&dout, count * N * sizeof(uint64_t)));
  CFFT_CUDA_TRY(cudaMalloc(&dbhat, count * n * sizeof(double2)));
  CFFT_CUDA_TRY(cudaMemset(da, 0, count * N * sizeof(uint64_t)));
  CFFT_CUDA_TRY(cudaMemset(dbhat, 0, count * n * sizeof(double2)));
  CFFT_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best_e = 1e30;
  int be = (*out)->emu;
  for (int e : kEmuLevels) {
    if (emu_level_for(best_algo, e) != e) continue;
    (*out)->emu = e;
    cfft_u64_product(*out, da, dbhat, n, dout, count, s);
    cudaEventRecord(e0, s);
    const int reps = 8;
    for (int r = 0; r < reps; ++r) cfft_u64_product(*out, da, dbhat, n, dout, count, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_e) {
      best_e = ms;
      be = e;
    }
  }
  (*out)->emu = be;
  tune_store(2, N, TuneVal{best_algo, best_base, kProdThreads, 1, be});
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(da);
  cudaFree(dout);
  cudaFree(dbhat);
  return CFFT_OK;
}

// Host-buffer products: the batch is cut into chunks that flow through three
// streams, so the host-to-device copy of one chunk, the kernel of the previous
// one and the device-to-host copy of the one before overlap (copy engines and
// SMs work at once).  Returns when every result is in host memory.
cfft_status cfft_u64_product_host(const cfft_u64_product_plan* plan, const uint64_t* a, const double* bhat,
                                  size_t bhat_stride, uint64_t* out, size_t count) {
  if (!plan || !a || !bhat || !out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (bhat_stride != 0 && bhat_stride != plan->n)
    return fail(CFFT_ERR_INVALID_ARGUMENT, "bhat_stride must be 0 or N/2");
  if (count == 0) return CFFT_OK;
  // About 24 chunks per call on 4 streams: the first copy in and the last
  // copy out, which nothing overlaps, are then 1/24 of the data each, and 4
  // chunks in flight keep kernels of several chunks resident at once.  When
  // `out` is page-locked the kernels store the results there themselves (no
  // copy out, no drain): 6.56 vs 6.40 M products/s at N = 2048, 8192 per call.
  // Measured schedules (M products/s, Dif4, 8192 per call, direct stores):
  // 24 chunks on 4 streams 6.58, on 6 6.53, on 8 6.48; 12 on 6 6.38, 48 on 6
  // 6.50; a first chunk of 76 or 152 products or a last one of 152: within
  // 0.03 of the equal chunks.  Device buffers alone: 6.88.
  // The operands still come in by copy: kernels reading them from host memory
  // wait on every product's first loads (6.60 M/s for one launch with both
  // sides in host memory, against 6.94 M/s on device buffers).
  const HostChunks hc = host_chunks();
  const int nslots = hc.slots;
  const size_t poly_bytes = plan->N * sizeof(uint64_t);
  // the schedule: an optional first and last chunk, the rest in `chunks` equal chunks of
  // at least two products per SM
  const size_t first_c = std::min(count, (size_t)hc.first);
  const size_t last_c = std::min(count - first_c, (size_t)hc.last);
  const size_t mid = count - first_c - last_c;
  const size_t min_chunk = (size_t)sm_count() * 2;
  const size_t chunk = mid ? std::min(mid, std::max(min_chunk, (mid + hc.chunks - 1) / hc.chunks)) : 0;
  const size_t cap = std::max(chunk, std::max(first_c, last_c));
  uint64_t* mapped_out = (uint64_t*)mapped_host_range(out, count * poly_bytes);
  PipeSlot slot[8];
  cfft_status st = host_pipeline(nslots, 2 * cap * poly_bytes, slot);
  if (st != CFFT_OK) return st;
  size_t i = 0;
  for (size_t first = 0; first < count; ++i) {
    const size_t c = first == 0 && first_c ? first_c
                     : (last_c && first + last_c >= count) ? count - first : std::min(chunk, count - first - last_c);
    const PipeSlot& sl = slot[i % nslots];
    uint64_t* da = (uint64_t*)sl.dev;
    uint64_t* dout = mapped_out ? mapped_out + first * plan->N : da + cap * plan->N;
    CFFT_CUDA_TRY(cudaMemcpyAsync(da, a + first * plan->N, c * poly_bytes, cudaMemcpyHostToDevice, sl.stream));
    const double* bh = bhat + (bhat_stride ? first * bhat_stride * 2 : 0);
    st = cfft_u64_product(plan, da, bh, bhat_stride, dout, c, sl.stream);
    if (st != CFFT_OK) return st;
    if (!mapped_out)
      CFFT_CUDA_TRY(cudaMemcpyAsync(out + first * plan->N, dout, c * poly_bytes, cudaMemcpyDeviceToHost, sl.stream));
    first += c;
  }
  for (int k = 0; k < nslots; ++k) CFFT_CUDA_TRY(cudaStreamSynchronize(slot[k].stream));
  return CFFT_OK;
}

}  // extern "C"
