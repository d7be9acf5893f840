// c64.cu -- ordered::Plan and unordered::Plan on the GPU (c64 transforms).
//
// Execution: transforms (or, above 4096 points, the sub-transforms below the
// top unordered levels) are loaded into one CTA's shared memory, run through
// the reference's passes there and written back; unordered levels of larger
// transforms run in place in global memory first (forward) or last (inverse).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "cfft_internal.h"
#include "runtime.h"
#include "c64_kernels.cuh"
#include "tune_cache.h"

using namespace cfft;

namespace cfft {

// One unordered level in place in global memory, over every chunk of 2^log2nl points.
template <bool FWD>
__global__ void __launch_bounds__(256) c64_level_kernel(double2* data, long total, int log2r, int log2nl,
                                                        const double2* __restrict__ wl) {
  const int lm = log2nl - log2r;
  grid_dependency_wait();
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    double2* zc = data + ((g >> lm) << log2nl);
    const int i = (int)(g & ((1L << lm) - 1));
    if (log2r == 1) outer_group<2, FWD, 0>(zc, lm, i, wl);
    else if (log2r == 2) outer_group<4, FWD, 0>(zc, lm, i, wl);
    else outer_group<8, FWD, 0>(zc, lm, i, wl);
  }
}

__device__ __forceinline__ unsigned bit_rev_dev(int nbits, unsigned i) {
  return nbits == 0 ? 0u : (__brev(i) >> (32 - nbits));
}
// src/unordered.rs:1046-1059
__device__ __forceinline__ unsigned bit_rev_twice_dev(int nbits, int base_nbits, unsigned i) {
  const unsigned i_rev = bit_rev_dev(nbits, i);
  const unsigned mask = (1u << base_nbits) - 1u;
  return (i_rev & ~mask) | bit_rev_dev(base_nbits, i_rev & mask);
}
__device__ __forceinline__ unsigned bit_rev_twice_inv_dev(int nbits, int base_nbits, unsigned i) {
  const unsigned mask = (1u << base_nbits) - 1u;
  return bit_rev_dev(nbits, (i & ~mask) | bit_rev_dev(base_nbits, i & mask));
}

// standard[i] = permuted[bit_rev_twice(i)] (to_standard) or the scatter back.
template <bool TO_STD>
__global__ void c64_permute_kernel(const double2* __restrict__ src, double2* __restrict__ dst, long total, int nbits,
                                   int base_nbits) {
  const long mask = (1L << nbits) - 1;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long)gridDim.x * blockDim.x) {
    const long b = g & ~mask;
    const unsigned i = (unsigned)(g & mask);
    const unsigned j = bit_rev_twice_dev(nbits, base_nbits, i);
    if (TO_STD) dst[g] = src[b + j];
    else dst[b + j] = src[g];
  }
}

// The same conversion through shared memory, for n <= 4096: a CTA reads a
// tile of whole transforms with coalesced loads, then writes the tile's
// destination in order, gathering from shared memory.  Shared-memory slot of
// element e: e with its low 3 bits XORed with its higher 3-bit groups, so the
// 8 lanes of a 128-bit access phase hit distinct bank groups both for the
// linear writes and for the permuted reads (whose varying bits are 3
// adjacent bit positions of e).  TO_STD gathers with bit_rev_twice (standard
// from permuted), otherwise with its inverse (permuted from standard).
__device__ __forceinline__ int perm_slot(int e) { return e ^ (((e >> 3) ^ (e >> 6) ^ (e >> 9)) & 7); }

template <bool TO_STD>
__global__ void __launch_bounds__(256) c64_permute_tile_kernel(const double2* __restrict__ src,
                                                               double2* __restrict__ dst, int nbits, int base_nbits,
                                                               int log2tile) {
  extern __shared__ double2 tile[];
  const int npts = 1 << log2tile;
  const long off = (long)blockIdx.x << log2tile;
  // eight loads in flight per thread before any shared-memory store
  constexpr int kU = 8;
  for (int b = 0; b < npts; b += kU * 256) {
    double2 v[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int i = b + u * 256 + (int)threadIdx.x;
      if (i < npts) v[u] = __ldcs(src + off + i);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int i = b + u * 256 + (int)threadIdx.x;
      if (i < npts) tile[perm_slot(i)] = v[u];
    }
  }
  __syncthreads();
  const int mask = (1 << nbits) - 1;
  for (int k = threadIdx.x; k < npts; k += blockDim.x) {
    const unsigned kk = (unsigned)(k & mask);
    const unsigned e = TO_STD ? bit_rev_twice_dev(nbits, base_nbits, kk) : bit_rev_twice_inv_dev(nbits, base_nbits, kk);
    __stcs(dst + off + k, tile[perm_slot((k & ~mask) | (int)e)]);
  }
}

// src/unordered.rs:844-900
__global__ void c64_monomial_kernel(double2* __restrict__ buf, const double2* __restrict__ tw, int nbits,
                                    int base_nbits, unsigned long long degree) {
  const unsigned n = 1u << nbits;
  const unsigned long long mask = n - 1;
  const int ratio_log = nbits - base_nbits;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    unsigned long long idx;
    if (ratio_log == 0) idx = j;
    else if (ratio_log == 1) idx = j < n / 2 ? 2ull * j : 2ull * (j - n / 2) + 1;
    else idx = bit_rev_twice_inv_dev(nbits, base_nbits, j);
    buf[j] = tw[(idx * degree) & mask];
  }
}

}  // namespace cfft

// ============================================================ plan object
struct C64Plan {
  size_t n = 0, base_n = 0;
  int base_algo = 0;
  bool unordered = false;
  LevelDesc lv{};
  DevLevels dlv{};
  double2* d_w = nullptr;
  double2* d_winv = nullptr;
  double2* d_mono = nullptr;
  int device = 0;
  int d0 = 0;        // first level handled in shared memory
  int threads = 128;  // CTA size of the shared-memory kernel
  int tpc = 1;       // sub-transforms per CTA
  int emu = 0;       // eighths of the butterfly additions issued on the integer pipe
  int cluster = 0;   // CTAs per transform: 0 automatic, 1 one CTA, 2/4/8 a cluster of that size
  bool block_set = false;  // block size chosen by the caller (no per-call change)
};

struct cfft_ordered_plan {
  C64Plan p;
};
struct cfft_unordered_plan {
  C64Plan p;
};

namespace {

DevLevels to_dev(const LevelDesc& l) {
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

// First level of at most 2048 points (measured, fwd+inv, Dif16 base 1024:
// n = 4096 x 4096 transforms 2527 vs 2864 us with 4096-point blocks; n = 32768
// x 512: 3195 vs 3530 us; n = 2^18 x 64: 3862 vs 4197 us).  Plans whose levels
// skip from above 4096 points to the base keep the first level of at most 4096.
int auto_block_level(const LevelDesc& lv) {
  int d = 0;
  while (lv.log2n[d] > kSmemLog2Max) ++d;
  if (lv.log2n[d] > kBlockLog2Auto && d < lv.nlevels) ++d;
  return d;
}

void default_launch(C64Plan& p) {
  const int log2sub = p.lv.log2n[p.d0];
  const size_t sub = size_t(1) << log2sub;
  const size_t pts = std::max<size_t>(sub, 1024);
  p.tpc = (int)(pts / sub);
  p.threads = (int)std::min<size_t>(256, std::max<size_t>(64, pts / 8));
}

size_t smem_bytes(const C64Plan& p) { return (size_t)2 * p.tpc * (size_t(1) << p.lv.log2n[p.d0]) * sizeof(double2); }

void free_plan(C64Plan& p) {
  if (p.d_w) cudaFree(p.d_w);
  if (p.d_winv) cudaFree(p.d_winv);
  if (p.d_mono) cudaFree(p.d_mono);
  p.d_w = p.d_winv = p.d_mono = nullptr;
}

int emu_level(const C64Plan& p) { return emu_level_for(p.base_algo, p.emu); }

cfft_status launch_smem(const C64Plan& p, bool fwd, int blocks, size_t smem, cudaStream_t stream, double2* data,
                        int nsub, const double2* w) {
  DevLevels L = p.dlv;
  int tpc = p.tpc, d0 = p.d0;
  void* args[] = {&data, &nsub, &tpc, &L, &d0, (void*)&w};
  const void* fn = c64_kernel(p.base_algo, p.emu, fwd);
  return launch_kernel(fn, blocks, p.threads, args, spread_smem(fn, blocks, p.threads, 1, smem), stream, true);
}

cfft_status build_plan(C64Plan& p, size_t n, size_t base_n, int algo, bool unordered) {
  p.n = n;
  p.base_n = base_n;
  p.base_algo = algo;
  p.unordered = unordered;
  CFFT_CUDA_TRY(cudaGetDevice(&p.device));
  cfft_status st = CFFT_OK;
  p.lv = make_levels(n, base_n);
  p.dlv = to_dev(p.lv);
  p.d0 = auto_block_level(p.lv);
  default_launch(p);
  const size_t len = n + base_n;
  std::vector<c64h> w(len), wi(len);
  unordered_twiddles(n, base_n, algo_radix(algo), w.data(), wi.data());
  st = upload((const double2*)w.data(), len, &p.d_w);
  if (st == CFFT_OK) st = upload((const double2*)wi.data(), len, &p.d_winv);
  if (st == CFFT_OK && unordered) {
    std::vector<c64h> mono(n);
    monomial_twiddles(n, mono.data());
    st = upload((const double2*)mono.data(), n, &p.d_mono);
  }
  if (st != CFFT_OK) free_plan(p);
  return st;
}

// CTAs per transform for a call, as a log2 (0: one CTA).  A transform is
// split over S = 2^ls CTAs (split.cuh) when the batch is too small to give
// every SM work, or as the plan forces.  Only plans whose transform fits one
// CTA whole (d0 == 0).  S is bounded by the radix of the step that is split
// (the base radix without outer levels, level 0's radix with them) and by 8;
// with one outer level of radix 2, 4 or 8 over a DIF base, by level 0's radix
// times the base classes (modes 2, 3 and 4), up to 16 CTAs for a batch whose
// CTAs fit the SMs one each, where one 16-CTA cluster fits the device.
int split_log2(const C64Plan& p, long batch, int* mode) {
  if (p.cluster == 1) return 0;
  const int log2n = p.lv.log2n[0];
  int max_ls, min_ls = 0;
  if (p.lv.nlevels == 0) {
    *mode = 0;
    const int lr = ilog2((size_t)algo_radix(p.base_algo));
    max_ls = std::min(3, std::min(lr, log2n - lr - 1));
  } else {
    *mode = 1;
    max_ls = std::min(3, p.lv.log2r[0]);
    // transforms larger than one CTA's shared memory: parts of at most 2^kSmemLog2Max points
    min_ls = std::max(0, log2n - kSmemLog2Max);
  }
  if (log2n < 6 || max_ls < 1 || min_ls > max_ls) return 0;
  // one outer level of radix 2, 4 or 8 over a DIF base: level 0's slices times
  // S1 = 2^ls1 classes of the base (c64_split2_kernel, modes 2, 3 and 4), with at
  // least 64 points per CTA and 32 butterflies per class pass, and not a radix-2
  // base under a radix-4 level
  int ls1 = 0;
  const int ls0 = p.lv.nlevels == 1 ? p.lv.log2r[0] : 0;
  // (a part is at most half the base, so it fits one CTA at every size)
  if (p.lv.nlevels == 1 && ls0 <= 3 && !(p.base_algo & 1)) {
    const int lr = ilog2((size_t)algo_radix(p.base_algo));
    const int log2m = p.lv.log2n[1];
    if (!(lr == 1 && ls0 > 1)) {
      for (int max_total = p.cluster == 0 && (batch << 4) <= (long)sm_count() ? 4 : 3; max_total >= 3; --max_total) {
        ls1 = std::max(0, std::min(max_total - ls0, lr));
        while (ls1 > 0 && (log2m - ls1 < 6 || log2m - ls1 - lr < 5)) --ls1;
        if (ls1 < 1 || ls0 + ls1 <= 3) break;
        // 16 CTAs: every transform's cluster resident at once, one CTA per SM, in
        // both directions (with one cluster more than fit, some SMs run two CTAs)
        const size_t part = p.n >> (ls0 + ls1);
        const int threads = (int)std::min<size_t>(256, std::max<size_t>(32, 2 * part / (size_t)(1 << lr)));
        const void* f = c64_split_kernel_ptr(p.base_algo, true, ls0 + ls1, 1 + ls0);
        const void* i = c64_split_kernel_ptr(p.base_algo, false, ls0 + ls1, 1 + ls0);
        if (f && i && batch <= spread_clusters(f, threads, 16) && batch <= spread_clusters(i, threads, 16)) break;
        ls1 = 0;
      }
    }
  }
  const long target = 4L * sm_count();
  if (p.cluster >= 2) {
    const int want = ilog2((size_t)p.cluster);
    if (want > max_ls && ls1 >= 1) {
      *mode = 1 + ls0;
      return ls0 + std::min(ls1, want - ls0);
    }
    return std::max(min_ls, std::min(max_ls, want));
  }
  // a small batch, up to 2 CTAs per SM: the most CTAs per transform.  fwd+inv of
  // 2048 points on Dif4/1024: batch 1 12.8 us on 8 CTAs, 28.1 on 2; batch 16 17.8 and
  // 28.1.  From 4 CTAs per SM it lost (4096 points, batch 64: 55.8 against 52.3 on 4)
  if (ls1 >= 1 && (batch << (ls0 + ls1)) <= 2L * sm_count()) {
    *mode = 1 + ls0;
    return ls0 + ls1;
  }
  if (min_ls > 0) {
    // transforms above one CTA's shared memory: a cluster of 8 SMs beats the global-level
    // path (all SMs, several launches) only up to 8192 points and for small batches
    // (measured, batch 1 fwd+inv: 37 vs 47 us at 8192, 70 vs 72 at 16384, 131 vs 123 at 32768)
    if (log2n > 13 || (batch << max_ls) >= target) return 0;
    return max_ls;
  }
  // without levels, keep at least 32 butterflies in each of a class's passes (64 for
  // DIT, one thread per butterfly), but split at least in two: with fewer butterflies
  // the CTAs idle (fwd+inv of 512 points on Dif8: 12.8 us on 2 CTAs, 19.2 on 8; 1024
  // points on Dif16: 24.9 on 2, 36.3 on 8), while the one-CTA kernel packs several
  // small transforms per CTA (256 points on Dit4, batch 16: 20.8 us, 12.9 on 2 CTAs)
  if (*mode == 0) {
    const int lr = ilog2((size_t)algo_radix(p.base_algo));
    const int min_lb = (p.base_algo & 1) ? 6 : 5;
    while (max_ls > 1 && log2n - max_ls - lr < min_lb) --max_ls;
  }
  int ls = 0;
  while (ls < max_ls && (batch << ls) < target) ++ls;
  return ls;
}

cfft_status launch_split(const C64Plan& p, bool fwd, int ls, int mode, long nsub, cudaStream_t stream,
                         double2* data) {
  const void* fn = c64_split_kernel_ptr(p.base_algo, fwd, ls, mode);
  const size_t part = p.n >> ls;
  const size_t smem = 2 * part * sizeof(double2);
  // one thread per butterfly of a pass over the part (more would idle at the barriers);
  // two for the DIF algorithms, whose passes split each butterfly into halves
  const int R = algo_radix(p.base_algo);
  const bool halves = (p.base_algo & 1) == 0;
  const int threads = (int)std::min<size_t>(256, std::max<size_t>(32, (halves ? 2 : 1) * part / (size_t)R));
  DevLevels L = p.dlv;
  const double2* w = fwd ? p.d_w : p.d_winv;
  void* args[] = {&data, &L, (void*)&w};
  if ((nsub << ls) > 0x7fffffffL) return fail(CFFT_ERR_INVALID_SIZE, "batch too large");
  const int grid = (int)(nsub << ls);
  return launch_kernel_cluster(fn, grid, threads, 1 << ls, args, spread_smem(fn, grid, threads, 1 << ls, smem),
                               stream, true);
}

cfft_status launch_level(bool fwd, double2* data, long total, int log2r, int log2nl, const double2* wl, int nsm,
                         cudaStream_t stream) {
  // fewer butterflies than 256 per SM: smaller CTAs, so that the level's FP64 work
  // spreads over the SMs (one forward of 16384 points on Dif8/512, a radix-8 level
  // in global memory, then 8 sub-transforms on clusters: 15.2 us with 256-thread
  // level CTAs, 12.3 us with 32-thread ones)
  int threads = 256;
  while (threads > 32 && (total + threads - 1) / threads < nsm) threads >>= 1;
  const int grid = (int)std::min<long>((total + threads - 1) / threads, (long)nsm * 16);
  void* args[] = {&data, &total, &log2r, &log2nl, (void*)&wl};
  const void* fn = fwd ? (const void*)c64_level_kernel<true> : (const void*)c64_level_kernel<false>;
  return launch_kernel(fn, grid, threads, args, 0, stream, true);
}

// The plan of the sub-transforms from level e on (levels e..L-1 over the same
// base), on the same device tables: after levels 0..e-1 every block of 2^log2n[e]
// consecutive points is one such transform.
C64Plan sub_plan(const C64Plan& p, int e) {
  C64Plan s = p;
  s.n = size_t(1) << p.lv.log2n[e];
  s.lv.nlevels = p.lv.nlevels - e;
  for (int i = 0; i <= kMaxLevels; ++i) {
    s.lv.log2n[i] = i + e <= kMaxLevels ? p.lv.log2n[i + e] : 0;
    s.lv.w_off[i] = i + e <= kMaxLevels ? p.lv.w_off[i + e] : 0;
  }
  for (int i = 0; i < kMaxLevels; ++i) {
    s.lv.log2r[i] = i + e < kMaxLevels ? p.lv.log2r[i + e] : 0;
    s.lv.winv_off[i] = i + e < kMaxLevels ? p.lv.winv_off[i + e] : 0;
  }
  s.dlv = to_dev(s.lv);
  s.d0 = 0;
  return s;
}

cfft_status run_plan(const C64Plan& plan, double* buf, size_t batch, bool fwd, cudaStream_t stream,
                     bool allow_split = true) {
  if (batch == 0) return CFFT_OK;
  if (buf == nullptr) return fail(CFFT_ERR_INVALID_ARGUMENT, "null buffer");
  if (plan.n == 1) return CFFT_OK;
  double2* data = (double2*)buf;
  const int log2n = plan.lv.log2n[0];
  int mode = 0;
  const int ls = allow_split ? split_log2(plan, (long)batch, &mode) : 0;
  if (ls > 0) return launch_split(plan, fwd, ls, mode, (long)batch, stream, data);
  const int nsm = sm_count();
  // Two or more levels over a DIF base and a small batch: the levels above the last
  // in global memory over all SMs, then every sub-transform (the last level over the
  // base) on a cluster, of its level-0 slices times the base's classes
  // (c64_split2_kernel) or of its slices, as split_log2 gives it (the levels take
  // small CTAs, spread over the SMs: launch_level)
  if (allow_split && plan.cluster == 0 && !plan.block_set && plan.lv.nlevels >= 2 && !(plan.base_algo & 1)) {
    int e = plan.lv.nlevels - 1;
    long nsub = (long)batch << (log2n - plan.lv.log2n[e]);
    C64Plan sub = sub_plan(plan, e);
    int smode = 0;
    int sls = split_log2(sub, nsub, &smode);
    {
      // or every level in global memory and the bases on clusters of their classes,
      // where that runs on more CTAs (one transform, fwd: 32768 points on Dif4/1024
      // 11.8 us against 13.3, 65536 points 16.1 against 20.9; 16384 points on
      // Dif8/512, 64 CTAs either way: 12.2 us with the sub-transforms' clusters,
      // 12.9 with the bases')
      const int eb = plan.lv.nlevels;
      const long nb = (long)batch << (log2n - plan.lv.log2n[eb]);
      const C64Plan bsub = sub_plan(plan, eb);
      int bmode = 0;
      const int bls = split_log2(bsub, nb, &bmode);
      const bool sub_ok = sls > 0 && (nsub << sls) <= 2L * nsm;
      if (bls > 0 && (nb << bls) <= 2L * nsm && (!sub_ok || (nb << bls) > (nsub << sls))) {
        e = eb;
        nsub = nb;
        sub = bsub;
        smode = bmode;
        sls = bls;
      }
    }
    // up to 2 CTAs per SM (one wave); larger batches keep the block path below
    if (sls > 0 && (nsub << sls) <= 2L * nsm) {
      if (!fwd) {
        cfft_status st = launch_split(sub, false, sls, smode, nsub, stream, data);
        if (st != CFFT_OK) return st;
      }
      for (int k = 0; k < e; ++k) {
        const int l = fwd ? k : e - 1 - k;
        cfft_status st = launch_level(fwd, data, ((long)batch << log2n) >> plan.lv.log2r[l], plan.lv.log2r[l],
                                      plan.lv.log2n[l],
                                      fwd ? plan.d_w + plan.lv.w_off[l] : plan.d_winv + plan.lv.winv_off[l], nsm,
                                      stream);
        if (st != CFFT_OK) return st;
      }
      if (fwd) return launch_split(sub, true, sls, smode, nsub, stream, data);
      return CFFT_OK;
    }
  }
  // A plan with levels in global memory and a batch whose blocks would cover
  // fewer than half the SMs takes smaller blocks for this call (one more level
  // in global memory, blocks of at least 512 points): one transform of 16384
  // points runs on 16 CTAs of 1024 points instead of 8 of 2048.
  int d = plan.d0;
  while (!plan.block_set && d > 0 && d < plan.lv.nlevels && plan.lv.log2n[d + 1] >= 9 &&
         ((long)batch << (log2n - plan.lv.log2n[d])) < nsm / 2)
    ++d;
  C64Plan deeper;
  if (d != plan.d0) {
    deeper = plan;
    deeper.d0 = d;
    default_launch(deeper);
  }
  const C64Plan& p = d != plan.d0 ? deeper : plan;
  const int log2sub = p.lv.log2n[p.d0];
  const long nsub = (long)batch << (log2n - log2sub);
  if (nsub > 0x7fffffffL * (long)p.tpc) return fail(CFFT_ERR_INVALID_SIZE, "batch too large");
  const int blocks = (int)((nsub + p.tpc - 1) / p.tpc);
  const size_t smem = smem_bytes(p);
  if (fwd) {
    for (int l = 0; l < p.d0; ++l) {
      cfft_status st = launch_level(true, data, ((long)batch << log2n) >> p.lv.log2r[l], p.lv.log2r[l],
                                    p.lv.log2n[l], p.d_w + p.lv.w_off[l], nsm, stream);
      if (st != CFFT_OK) return st;
    }
    cfft_status st = launch_smem(p, true, blocks, smem, stream, data, (int)nsub, p.d_w);
    if (st != CFFT_OK) return st;
  } else {
    cfft_status st = launch_smem(p, false, blocks, smem, stream, data, (int)nsub, p.d_winv);
    if (st != CFFT_OK) return st;
    for (int l = p.d0 - 1; l >= 0; --l) {
      st = launch_level(false, data, ((long)batch << log2n) >> p.lv.log2r[l], p.lv.log2r[l], p.lv.log2n[l],
                        p.d_winv + p.lv.winv_off[l], nsm, stream);
      if (st != CFFT_OK) return st;
    }
  }
  return CFFT_OK;
}

cfft_status run_host(const C64Plan& p, double* buf, size_t batch, bool fwd) {
  if (buf == nullptr) return fail(CFFT_ERR_INVALID_ARGUMENT, "null buffer");
  const size_t bytes = batch * p.n * sizeof(double2);
  void* d = nullptr;
  cudaStream_t s;
  // A page-locked buffer, and a transform that one kernel does whole (no level in
  // global memory): the kernel reads and writes the caller's memory in place,
  // across NVLink-C2C on a Grace host, with no staging copy.  From 16 transforms
  // on, one CTA per transform: the parts of a split transform each read the
  // whole transform, which over the link costs more than the split gains.
  void* mapped = mapped_host_range(buf, bytes);
  if (p.d0 == 0 && mapped) {
    cfft_status st = host_staging(0, &d, &s);
    if (st != CFFT_OK) return st;
    st = run_plan(p, (double*)mapped, batch, fwd, s, batch < 16);
    if (st != CFFT_OK) return st;
    CFFT_CUDA_TRY(cudaStreamSynchronize(s));
    return CFFT_OK;
  }
  // Pageable memory, up to 128 KiB: a CPU copy into the thread's page-locked bounce
  // buffer, then the page-locked path on it (in place, or copies at full DMA rate),
  // and a CPU copy back.  A pageable cudaMemcpy costs ~10 us of driver time each way:
  // one 1024-point transform through the slice API took 35.9 us, now 23.4 us.  Larger
  // buffers keep the driver's pageable copies, which overlap the CPU copy with the DMA
  // (65536 points: 68 us, against 143 us through the bounce buffer).
  if (!mapped && bytes <= (size_t(128) << 10)) {
    void *hb = nullptr, *db = nullptr;
    cfft_status st = host_bounce(bytes, &hb, &db);
    if (st != CFFT_OK) return st;
    st = host_staging(p.d0 == 0 ? 0 : bytes, &d, &s);
    if (st != CFFT_OK) return st;
    std::memcpy(hb, buf, bytes);
    if (p.d0 == 0) {
      st = run_plan(p, (double*)db, batch, fwd, s, batch < 16);
    } else {
      CFFT_CUDA_TRY(cudaMemcpyAsync(d, hb, bytes, cudaMemcpyHostToDevice, s));
      st = run_plan(p, (double*)d, batch, fwd, s);
      if (st == CFFT_OK) CFFT_CUDA_TRY(cudaMemcpyAsync(hb, d, bytes, cudaMemcpyDeviceToHost, s));
    }
    if (st != CFFT_OK) return st;
    CFFT_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(buf, hb, bytes);
    return CFFT_OK;
  }
  cfft_status st = host_staging(bytes, &d, &s);
  if (st != CFFT_OK) return st;
  CFFT_CUDA_TRY(cudaMemcpyAsync(d, buf, bytes, cudaMemcpyHostToDevice, s));
  st = run_plan(p, (double*)d, batch, fwd, s);
  if (st != CFFT_OK) return st;
  CFFT_CUDA_TRY(cudaMemcpyAsync(buf, d, bytes, cudaMemcpyDeviceToHost, s));
  CFFT_CUDA_TRY(cudaStreamSynchronize(s));
  return CFFT_OK;
}

// Average device time of one forward call over `batch` transforms (events on a private stream).
double time_forward(const C64Plan& p, double2* scratch, size_t batch, double seconds) {
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  run_plan(p, (double*)scratch, batch, true, s);  // warm-up
  int reps = 1;
  double per = 0.0;
  for (;;) {
    cudaEventRecord(e0, s);
    for (int i = 0; i < reps; ++i) run_plan(p, (double*)scratch, batch, true, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    per = ms * 1e-3 / reps;
    if (ms * 1e-3 >= std::max(seconds, 1e-3) || reps >= (1 << 20)) break;
    reps *= 2;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  return per;
}

// Method::Measure for one ordered size: the reference times its 8 algorithms
// (src/ordered.rs:99-180); here each algorithm, and then CTA shapes for the
// winner, are timed on the GPU over a batch large enough to fill every SM.
// *best_time receives the winner's score (seconds per transform, the two batches summed).
cfft_status measure_ordered(size_t n, double seconds, double2* scratch, size_t batch, int* best_algo,
                            int* best_threads, int* best_tpc, double* best_time) {
  // scored on a large batch and on one that fills the SMs about once (per-transform
  // times summed): the radix-4 algorithms tie at 4096 transforms of 1024 points, and
  // at 256 the split kernels decide (Dif4 37.6 against Dit4 41.5 us per fwd+inv)
  // A DIT winner gives way to the fastest DIF algorithm within 2%: the split
  // kernels of small batches are faster on DIF passes (half butterflies, and the
  // one-level class split), so near-ties go to them.
  const size_t small = std::min(batch, std::max<size_t>(1, 2 * (size_t)sm_count()));
  double t_algo[8];
  int threads_algo[8], tpc_algo[8];
  for (int algo = 0; algo < 8; ++algo) {
    C64Plan p;
    cfft_status st = build_plan(p, n, n, algo, false);
    if (st != CFFT_OK) return st;
    t_algo[algo] = time_forward(p, scratch, batch, seconds) / (double)batch +
                   time_forward(p, scratch, small, seconds) / (double)small;
    threads_algo[algo] = p.threads;
    tpc_algo[algo] = p.tpc;
    free_plan(p);
  }
  int best = 0;
  for (int algo = 1; algo < 8; ++algo)
    if (t_algo[algo] < t_algo[best]) best = algo;
  if (best & 1) {
    int dif = -1;
    for (int algo = 0; algo < 8; algo += 2)
      if (t_algo[algo] <= t_algo[best] * 1.02 && (dif < 0 || t_algo[algo] < t_algo[dif])) dif = algo;
    if (dif >= 0) best = dif;
  }
  *best_algo = best;
  *best_threads = threads_algo[best];
  *best_tpc = tpc_algo[best];
  *best_time = t_algo[best];
  return CFFT_OK;
}

cfft_status alloc_measure_scratch(size_t n, double2** scratch, size_t* batch) {
  *batch = std::max<size_t>(1, (size_t(1) << 22) / n);  // 64 MiB of c64
  CFFT_CUDA_TRY(cudaMalloc((void**)scratch, *batch * n * sizeof(double2)));
  CFFT_CUDA_TRY(cudaMemset(*scratch, 0, *batch * n * sizeof(double2)));
  return CFFT_OK;
}

// CTA-shape sweep for a fixed algorithm (the "threads per transform and
// transforms per CTA" part of the autotuner).
void tune_launch(C64Plan& p, double2* scratch, size_t batch, double seconds) {
  const int log2sub = p.lv.log2n[p.d0];
  const size_t sub = size_t(1) << log2sub;
  double best = time_forward(p, scratch, batch, seconds);
  int bt = p.threads, bp = p.tpc;
  for (size_t pts : {size_t(512), size_t(1024), size_t(2048), size_t(4096)}) {
    if (pts < sub) continue;
    for (int th : {64, 128, 256}) {
      C64Plan q = p;
      q.tpc = (int)(pts / sub);
      q.threads = th;
      if (smem_bytes(q) > (size_t)2 * (1 << kSmemLog2Max) * sizeof(double2)) continue;
      const double t = time_forward(q, scratch, batch, seconds);
      if (t < best) {
        best = t;
        bt = th;
        bp = q.tpc;
      }
    }
  }
  p.threads = bt;
  p.tpc = bp;
  int be = p.emu;
  for (int e : kEmuLevels) {
    if (emu_level_for(p.base_algo, e) != e) continue;
    C64Plan q = p;
    q.emu = e;
    const double t = time_forward(q, scratch, batch, seconds);
    if (t < best) {
      best = t;
      be = e;
    }
  }
  p.emu = be;
}

bool valid_algo(int a) { return a >= 0 && a <= 7; }

}  // namespace

// ================================================================= C ABI
extern "C" {

cfft_status cfft_ordered_plan_create(size_t n, cfft_algo algo, cfft_ordered_plan** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!is_pow2(n)) return fail(CFFT_ERR_INVALID_SIZE, "ordered plan: n must be a power of two");
  if (ilog2(n) >= 11) return fail(CFFT_ERR_INVALID_SIZE, "ordered plan: n must be at most 1024");
  if (!valid_algo(algo)) return fail(CFFT_ERR_INVALID_ARGUMENT, "unknown FftAlgo");
  auto* plan = new cfft_ordered_plan();
  cfft_status st = build_plan(plan->p, n, n, algo, false);
  if (st != CFFT_OK) {
    delete plan;
    return st;
  }
  *out = plan;
  return CFFT_OK;
}

cfft_status cfft_ordered_plan_create_measure(size_t n, double seconds, cfft_ordered_plan** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!is_pow2(n) || ilog2(n) >= 11) return fail(CFFT_ERR_INVALID_SIZE, "ordered plan: n must be 2^k, k <= 10");
  if (n == 1) return cfft_ordered_plan_create(n, CFFT_DIF2, out);
  TuneVal tv;
  if (tune_lookup(0, n, &tv)) {  // measured before on this GPU model
    cfft_status st = cfft_ordered_plan_create(n, (cfft_algo)tv.algo, out);
    if (st == CFFT_OK) {
      (*out)->p.threads = tv.threads;
      (*out)->p.tpc = tv.tpc;
      (*out)->p.emu = tv.emu;
    }
    return st;
  }
  double2* scratch = nullptr;
  size_t batch = 0;
  cfft_status st = alloc_measure_scratch(n, &scratch, &batch);
  int algo = 0, th = 128, tpc = 1;
  double t = 0;
  if (st == CFFT_OK) st = measure_ordered(n, seconds, scratch, batch, &algo, &th, &tpc, &t);
  if (st == CFFT_OK) st = cfft_ordered_plan_create(n, (cfft_algo)algo, out);
  if (st == CFFT_OK) {
    tune_launch((*out)->p, scratch, batch, seconds);
    const C64Plan& p = (*out)->p;
    tune_store(0, n, TuneVal{p.base_algo, p.base_n, p.threads, p.tpc, p.emu});
  }
  if (scratch) cudaFree(scratch);
  return st;
}

void cfft_ordered_plan_destroy(cfft_ordered_plan* plan) {
  if (!plan) return;
  free_plan(plan->p);
  delete plan;
}
size_t cfft_ordered_fft_size(const cfft_ordered_plan* plan) { return plan ? plan->p.n : 0; }
cfft_algo cfft_ordered_algo(const cfft_ordered_plan* plan) { return (cfft_algo)(plan ? plan->p.base_algo : 0); }
size_t cfft_ordered_scratch_bytes(const cfft_ordered_plan*) { return 0; }

cfft_status cfft_ordered_fwd(const cfft_ordered_plan* plan, double* buf, size_t batch, void* stream) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_plan(plan->p, buf, batch, true, (cudaStream_t)stream);
}
cfft_status cfft_ordered_inv(const cfft_ordered_plan* plan, double* buf, size_t batch, void* stream) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_plan(plan->p, buf, batch, false, (cudaStream_t)stream);
}
cfft_status cfft_ordered_fwd_host(const cfft_ordered_plan* plan, double* buf, size_t batch) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_host(plan->p, buf, batch, true);
}
cfft_status cfft_ordered_inv_host(const cfft_ordered_plan* plan, double* buf, size_t batch) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_host(plan->p, buf, batch, false);
}

cfft_status cfft_ordered_set_int_adds(cfft_ordered_plan* plan, int eighths) {
  if (!plan || eighths < 0 || eighths > 8) return fail(CFFT_ERR_INVALID_ARGUMENT, "eighths must be in 0..8");
  plan->p.emu = eighths;
  return CFFT_OK;
}
int cfft_ordered_int_adds(const cfft_ordered_plan* plan) { return plan ? emu_level(plan->p) : -1; }

cfft_status cfft_ordered_set_cluster_size(cfft_ordered_plan* plan, int ctas) {
  if (!plan || !(ctas == 0 || ctas == 1 || ctas == 2 || ctas == 4 || ctas == 8))
    return fail(CFFT_ERR_INVALID_ARGUMENT, "cluster size must be 0 (automatic), 1, 2, 4 or 8");
  plan->p.cluster = ctas;
  return CFFT_OK;
}

cfft_status cfft_unordered_set_cluster_size(cfft_unordered_plan* plan, int ctas) {
  if (!plan || !(ctas == 0 || ctas == 1 || ctas == 2 || ctas == 4 || ctas == 8))
    return fail(CFFT_ERR_INVALID_ARGUMENT, "cluster size must be 0 (automatic), 1, 2, 4 or 8");
  plan->p.cluster = ctas;
  return CFFT_OK;
}

cfft_status cfft_unordered_set_block_points(cfft_unordered_plan* plan, size_t points) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  C64Plan& p = plan->p;
  int d = points == 0 ? auto_block_level(p.lv) : -1;
  for (int l = 0; d < 0 && l <= p.lv.nlevels; ++l)
    if ((size_t(1) << p.lv.log2n[l]) == points && p.lv.log2n[l] <= kSmemLog2Max) d = l;
  if (d < 0) return fail(CFFT_ERR_INVALID_ARGUMENT, "block points must be 0 or a level size of at most 4096 points");
  p.d0 = d;
  p.block_set = points != 0;
  default_launch(p);
  return CFFT_OK;
}
size_t cfft_unordered_block_points(const cfft_unordered_plan* plan) {
  return plan ? size_t(1) << plan->p.lv.log2n[plan->p.d0] : 0;
}

cfft_status cfft_unordered_set_int_adds(cfft_unordered_plan* plan, int eighths) {
  if (!plan || eighths < 0 || eighths > 8) return fail(CFFT_ERR_INVALID_ARGUMENT, "eighths must be in 0..8");
  plan->p.emu = eighths;
  return CFFT_OK;
}
int cfft_unordered_int_adds(const cfft_unordered_plan* plan) { return plan ? emu_level(plan->p) : -1; }

cfft_status cfft_unordered_plan_create(size_t n, cfft_algo base_algo, size_t base_n, cfft_unordered_plan** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!is_pow2(n)) return fail(CFFT_ERR_INVALID_SIZE, "unordered plan: n must be a power of two");
  if (ilog2(n) > kUnorderedMaxLog2) return fail(CFFT_ERR_INVALID_SIZE, "unordered plan: n must be at most 2^28");
  if (!is_pow2(base_n)) return fail(CFFT_ERR_INVALID_ARGUMENT, "base_n must be a power of two");
  if (base_n > n) return fail(CFFT_ERR_INVALID_ARGUMENT, "base_n must not exceed n");
  if (base_n != n && base_n < 32) return fail(CFFT_ERR_INVALID_ARGUMENT, "base_n must be >= 32 when base_n != n");
  if (ilog2(base_n) > 10) return fail(CFFT_ERR_INVALID_ARGUMENT, "base_n must be at most 1024");
  if (!valid_algo(base_algo)) return fail(CFFT_ERR_INVALID_ARGUMENT, "unknown FftAlgo");
  auto* plan = new cfft_unordered_plan();
  cfft_status st = build_plan(plan->p, n, base_n, base_algo, true);
  if (st != CFFT_OK) {
    delete plan;
    return st;
  }
  *out = plan;
  return CFFT_OK;
}

// src/unordered.rs:540-640: n <= 256 measures the ordered algorithms at n;
// otherwise bases 512 and 1024 (those <= n), each with its fastest ordered
// algorithm, timed on the full unordered forward transform.
cfft_status cfft_unordered_plan_create_measure(size_t n, double seconds, cfft_unordered_plan** out) {
  if (!out) return fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *out = nullptr;
  if (!is_pow2(n) || ilog2(n) > kUnorderedMaxLog2)
    return fail(CFFT_ERR_INVALID_SIZE, "unordered plan: n must be 2^k, k <= 28");
  TuneVal tv;
  if (tune_lookup(1, n, &tv)) {  // measured before on this GPU model
    cfft_status st = cfft_unordered_plan_create(n, (cfft_algo)tv.algo, tv.base_n, out);
    if (st == CFFT_OK) {
      (*out)->p.threads = tv.threads;
      (*out)->p.tpc = tv.tpc;
      (*out)->p.emu = tv.emu;
    }
    return st;
  }
  double2* scratch = nullptr;
  size_t batch = 0;
  cfft_status st = alloc_measure_scratch(n, &scratch, &batch);
  if (st != CFFT_OK) return st;
  int best_algo = 0;
  size_t best_base = n;
  if (n <= 256) {
    int th, tpc;
    double t;
    st = measure_ordered(n, seconds, scratch, batch, &best_algo, &th, &tpc, &t);
  } else {
    double best = 1e30;
    for (size_t base : {size_t(512), size_t(1024)}) {
      if (n < base) break;
      double2* bs = nullptr;
      size_t bb = 0;
      st = alloc_measure_scratch(base, &bs, &bb);
      if (st != CFFT_OK) break;
      int algo = 0, th, tpc;
      double t;
      st = measure_ordered(base, seconds, bs, bb, &algo, &th, &tpc, &t);
      cudaFree(bs);
      if (st != CFFT_OK) break;
      C64Plan p;
      st = build_plan(p, n, base, algo, true);
      if (st != CFFT_OK) break;
      const double tu = time_forward(p, scratch, batch, seconds);
      free_plan(p);
      if (tu < best) {
        best = tu;
        best_algo = algo;
        best_base = base;
      }
    }
  }
  if (st == CFFT_OK) st = cfft_unordered_plan_create(n, (cfft_algo)best_algo, best_base, out);
  if (st == CFFT_OK) {
    tune_launch((*out)->p, scratch, batch, seconds);
    const C64Plan& p = (*out)->p;
    tune_store(1, n, TuneVal{p.base_algo, p.base_n, p.threads, p.tpc, p.emu});
  }
  cudaFree(scratch);
  return st;
}

void cfft_unordered_plan_destroy(cfft_unordered_plan* plan) {
  if (!plan) return;
  free_plan(plan->p);
  delete plan;
}
size_t cfft_unordered_fft_size(const cfft_unordered_plan* plan) { return plan ? plan->p.n : 0; }
void cfft_unordered_algo(const cfft_unordered_plan* plan, cfft_algo* base_algo, size_t* base_n) {
  if (!plan) return;
  if (base_algo) *base_algo = (cfft_algo)plan->p.base_algo;
  if (base_n) *base_n = plan->p.base_n;
}
size_t cfft_unordered_scratch_bytes(const cfft_unordered_plan*) { return 0; }

cfft_status cfft_unordered_fwd(const cfft_unordered_plan* plan, double* buf, size_t batch, void* stream) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_plan(plan->p, buf, batch, true, (cudaStream_t)stream);
}
cfft_status cfft_unordered_inv(const cfft_unordered_plan* plan, double* buf, size_t batch, void* stream) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_plan(plan->p, buf, batch, false, (cudaStream_t)stream);
}
cfft_status cfft_unordered_fwd_host(const cfft_unordered_plan* plan, double* buf, size_t batch) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_host(plan->p, buf, batch, true);
}
cfft_status cfft_unordered_inv_host(const cfft_unordered_plan* plan, double* buf, size_t batch) {
  if (!plan) return fail(CFFT_ERR_INVALID_ARGUMENT, "null plan");
  return run_host(plan->p, buf, batch, false);
}

cfft_status cfft_unordered_fwd_monomial(const cfft_unordered_plan* plan, size_t degree, double* buf, void* stream) {
  if (!plan || !buf) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (degree >= plan->p.n) return fail(CFFT_ERR_INVALID_ARGUMENT, "degree must be < fft size");
  const int nbits = ilog2(plan->p.n), bb = ilog2(plan->p.base_n);
  const int blocks = (int)std::min<size_t>((plan->p.n + 255) / 256, 1024);
  c64_monomial_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>((double2*)buf, plan->p.d_mono, nbits, bb,
                                                                 (unsigned long long)degree);
  CFFT_CHECK_LAUNCH();
  return CFFT_OK;
}

cfft_status cfft_unordered_fwd_monomial_host(const cfft_unordered_plan* plan, size_t degree, double* buf) {
  if (!plan || !buf) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  const size_t bytes = plan->p.n * sizeof(double2);
  void* d;
  cudaStream_t s;
  cfft_status st = host_staging(bytes, &d, &s);
  if (st != CFFT_OK) return st;
  // the kernel writes straight into page-locked memory: the caller's, or the
  // thread's bounce buffer for pageable memory up to 32 KiB (then one CPU copy; for
  // larger buffers the driver's pageable copy measured faster)
  void* out = mapped_host_range(buf, bytes);
  void* hb = nullptr;
  if (!out && bytes <= (size_t(32) << 10)) {
    st = host_bounce(bytes, &hb, &out);
    if (st != CFFT_OK) return st;
  }
  st = cfft_unordered_fwd_monomial(plan, degree, out ? (double*)out : (double*)d, s);
  if (st != CFFT_OK) return st;
  if (!out) CFFT_CUDA_TRY(cudaMemcpyAsync(buf, d, bytes, cudaMemcpyDeviceToHost, s));
  CFFT_CUDA_TRY(cudaStreamSynchronize(s));
  if (hb) std::memcpy(buf, hb, bytes);
  return CFFT_OK;
}

static cfft_status permute(const cfft_unordered_plan* plan, const double* src, double* dst, size_t batch,
                           cudaStream_t stream, bool to_std) {
  if (!plan || !src || !dst) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (src == dst) return fail(CFFT_ERR_INVALID_ARGUMENT, "permutation is out of place: src and dst must differ");
  if (batch == 0) return CFFT_OK;
  const long total = (long)(batch * plan->p.n);
  const int nbits = ilog2(plan->p.n), bb = ilog2(plan->p.base_n);
  if (nbits >= 6 && nbits <= 12) {
    // tiles of 2048 points (whole transforms; 4096 for n = 4096), one CTA each
    const int log2tile = std::max(nbits, std::min(11, nbits + ilog2(batch & (~batch + 1))));
    const long tiles = total >> log2tile;
    if (tiles > 0x7fffffffL) return fail(CFFT_ERR_INVALID_SIZE, "batch too large");
    const size_t smem = sizeof(double2) << log2tile;
    const void* fn = to_std ? (const void*)c64_permute_tile_kernel<true> : (const void*)c64_permute_tile_kernel<false>;
    const double2* s2 = (const double2*)src;
    double2* d2 = (double2*)dst;
    int nb = nbits, bbits = bb, lt = log2tile;
    void* args[] = {(void*)&s2, (void*)&d2, &nb, &bbits, &lt};
    return launch_kernel(fn, (int)tiles, 256, args, smem, stream);
  }
  const int grid = (int)std::min<long>((total + 255) / 256, (long)sm_count() * 16);
  if (to_std)
    c64_permute_kernel<true><<<grid, 256, 0, stream>>>((const double2*)src, (double2*)dst, total, nbits, bb);
  else
    c64_permute_kernel<false><<<grid, 256, 0, stream>>>((const double2*)src, (double2*)dst, total, nbits, bb);
  CFFT_CHECK_LAUNCH();
  return CFFT_OK;
}

cfft_status cfft_unordered_to_standard(const cfft_unordered_plan* plan, const double* permuted, double* standard,
                                       size_t batch, void* stream) {
  return permute(plan, permuted, standard, batch, (cudaStream_t)stream, true);
}
cfft_status cfft_unordered_from_standard(const cfft_unordered_plan* plan, const double* standard, double* permuted,
                                         size_t batch, void* stream) {
  return permute(plan, standard, permuted, batch, (cudaStream_t)stream, false);
}

static cfft_status permute_host(const cfft_unordered_plan* plan, const double* src, double* dst, size_t batch,
                                bool to_std) {
  if (!plan || !src || !dst) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  const size_t bytes = batch * plan->p.n * sizeof(double2);
  void* d;
  cudaStream_t s;
  cfft_status st = host_staging(2 * bytes, &d, &s);
  if (st != CFFT_OK) return st;
  double* din = (double*)d;
  double* dout = (double*)((char*)d + bytes);
  CFFT_CUDA_TRY(cudaMemcpyAsync(din, src, bytes, cudaMemcpyHostToDevice, s));
  st = permute(plan, din, dout, batch, s, to_std);
  if (st != CFFT_OK) return st;
  CFFT_CUDA_TRY(cudaMemcpyAsync(dst, dout, bytes, cudaMemcpyDeviceToHost, s));
  CFFT_CUDA_TRY(cudaStreamSynchronize(s));
  return CFFT_OK;
}
cfft_status cfft_unordered_to_standard_host(const cfft_unordered_plan* plan, const double* permuted, double* standard,
                                            size_t batch) {
  return permute_host(plan, permuted, standard, batch, true);
}
cfft_status cfft_unordered_from_standard_host(const cfft_unordered_plan* plan, const double* standard,
                                              double* permuted, size_t batch) {
  return permute_host(plan, standard, permuted, batch, false);
}

// Host standard order <-> device permuted order in one call.  Page-locked host
// memory is read (or written) by the permutation kernel itself, on `stream`,
// asynchronously; pageable memory is staged through a device buffer on
// `stream` and the call returns when the copy is done.
cfft_status cfft_unordered_from_standard_h2d(const cfft_unordered_plan* plan, const double* standard,
                                             double* permuted, size_t batch, void* stream) {
  if (!plan || !standard || !permuted) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (batch == 0) return CFFT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = batch * plan->p.n * sizeof(double2);
  if (const void* m = mapped_host_range(standard, bytes)) return permute(plan, (const double*)m, permuted, batch, s, false);
  void* d;
  cudaStream_t own;
  cfft_status st = host_staging(bytes, &d, &own);
  if (st != CFFT_OK) return st;
  CFFT_CUDA_TRY(cudaStreamSynchronize(own));
  CFFT_CUDA_TRY(cudaMemcpyAsync(d, standard, bytes, cudaMemcpyHostToDevice, s));
  st = permute(plan, (const double*)d, permuted, batch, s, false);
  if (st != CFFT_OK) return st;
  CFFT_CUDA_TRY(cudaStreamSynchronize(s));  // the staging buffer is free again
  return CFFT_OK;
}
cfft_status cfft_unordered_to_standard_d2h(const cfft_unordered_plan* plan, const double* permuted, double* standard,
                                           size_t batch, void* stream) {
  if (!plan || !standard || !permuted) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (batch == 0) return CFFT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = batch * plan->p.n * sizeof(double2);
  if (void* m = mapped_host_range(standard, bytes)) return permute(plan, permuted, (double*)m, batch, s, true);
  void* d;
  cudaStream_t own;
  cfft_status st = host_staging(bytes, &d, &own);
  if (st != CFFT_OK) return st;
  CFFT_CUDA_TRY(cudaStreamSynchronize(own));
  st = permute(plan, permuted, (double*)d, batch, s, true);
  if (st != CFFT_OK) return st;
  CFFT_CUDA_TRY(cudaMemcpyAsync(standard, d, bytes, cudaMemcpyDeviceToHost, s));
  CFFT_CUDA_TRY(cudaStreamSynchronize(s));
  return CFFT_OK;
}

}  // extern "C"
