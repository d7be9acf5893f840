// cfft_internal.h -- host-side internals shared by the library's translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cfft.h"

namespace cfft {

struct c64h {
  double re, im;
};

// ---- twiddle generation (twiddles.cpp; host, no FMA contraction) ----
void sincospi64(double a, double* s, double* c);
// src/fft_simd.rs:298-321: 2n entries each
void init_wt(int r, size_t n, c64h* w, c64h* w_inv);
// src/unordered.rs:349-389 (complex_per_reg = 1 layout): n + base_n entries each
void unordered_twiddles(size_t n, size_t base_n, int base_r, c64h* w, c64h* w_inv);
// src/unordered.rs:694-699: monomial twiddles exp(-2 pi i k / n)
void monomial_twiddles(size_t n, c64h* tw);
// src/fft128/mod.rs:1805-1828: n entries each
void f128_twiddles(size_t n, double* re0, double* re1, double* im0, double* im1);
// u64 product twist tables: tw[j] = exp(i pi j / N), itw[j] = conj(tw[j]) / (N/2), j < N/2
void product_twist_tables(size_t N, c64h* tw, c64h* itw);
// Runs f(begin, end) over [0, count) on up to 16 host threads for large tables
// (every entry is computed independently, so the bits do not depend on the split).
void parallel_range(size_t count, void (*f)(size_t, size_t, void*), void* ctx);

// Largest transforms accepted (the reference has no upper bound): 2^28 c64
// points (4 GiB) per unordered transform, 2^24 points (512 MiB) per fft128
// transform.  The level descriptors hold 8 outer levels, enough for 2^28 over
// the smallest base (32 points).
constexpr int kUnorderedMaxLog2 = 28;
constexpr int kF128MaxLog2 = 24;

inline bool is_pow2(size_t n) { return n != 0 && (n & (n - 1)) == 0; }
inline int ilog2(size_t n) {
  int l = 0;
  while ((size_t(1) << l) < n) ++l;
  return l;
}
inline int algo_radix(int algo) { return 2 << (algo / 2); }
inline int outer_radix(size_t n, size_t base_n) { return n == 2 * base_n ? 2 : (n == 4 * base_n ? 4 : 8); }

// Level structure of an unordered plan: sizes n_0 = n > n_1 > ... > n_L = base_n.
constexpr int kMaxLevels = 8;
struct LevelDesc {
  int nlevels;                 // L
  int log2n[kMaxLevels + 1];   // log2 of n_l, l = 0..L (n_L = base_n)
  int log2r[kMaxLevels];       // outer radix of level l
  int w_off[kMaxLevels + 1];   // forward table offset of level l (l = L: base table)
  int winv_off[kMaxLevels];    // inverse table offset of level l (the base table is at 0)
};
LevelDesc make_levels(size_t n, size_t base_n);

void set_error(const std::string& msg);

// Products from a device item array (one plan's N) on a thread-block cluster
// each (split_product.cuh), the largest the plan allows.
cfft_status u64_product_split_items(const cfft_u64_product_plan* plan, const cfft_product_item* items, size_t count,
                                    void* stream);
bool u64_product_splittable(const cfft_u64_product_plan* plan);
// The serving loop and the work queue, with an automatic cluster threshold: a launch
// of at most this many products runs every product whose plan has a cluster kernel on
// a cluster (up to 8 CTAs each, so the launch still has an SM per CTA); a larger one
// only the products of N >= 8192.
constexpr size_t kClusterAllItems = 12;
// Device tables of a u64 product plan (forward/inverse FFT tables, twist, untwist).
void u64_product_tables(const cfft_u64_product_plan* p, const void** w, const void** winv, const void** tw,
                        const void** itw);

// The largest (sub)transform kept entirely in one CTA's shared memory
// (data + ping-pong scratch, 16 B per point each: 128 KiB at 4096 points).
constexpr int kSmemLog2Max = 12;
// The block size chosen automatically: 4096 points leave one CTA (8 warps) per
// SM, too few to keep the FP64 pipe busy; blocks of at most 2048 points after
// one more level in global memory, or two CTAs of a cluster, measured 8-27%
// faster at every batch size.
constexpr int kBlockLog2Auto = 11;

}  // namespace cfft
