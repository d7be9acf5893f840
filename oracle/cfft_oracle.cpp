// cfft_oracle.cpp -- scalar CPU restatement of concrete-fft v0.5.1 (test infrastructure).
//
// TEST INFRASTRUCTURE ONLY: the checker for tests/, smoke() and the CPU-baseline
// leg of bench.py.  The shipped library never links or loads this file.
//
// Every routine restates one function of the reference crate and cites it as
// path:line inside the crate.  The arithmetic is the reference's `Scalar`
// backend (src/fft_simd.rs:164-234): complex add/sub are two IEEE adds, the
// complex product is one FMA plus one multiply per component, and nothing is
// contracted or reassociated (this file must be compiled with
// -ffp-contract=off).  The reference's AVX2/AVX-512 backends produce the same
// bits (src/x86.rs:51-58 is the same FMA+MUL order; the golden vector at
// src/unordered.rs:1176-9395 is checked with assert_eq! on every backend).
#include "cfft_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace {

struct c64 {
  double re, im;
};

// ---------------------------------------------------------------- Scalar ops
// src/fft_simd.rs:209-233
inline c64 add(c64 a, c64 b) { return {a.re + b.re, a.im + b.im}; }
inline c64 sub(c64 a, c64 b) { return {a.re - b.re, a.im - b.im}; }
inline c64 mul(c64 ab, c64 xy) {
  return {std::fma(ab.re, xy.re, -(ab.im * xy.im)), std::fma(ab.re, xy.im, ab.im * xy.re)};
}
inline c64 real_mul(double r, c64 v) { return {r * v.re, r * v.im}; }
// src/fft_simd.rs:106-119: conj flips the sign bit of im, swap exchanges re/im.
inline c64 mul_j(bool fwd, c64 v) { return fwd ? c64{-v.im, v.re} : c64{v.im, -v.re}; }

const double kFrac1Sqrt2 = 0.70710678118654752440;  // core::f64::consts::FRAC_1_SQRT_2
const double kH1X = 0.9238795325112867;             // cos(-pi/8), src/fft_simd.rs:49
const double kH1Y = -0.38268343236508984;           // sin(-pi/8), src/fft_simd.rs:52

// src/fft_simd.rs:121-160
inline c64 mul_exp_pi_over_8(bool fwd, c64 v) { return real_mul(kFrac1Sqrt2, add(v, mul_j(fwd, v))); }
inline c64 mul_exp_neg_pi_over_8(bool fwd, c64 v) { return mul_exp_pi_over_8(!fwd, v); }
inline c64 mul_exp_pi_over_16(bool fwd, c64 v) { return mul(fwd ? c64{kH1X, kH1Y} : c64{kH1X, -kH1Y}, v); }
inline c64 mul_exp_17pi_over_16(bool fwd, c64 v) {
  return mul(fwd ? c64{-kH1Y, -kH1X} : c64{-kH1Y, kH1X}, v);
}
inline c64 mul_exp_neg_pi_over_16(bool fwd, c64 v) { return mul_exp_pi_over_16(!fwd, v); }
inline c64 mul_exp_neg_17pi_over_16(bool fwd, c64 v) { return mul_exp_17pi_over_16(!fwd, v); }

// ------------------------------------------------------- butterfly kernels
// Radix-R DFT without twiddles ("last_butterfly" of each file).  The DIF
// passes multiply output k by w_k, the DIT passes multiply input k by w_k,
// and the end passes use the core alone.
// src/dif2.rs:108-115
inline void core2(bool, const c64* x, c64* o) {
  o[0] = add(x[0], x[1]);
  o[1] = sub(x[0], x[1]);
}
// src/dif4.rs:171-192
inline void core4(bool fwd, const c64* x, c64* o) {
  c64 apc = add(x[0], x[2]);
  c64 amc = sub(x[0], x[2]);
  c64 bpd = add(x[1], x[3]);
  c64 jbmd = mul_j(fwd, sub(x[1], x[3]));
  o[0] = add(apc, bpd);
  o[1] = sub(amc, jbmd);
  o[2] = sub(apc, bpd);
  o[3] = add(amc, jbmd);
}
// src/dif8.rs:311-352
inline void core8(bool fwd, const c64* x, c64* o) {
  c64 a04 = add(x[0], x[4]);
  c64 s04 = sub(x[0], x[4]);
  c64 a26 = add(x[2], x[6]);
  c64 js26 = mul_j(fwd, sub(x[2], x[6]));
  c64 a15 = add(x[1], x[5]);
  c64 s15 = sub(x[1], x[5]);
  c64 a37 = add(x[3], x[7]);
  c64 js37 = mul_j(fwd, sub(x[3], x[7]));
  c64 a04_p1_a26 = add(a04, a26);
  c64 s04_mj_s26 = sub(s04, js26);
  c64 a04_m1_a26 = sub(a04, a26);
  c64 s04_pj_s26 = add(s04, js26);
  c64 a15_p1_a37 = add(a15, a37);
  c64 w8_s15_mj_s37 = mul_exp_neg_pi_over_8(fwd, sub(s15, js37));
  c64 j_a15_m1_a37 = mul_j(fwd, sub(a15, a37));
  c64 v8_s15_pj_s37 = mul_exp_pi_over_8(fwd, add(s15, js37));
  o[0] = add(a04_p1_a26, a15_p1_a37);
  o[1] = add(s04_mj_s26, w8_s15_mj_s37);
  o[2] = sub(a04_m1_a26, j_a15_m1_a37);
  o[3] = sub(s04_pj_s26, v8_s15_pj_s37);
  o[4] = sub(a04_p1_a26, a15_p1_a37);
  o[5] = sub(s04_mj_s26, w8_s15_mj_s37);
  o[6] = add(a04_m1_a26, j_a15_m1_a37);
  o[7] = add(s04_pj_s26, v8_s15_pj_s37);
}
// src/dif16.rs:650-779
inline void core16(bool fwd, const c64* x, c64* o) {
  c64 a08 = add(x[0], x[8]), s08 = sub(x[0], x[8]);
  c64 a4c = add(x[4], x[12]), s4c = sub(x[4], x[12]);
  c64 a2a = add(x[2], x[10]), s2a = sub(x[2], x[10]);
  c64 a6e = add(x[6], x[14]), s6e = sub(x[6], x[14]);
  c64 a19 = add(x[1], x[9]), s19 = sub(x[1], x[9]);
  c64 a5d = add(x[5], x[13]), s5d = sub(x[5], x[13]);
  c64 a3b = add(x[3], x[11]), s3b = sub(x[3], x[11]);
  c64 a7f = add(x[7], x[15]), s7f = sub(x[7], x[15]);

  c64 js4c = mul_j(fwd, s4c), js6e = mul_j(fwd, s6e), js5d = mul_j(fwd, s5d), js7f = mul_j(fwd, s7f);

  c64 a08p1a4c = add(a08, a4c), s08mjs4c = sub(s08, js4c);
  c64 a08m1a4c = sub(a08, a4c), s08pjs4c = add(s08, js4c);
  c64 a2ap1a6e = add(a2a, a6e), s2amjs6e = sub(s2a, js6e);
  c64 a2am1a6e = sub(a2a, a6e), s2apjs6e = add(s2a, js6e);
  c64 a19p1a5d = add(a19, a5d), s19mjs5d = sub(s19, js5d);
  c64 a19m1a5d = sub(a19, a5d), s19pjs5d = add(s19, js5d);
  c64 a3bp1a7f = add(a3b, a7f), s3bmjs7f = sub(s3b, js7f);
  c64 a3bm1a7f = sub(a3b, a7f), s3bpjs7f = add(s3b, js7f);

  c64 w8_s2amjs6e = mul_exp_neg_pi_over_8(fwd, s2amjs6e);
  c64 j_a2am1a6e = mul_j(fwd, a2am1a6e);
  c64 v8_s2apjs6e = mul_exp_pi_over_8(fwd, s2apjs6e);

  c64 e0 = add(a08p1a4c, a2ap1a6e);
  c64 e1 = add(s08mjs4c, w8_s2amjs6e);
  c64 e2 = sub(a08m1a4c, j_a2am1a6e);
  c64 e3 = sub(s08pjs4c, v8_s2apjs6e);
  c64 e4 = sub(a08p1a4c, a2ap1a6e);
  c64 e5 = sub(s08mjs4c, w8_s2amjs6e);
  c64 e6 = add(a08m1a4c, j_a2am1a6e);
  c64 e7 = add(s08pjs4c, v8_s2apjs6e);

  c64 w8_s3bmjs7f = mul_exp_neg_pi_over_8(fwd, s3bmjs7f);
  c64 j_a3bm1a7f = mul_j(fwd, a3bm1a7f);
  c64 v8_s3bpjs7f = mul_exp_pi_over_8(fwd, s3bpjs7f);

  c64 f0 = add(a19p1a5d, a3bp1a7f);
  c64 f1 = add(s19mjs5d, w8_s3bmjs7f);
  c64 f2 = sub(a19m1a5d, j_a3bm1a7f);
  c64 f3 = sub(s19pjs5d, v8_s3bpjs7f);
  c64 f4 = sub(a19p1a5d, a3bp1a7f);
  c64 f5 = sub(s19mjs5d, w8_s3bmjs7f);
  c64 f6 = add(a19m1a5d, j_a3bm1a7f);
  c64 f7 = add(s19pjs5d, v8_s3bpjs7f);

  c64 h1 = mul_exp_pi_over_16(fwd, f1);
  c64 w8 = mul_exp_neg_pi_over_8(fwd, f2);
  c64 h3 = mul_exp_17pi_over_16(fwd, f3);
  c64 j4 = mul_j(fwd, f4);
  c64 hd = mul_exp_neg_17pi_over_16(fwd, f5);
  c64 v8 = mul_exp_pi_over_8(fwd, f6);
  c64 hf = mul_exp_neg_pi_over_16(fwd, f7);

  o[0] = add(e0, f0);
  o[1] = add(e1, h1);
  o[2] = add(e2, w8);
  o[3] = add(e3, h3);
  o[4] = sub(e4, j4);
  o[5] = sub(e5, hd);
  o[6] = sub(e6, v8);
  o[7] = sub(e7, hf);
  o[8] = sub(e0, f0);
  o[9] = sub(e1, h1);
  o[10] = sub(e2, w8);
  o[11] = sub(e3, h3);
  o[12] = add(e4, j4);
  o[13] = add(e5, hd);
  o[14] = add(e6, v8);
  o[15] = add(e7, hf);
}

inline void core(int r, bool fwd, const c64* x, c64* o) {
  switch (r) {
    case 2: core2(fwd, x, o); break;
    case 4: core4(fwd, x, o); break;
    case 8: core8(fwd, x, o); break;
    default: core16(fwd, x, o); break;
  }
}

// ------------------------------------------------------ Stockham passes
// Generic DIF pass at stride s (src/dif4.rs:118-168 and its radix-2/8/16
// twins): inputs x[k*n/R + p*s + q], outputs y[R*s*p + k*s + q] = w_k * out_k,
// twiddle w_k = w[R*s*p + k] from the second half of the init_wt table.
void dif_pass(int R, bool fwd, size_t n, size_t s, const c64* x, c64* y, const c64* w) {
  const size_t m = n / (size_t)R;
  const size_t nchunks = m / s;
  c64 in[16], out[16];
  for (size_t p = 0; p < nchunks; ++p) {
    const c64* tw = w + (size_t)R * s * p;
    for (size_t q = 0; q < s; ++q) {
      for (int k = 0; k < R; ++k) in[k] = x[(size_t)k * m + p * s + q];
      core(R, fwd, in, out);
      c64* dst = y + (size_t)R * s * p + q;
      dst[0] = out[0];
      for (int k = 1; k < R; ++k) dst[(size_t)k * s] = mul(tw[k], out[k]);
    }
  }
}

// Generic DIT pass at stride s (src/dit4.rs:94-140 and twins): inputs
// y[R*s*p + k*s + q] times w_k, outputs x[k*n/R + p*s + q].
void dit_pass(int R, bool fwd, size_t n, size_t s, const c64* y, c64* x, const c64* w) {
  const size_t m = n / (size_t)R;
  const size_t nchunks = m / s;
  c64 in[16], out[16];
  for (size_t p = 0; p < nchunks; ++p) {
    const c64* tw = w + (size_t)R * s * p;
    for (size_t q = 0; q < s; ++q) {
      const c64* src = y + (size_t)R * s * p + q;
      in[0] = src[0];
      for (int k = 1; k < R; ++k) in[k] = mul(tw[k], src[(size_t)k * s]);
      core(R, fwd, in, out);
      for (int k = 0; k < R; ++k) x[(size_t)k * m + p * s + q] = out[k];
    }
  }
}

// End butterfly of size m at stride s = n/m, in place (src/dif2.rs:187-205,
// src/dif4.rs:195-244, src/dif8.rs:354-385, src/dif16.rs:781-827 and the DIT twins).
void end_pass(int m, bool fwd, size_t s, c64* x) {
  c64 in[16], out[16];
  for (size_t q = 0; q < s; ++q) {
    for (int k = 0; k < m; ++k) in[k] = x[(size_t)k * s + q];
    core(m, fwd, in, out);
    for (int k = 0; k < m; ++k) x[(size_t)k * s + q] = out[k];
  }
}

bool is_dit(int algo) { return (algo & 1) != 0; }
int radix_of(int algo) { return 2 << (algo / 2); }

bool is_pow2(size_t n) { return n != 0 && (n & (n - 1)) == 0; }
unsigned log2u(size_t n) {
  unsigned l = 0;
  while ((size_t(1) << l) < n) ++l;
  return l;
}

// The recursion of src/dif{R}.rs (e.g. src/dif4.rs:285-303): radix-R passes at
// s = 1, R, R^2, ... while the remaining size exceeds R, then an end butterfly
// of the remaining size (2, 4, 8 or 16).  DIT (src/dit4.rs:280-300) runs the
// same passes in reverse: end butterfly first at the largest stride.
void ordered_transform(int algo, bool fwd, size_t n, c64* x, c64* y, const c64* w) {
  if (n <= 1) return;  // src/ordered.rs:208-210 (do_nothing)
  const int R = radix_of(algo);
  size_t m = n;
  int npass = 0;
  while (m > (size_t)R) {
    m /= (size_t)R;
    ++npass;
  }
  c64* cur = x;
  c64* oth = y;
  if (!is_dit(algo)) {
    size_t s = 1;
    for (int i = 0; i < npass; ++i) {
      dif_pass(R, fwd, n, s, cur, oth, w);
      std::swap(cur, oth);
      s *= (size_t)R;
    }
    end_pass((int)m, fwd, s, cur);
  } else {
    size_t s_end = n / m;
    end_pass((int)m, fwd, s_end, cur);
    for (int i = npass - 1; i >= 0; --i) {
      size_t s = 1;
      for (int j = 0; j < i; ++j) s *= (size_t)R;
      dit_pass(R, fwd, n, s, cur, oth, w);
      std::swap(cur, oth);
    }
  }
  if (cur != x) std::memcpy(x, cur, n * sizeof(c64));
}

// ------------------------------------------------------------- twiddles
// src/fft_simd.rs:236-296 (the published sincospi of StackOverflow answer
// 42792940, cited by the reference); every step is IEEE double, no contraction.
void sincospi64(double a, double* sp, double* cp) {
  const double az = a * 0.0;
  a = (std::fabs(a) < 9007199254740992.0) ? a : az;
  double r = std::round(a + a);
  const int64_t i = (int64_t)r;
  const double t = std::fma(-0.5, r, a);
  const double s = t * t;
  r = -1.0369917389758117e-4;
  r = std::fma(r, s, 1.9294935641298806e-3);
  r = std::fma(r, s, -2.5806887942825395e-2);
  r = std::fma(r, s, 2.3533063028328211e-1);
  r = std::fma(r, s, -1.3352627688538006e+0);
  r = std::fma(r, s, 4.0587121264167623e+0);
  r = std::fma(r, s, -4.9348022005446790e+0);
  double c = std::fma(r, s, 1.0000000000000000e+0);
  r = 4.6151442520157035e-4;
  r = std::fma(r, s, -7.3700183130883555e-3);
  r = std::fma(r, s, 8.2145868949323936e-2);
  r = std::fma(r, s, -5.9926452893214921e-1);
  r = std::fma(r, s, 2.5501640398732688e+0);
  r = std::fma(r, s, -5.1677127800499516e+0);
  const double st = s * t;
  r *= st;
  double sn = std::fma(t, 3.1415926535897931e+0, r);
  if ((i & 2) != 0) {
    sn = 0.0 - sn;
    c = 0.0 - c;
  }
  if ((i & 1) != 0) {
    const double tt = 0.0 - sn;
    sn = c;
    c = tt;
  }
  if (a == std::floor(a)) sn = az;
  *sp = sn;
  *cp = c;
}

// src/fft_simd.rs:298-321
void init_wt(int r, size_t n, c64* w, c64* w_inv) {
  if (n < (size_t)r) return;
  const size_t nr = n / (size_t)r;
  const double theta = -2.0 / (double)n;
  const double nan = std::nan("");
  for (size_t i = 0; i < 2 * n; ++i) w[i] = c64{nan, nan};
  for (size_t p = 0; p < nr; ++p) {
    for (int k = 1; k < r; ++k) {
      double s, c;
      sincospi64(theta * (double)((size_t)k * p), &s, &c);
      const c64 z{c, s};
      const c64 zc{c, -s};
      w[p + (size_t)k * nr] = z;
      w[n + (size_t)r * p + (size_t)k] = z;
      w_inv[p + (size_t)k * nr] = zc;
      w_inv[n + (size_t)r * p + (size_t)k] = zc;
    }
  }
}

// ------------------------------------------------------------ unordered
int outer_radix(size_t n, size_t base_n) { return n == 2 * base_n ? 2 : (n == 4 * base_n ? 4 : 8); }

// src/unordered.rs:349-389 with complex_per_reg = 1 (the Scalar layout; the
// SIMD layouts interleave the same values).
void unordered_twiddles(size_t n, size_t base_n, int base_r, c64* w, c64* w_inv, size_t len) {
  const double theta = 2.0 / (double)n;
  if (n <= base_n) {
    init_wt(base_r, n, w, w_inv);
    return;
  }
  const int r = outer_radix(n, base_n);
  const size_t m = n / (size_t)r;
  const size_t head = (size_t)(r - 1) * m;
  c64* w_cur = w;
  c64* w_next = w + head;
  c64* w_inv_next = w_inv;
  c64* w_inv_cur = w_inv + (len - head);
  for (size_t p = 0; p < m; ++p) {
    for (int k = 1; k < r; ++k) {
      double sk, ck;
      sincospi64(theta * (double)((size_t)k * p), &sk, &ck);
      const size_t idx = (size_t)(r - 1) * p + (size_t)(k - 1);
      w_cur[idx] = c64{ck, -sk};
      w_inv_cur[idx] = c64{ck, sk};
    }
  }
  unordered_twiddles(n / (size_t)r, base_n, base_r, w_next, w_inv_next, len - head);
}

// src/unordered.rs:24-219: the outer butterflies (forward: twiddle after, inverse: before).
void fwd_butterfly(int r, c64* z, const c64* w) {
  if (r == 2) {
    c64 z0 = z[0], z1 = z[1];
    z[0] = add(z0, z1);
    z[1] = mul(w[0], sub(z0, z1));
  } else if (r == 4) {
    c64 z0p2 = add(z[0], z[2]);
    c64 z0m2 = sub(z[0], z[2]);
    c64 z1p3 = add(z[1], z[3]);
    c64 jz1m3 = mul_j(true, sub(z[1], z[3]));
    z[0] = add(z0p2, z1p3);
    z[1] = mul(w[0], sub(z0m2, jz1m3));
    z[2] = mul(w[1], sub(z0p2, z1p3));
    z[3] = mul(w[2], add(z0m2, jz1m3));
  } else {
    c64 o[8];
    core8(true, z, o);
    z[0] = o[0];
    for (int k = 1; k < 8; ++k) z[k] = mul(w[k - 1], o[k]);
  }
}

void inv_butterfly(int r, c64* z, const c64* w) {
  if (r == 2) {
    c64 z0 = z[0];
    c64 z1 = mul(w[0], z[1]);
    z[0] = add(z0, z1);
    z[1] = sub(z0, z1);
  } else if (r == 4) {
    c64 z0 = z[0];
    c64 z1 = mul(w[0], z[1]);
    c64 z2 = mul(w[1], z[2]);
    c64 z3 = mul(w[2], z[3]);
    c64 z0p2 = add(z0, z2);
    c64 z0m2 = sub(z0, z2);
    c64 z1p3 = add(z1, z3);
    c64 jz1m3 = mul_j(false, sub(z1, z3));
    z[0] = add(z0p2, z1p3);
    z[1] = sub(z0m2, jz1m3);
    z[2] = sub(z0p2, z1p3);
    z[3] = add(z0m2, jz1m3);
  } else {
    c64 in[8], o[8];
    in[0] = z[0];
    for (int k = 1; k < 8; ++k) in[k] = mul(w[k - 1], z[k]);
    core8(false, in, o);
    for (int k = 0; k < 8; ++k) z[k] = o[k];
  }
}

const int kBitRev2[2] = {0, 1};
const int kBitRev4[4] = {0, 2, 1, 3};
const int kBitRev8[8] = {0, 4, 2, 6, 1, 5, 3, 7};
const int* bitrev_slots(int r) { return r == 2 ? kBitRev2 : (r == 4 ? kBitRev4 : kBitRev8); }

// src/unordered.rs:222-293: fwd_process_xR stores butterfly output k into slot
// bitrev(k); inv_process_xR reads butterfly input k from slot bitrev(k).
void fwd_process(int r, size_t n, c64* z, const c64* w) {
  const size_t m = n / (size_t)r;
  const int* br = bitrev_slots(r);
  c64 v[8];
  for (size_t i = 0; i < m; ++i) {
    for (int k = 0; k < r; ++k) v[k] = z[(size_t)k * m + i];
    fwd_butterfly(r, v, w + (size_t)(r - 1) * i);
    for (int k = 0; k < r; ++k) z[(size_t)br[k] * m + i] = v[k];
  }
}

void inv_process(int r, size_t n, c64* z, const c64* w) {
  const size_t m = n / (size_t)r;
  const int* br = bitrev_slots(r);
  c64 v[8];
  for (size_t i = 0; i < m; ++i) {
    for (int k = 0; k < r; ++k) v[k] = z[(size_t)br[k] * m + i];
    inv_butterfly(r, v, w + (size_t)(r - 1) * i);
    for (int k = 0; k < r; ++k) z[(size_t)k * m + i] = v[k];
  }
}

// src/unordered.rs:392-439
void fwd_depth(size_t n, c64* z, const c64* w, int base_algo, size_t base_n, c64* scratch) {
  if (n == base_n) {
    ordered_transform(base_algo, true, n, z, scratch, w + n);
    return;
  }
  const int r = outer_radix(n, base_n);
  const size_t m = n / (size_t)r;
  fwd_process(r, n, z, w);
  const c64* w_tail = w + (size_t)(r - 1) * m;
  for (int c = 0; c < r; ++c) fwd_depth(m, z + (size_t)c * m, w_tail, base_algo, base_n, scratch);
}

// src/unordered.rs:442-489 (w points at a table of length len)
void inv_depth(size_t n, c64* z, const c64* w, size_t len, int base_algo, size_t base_n, c64* scratch) {
  if (n == base_n) {
    ordered_transform(base_algo, false, n, z, scratch, w + n);
    return;
  }
  const int r = outer_radix(n, base_n);
  const size_t m = n / (size_t)r;
  const size_t head_len = len - (size_t)(r - 1) * m;
  for (int c = 0; c < r; ++c) inv_depth(m, z + (size_t)c * m, w, head_len, base_algo, base_n, scratch);
  inv_process(r, n, z, w + head_len);
}

// src/unordered.rs:1040-1059
size_t bit_rev(unsigned nbits, size_t i) {
  size_t r = 0;
  for (unsigned b = 0; b < nbits; ++b) r |= ((i >> b) & 1u) << (nbits - 1 - b);
  return r;
}

bool unordered_args_ok(size_t n, size_t base_n) {
  if (!is_pow2(n) || !is_pow2(base_n) || base_n > n) return false;
  if (base_n != n && base_n < 32) return false;  // src/unordered.rs:663-670
  if (log2u(base_n) > 10) return false;
  return true;
}

// ------------------------------------------------------------ fft128
struct f128 {
  double hi, lo;
};

// src/fft128/f128_ops.rs:3-40
inline void quick_two_sum(double a, double b, double* s, double* e) {
  const double ss = a + b;
  *s = ss;
  *e = b - (ss - a);
}
inline void two_sum(double a, double b, double* s, double* e) {
  const double ss = a + b;
  const double bb = ss - a;
  *s = ss;
  *e = (a - (ss - bb)) + (b - bb);
}
inline void two_diff(double a, double b, double* s, double* e) {
  const double ss = a - b;
  const double bb = ss - a;
  *s = ss;
  *e = (a - (ss - bb)) - (b + bb);
}
inline void two_prod(double a, double b, double* p, double* e) {
  const double pp = a * b;
  *p = pp;
  *e = std::fma(a, b, -pp);
}

// src/fft128/f128_ops.rs:290-400
inline f128 add_f128_f64(f128 a, double b) {
  double s1, s2;
  two_sum(a.hi, b, &s1, &s2);
  s2 = s2 + a.lo;
  quick_two_sum(s1, s2, &s1, &s2);
  return {s1, s2};
}
inline f128 add_estimate(f128 a, f128 b) {
  double s, e;
  two_sum(a.hi, b.hi, &s, &e);
  e = e + (a.lo + b.lo);
  quick_two_sum(s, e, &s, &e);
  return {s, e};
}
inline f128 add_f128(f128 a, f128 b) {
  double s1, s2, t1, t2;
  two_sum(a.hi, b.hi, &s1, &s2);
  two_sum(a.lo, b.lo, &t1, &t2);
  s2 = s2 + t1;
  quick_two_sum(s1, s2, &s1, &s2);
  s2 = s2 + t2;
  quick_two_sum(s1, s2, &s1, &s2);
  return {s1, s2};
}
inline f128 sub_f128_f64(f128 a, double b) {
  double s1, s2;
  two_diff(a.hi, b, &s1, &s2);
  s2 = s2 + a.lo;
  quick_two_sum(s1, s2, &s1, &s2);
  return {s1, s2};
}
inline f128 sub_estimate(f128 a, f128 b) {
  double s, e;
  two_diff(a.hi, b.hi, &s, &e);
  e = e + a.lo;
  e = e - b.lo;
  quick_two_sum(s, e, &s, &e);
  return {s, e};
}
inline f128 sub_f128(f128 a, f128 b) {
  double s1, s2, t1, t2;
  two_diff(a.hi, b.hi, &s1, &s2);
  two_diff(a.lo, b.lo, &t1, &t2);
  s2 = s2 + t1;
  quick_two_sum(s1, s2, &s1, &s2);
  s2 = s2 + t2;
  quick_two_sum(s1, s2, &s1, &s2);
  return {s1, s2};
}
inline f128 mul_f128_f64(f128 a, double b) {
  double p1, p2;
  two_prod(a.hi, b, &p1, &p2);
  p2 = p2 + (a.lo * b);
  quick_two_sum(p1, p2, &p1, &p2);
  return {p1, p2};
}
inline f128 mul_f128(f128 a, f128 b) {
  double p1, p2;
  two_prod(a.hi, b.hi, &p1, &p2);
  p2 = p2 + (a.hi * b.lo + a.lo * b.hi);
  quick_two_sum(p1, p2, &p1, &p2);
  return {p1, p2};
}
inline f128 sqr_f128(f128 a) {
  double p1, p2;
  two_prod(a.hi, a.hi, &p1, &p2);
  p2 = p2 + 2.0 * (a.hi * a.lo);
  quick_two_sum(p1, p2, &p1, &p2);
  return {p1, p2};
}
// src/fft128/f128_ops.rs:473-486
inline f128 div_f128(f128 a, f128 b) {
  const double q1 = a.hi / b.hi;
  f128 r = sub_f128(a, mul_f128_f64(b, q1));
  const double q2 = r.hi / b.hi;
  r = sub_f128(r, mul_f128_f64(b, q2));
  const double q3 = r.hi / b.hi;
  double s, e;
  quick_two_sum(q1, q2, &s, &e);
  return add_f128_f64(f128{s, e}, q3);
}
inline f128 neg(f128 a) { return {-a.hi, -a.lo}; }

// The double-double constants of src/fft128/f128_ops.rs:581-620, regenerated
// from their definitions (pi^k/k! and sin/cos(k pi/16) at 1024 bits, split
// hi = round(x), lo = round(x - hi)) by oracle/gen_f128_constants.py; a CPU
// test checks them against the reference's literals.
#include "f128_constants.inc"

// src/fft128/f128_ops.rs:504-522
void sincospi_taylor(f128 x, f128* sin_out, f128* cos_out) {
  f128 sinc = kF128Pi;
  f128 cs = {1.0, 0.0};
  const f128 sq = sqr_f128(x);
  f128 pw = {1.0, 0.0};
  for (int i = 0; i < 9; ++i) {
    pw = mul_f128(pw, sq);
    sinc = add_f128(sinc, mul_f128(kSinPiTaylor[i], pw));
    cs = add_f128(cs, mul_f128(kCosPiTaylor[i], pw));
  }
  *sin_out = mul_f128(sinc, x);
  *cos_out = cs;
}

// src/fft128/f128_ops.rs:525-575 (inputs in [-1, 1])
int f128_sincospi(f128 x, f128* s_out, f128* c_out) {
  if (x.hi > 1.0 || (x.hi == 1.0 && x.lo > 0.0) || x.hi < -1.0 || (x.hi == -1.0 && x.lo < 0.0)) return -1;
  const double pd = std::round(x.hi * 2.0);
  f128 r = sub_f128_f64(x, pd * 0.5);
  const double qd = std::round(r.hi * 16.0);
  r = sub_f128_f64(r, qd * (1.0 / 16.0));
  const long p = (long)pd;
  const long q = (long)qd;
  const long q_abs = q < 0 ? -q : q;
  f128 sin_r, cos_r;
  sincospi_taylor(r, &sin_r, &cos_r);
  f128 s, c;
  if (q == 0) {
    s = sin_r;
    c = cos_r;
  } else {
    const f128 u = kCosKPiOver16[q_abs - 1];
    const f128 v = kSinKPiOver16[q_abs - 1];
    if (q > 0) {
      s = add_f128(mul_f128(u, sin_r), mul_f128(v, cos_r));
      c = sub_f128(mul_f128(u, cos_r), mul_f128(v, sin_r));
    } else {
      s = sub_f128(mul_f128(u, sin_r), mul_f128(v, cos_r));
      c = add_f128(mul_f128(u, cos_r), mul_f128(v, sin_r));
    }
  }
  if (p == 0) {
    *s_out = s;
    *c_out = c;
  } else if (p == 1) {
    *s_out = c;
    *c_out = neg(s);
  } else if (p == -1) {
    *s_out = neg(c);
    *c_out = s;
  } else {
    *s_out = neg(s);
    *c_out = neg(c);
  }
  return 0;
}

// src/fft128/mod.rs:285-349 with the Scalar backend (src/fft128/mod.rs:160-187):
// add/sub are the "estimate" variants, mul is mul_f128_f128.
inline void cplx_mul(f128 ar, f128 ai, f128 br, f128 bi, f128* or_, f128* oi) {
  const f128 rr = mul_f128(ar, br);
  const f128 ri = mul_f128(ar, bi);
  const f128 ir = mul_f128(ai, br);
  const f128 ii = mul_f128(ai, bi);
  *or_ = sub_estimate(rr, ii);
  *oi = add_estimate(ir, ri);
}
inline void cplx_mul_conj(f128 ar, f128 ai, f128 br, f128 bi, f128* or_, f128* oi) {
  const f128 rr = mul_f128(ar, br);
  const f128 ri = mul_f128(ar, bi);
  const f128 ir = mul_f128(ai, br);
  const f128 ii = mul_f128(ai, bi);
  *or_ = add_estimate(rr, ii);
  *oi = sub_estimate(ir, ri);
}

// src/fft128/mod.rs:1794-1802
size_t bitreverse_n(size_t i, size_t n) {
  const unsigned logn = log2u(n);
  size_t result = 0;
  for (unsigned k = 0; k < logn; ++k) result |= ((i >> k) & 1u) << (logn - k - 1);
  return result;
}

// src/fft128/mod.rs:352-402
void f128_fwd(size_t n, double* re0, double* re1, double* im0, double* im1, const double* tr0,
              const double* tr1, const double* ti0, const double* ti1) {
  size_t t = n, m = 1;
  while (m < n) {
    t /= 2;
    for (size_t i = 0; i < m; ++i) {
      const f128 wr{tr0[m + i], tr1[m + i]};
      const f128 wi{ti0[m + i], ti1[m + i]};
      const size_t start = 2 * i * t;
      for (size_t j = start; j < start + t; ++j) {
        const f128 z0r{re0[j], re1[j]}, z0i{im0[j], im1[j]};
        const f128 z1r{re0[j + t], re1[j + t]}, z1i{im0[j + t], im1[j + t]};
        f128 zwr, zwi;
        cplx_mul(z1r, z1i, wr, wi, &zwr, &zwi);
        const f128 ar = add_estimate(z0r, zwr), ai = add_estimate(z0i, zwi);
        const f128 sr = sub_estimate(z0r, zwr), si = sub_estimate(z0i, zwi);
        re0[j] = ar.hi; re1[j] = ar.lo; im0[j] = ai.hi; im1[j] = ai.lo;
        re0[j + t] = sr.hi; re1[j + t] = sr.lo; im0[j + t] = si.hi; im1[j + t] = si.lo;
      }
    }
    m *= 2;
  }
}

// src/fft128/mod.rs:1105-1155
void f128_inv(size_t n, double* re0, double* re1, double* im0, double* im1, const double* tr0,
              const double* tr1, const double* ti0, const double* ti1) {
  size_t t = 1, m = n;
  while (m > 1) {
    m /= 2;
    for (size_t i = 0; i < m; ++i) {
      const f128 wr{tr0[m + i], tr1[m + i]};
      const f128 wi{ti0[m + i], ti1[m + i]};
      const size_t start = 2 * i * t;
      for (size_t j = start; j < start + t; ++j) {
        const f128 z0r{re0[j], re1[j]}, z0i{im0[j], im1[j]};
        const f128 z1r{re0[j + t], re1[j + t]}, z1i{im0[j + t], im1[j + t]};
        const f128 dr = sub_estimate(z0r, z1r), di = sub_estimate(z0i, z1i);
        const f128 ar = add_estimate(z0r, z1r), ai = add_estimate(z0i, z1i);
        f128 mr, mi;
        cplx_mul_conj(dr, di, wr, wi, &mr, &mi);
        re0[j] = ar.hi; re1[j] = ar.lo; im0[j] = ai.hi; im1[j] = ai.lo;
        re0[j + t] = mr.hi; re1[j + t] = mr.lo; im0[j + t] = mi.hi; im1[j + t] = mi.lo;
      }
    }
    t *= 2;
  }
}

// src/fft128/mod.rs:1805-1828
void f128_twiddles(size_t n, double* re0, double* re1, double* im0, double* im1) {
  re0[0] = re1[0] = im0[0] = im1[0] = 0.0;
  size_t m = 1;
  while (m < n) {
    for (size_t i = 0; i < m; ++i) {
      const size_t k = 2 * m + i;
      const size_t pos = m + i;
      const f128 th{(double)bitreverse_n(k, 2 * n) / (double)(2 * n), 0.0};
      f128 s, c;
      f128_sincospi(th, &s, &c);
      re0[pos] = c.hi;
      re1[pos] = c.lo;
      im0[pos] = s.hi;
      im1[pos] = s.lo;
    }
    m *= 2;
  }
}

// ------------------------------------------------------- integer rounding
// floor(x + 1/2) mod 2^64 for any finite double, using only the bit pattern.
uint64_t round_half_up_mod64(double x) {
  uint64_t bits;
  std::memcpy(&bits, &x, 8);
  const bool neg = (bits >> 63) != 0;
  const int bexp = (int)((bits >> 52) & 0x7ff);
  if (bexp == 0x7ff || bexp == 0) return 0;  // inf/nan and subnormals (|x| < 2^-1022) -> 0
  const uint64_t m = (bits & ((uint64_t(1) << 52) - 1)) | (uint64_t(1) << 52);
  const int e = bexp - 1075;  // x = m * 2^e
  uint64_t mag;
  if (e >= 0) {
    mag = e >= 64 ? 0 : (m << e);
    return neg ? (uint64_t)0 - mag : mag;
  }
  const int k = -e;
  if (k > 54) return 0;  // |x| < 2^-1
  const uint64_t half = uint64_t(1) << (k - 1);
  if (!neg) return (m + half) >> k;
  // floor(-M 2^-k + 1/2) = -ceil(M 2^-k - 1/2) = -((M + half - 1) >> k)
  mag = (m + half - 1) >> k;
  return (uint64_t)0 - mag;
}

typedef unsigned __int128 u128;
typedef __int128 i128;

// trunc(x) mod 2^128 for a finite double with integral value handled exactly.
u128 trunc_mod128(double x, double* frac) {
  const double t = std::trunc(x);
  *frac = x - t;  // exact
  uint64_t bits;
  std::memcpy(&bits, &t, 8);
  const bool neg = (bits >> 63) != 0;
  const int bexp = (int)((bits >> 52) & 0x7ff);
  if (bexp == 0x7ff || bexp == 0) return 0;
  const u128 m = (u128)((bits & ((uint64_t(1) << 52) - 1)) | (uint64_t(1) << 52));
  const int e = bexp - 1075;
  u128 mag;
  if (e >= 0)
    mag = e >= 128 ? 0 : (m << e);
  else
    mag = (-e) >= 64 ? 0 : (m >> (-e));
  return neg ? (u128)0 - mag : mag;
}

// floor(hi + lo + 1/2) mod 2^128, exact for any finite double-double.
u128 round_half_up_mod128(double hi, double lo) {
  double fh, fl;
  const u128 ih = trunc_mod128(hi, &fh);
  const u128 il = trunc_mod128(lo, &fl);
  double s, e;
  two_sum(fh, fl, &s, &e);  // s + e = fh + fl exactly, in (-2, 2)
  // floor(v + 1/2) for v = s + e in (-2, 2) counts the thresholds -3/2..3/2 reached.
  auto ge = [&](double c) { return s > c || (s == c && e >= 0.0); };
  const int f = -2 + (int)ge(-1.5) + (int)ge(-0.5) + (int)ge(0.5) + (int)ge(1.5);
  return ih + il + (u128)(i128)f;
}

// i128 -> double-double: hi = RNE(a), lo = RNE(a - hi) (the remainder is exact in i128).
f128 i128_to_f128(u128 a) {
  const double hi = (double)(i128)a;
  double fr;
  const u128 hi_int = trunc_mod128(hi, &fr);
  const i128 rem = (i128)(a - hi_int);
  return {hi, (double)rem};
}

// ------------------------------------------------------- product pipelines
// The u64 negacyclic product as the reference's caller builds it on
// unordered::Plan (the reference crate has no product code): fold the N real
// coefficients into N/2 complex ones, twist by tau^j = exp(i pi j / N), forward
// unordered FFT, pointwise product with the resident operand, inverse, untwist
// by conj(tau^j)/(N/2), round each component to the nearest integer mod 2^64.
struct U64Pipeline {
  size_t N, n, base_n;
  int base_algo;
  std::vector<c64> tw, itw, w, w_inv;
  U64Pipeline(size_t N_, int base_algo_, size_t base_n_)
      : N(N_), n(N_ / 2), base_n(base_n_), base_algo(base_algo_), tw(N_ / 2), itw(N_ / 2), w(N_ / 2 + base_n_),
        w_inv(N_ / 2 + base_n_) {
    const double inv_n = 1.0 / (double)n;
    for (size_t j = 0; j < n; ++j) {
      double s, c;
      sincospi64((double)j / (double)N, &s, &c);
      tw[j] = c64{c, s};
      itw[j] = c64{c * inv_n, -s * inv_n};
    }
    unordered_twiddles(n, base_n, radix_of(base_algo), w.data(), w_inv.data(), n + base_n);
  }
  void forward(c64* z, c64* scratch) const { fwd_depth(n, z, w.data(), base_algo, base_n, scratch); }
  void inverse(c64* z, c64* scratch) const {
    inv_depth(n, z, w_inv.data(), n + base_n, base_algo, base_n, scratch);
  }
};

void u64_product_one(const U64Pipeline& P, const uint64_t* a, const c64* bhat, uint64_t* out, c64* z,
                     c64* scratch) {
  const size_t n = P.n;
  for (size_t j = 0; j < n; ++j) {
    const c64 v{(double)(int64_t)a[j], (double)(int64_t)a[j + n]};
    z[j] = mul(P.tw[j], v);
  }
  P.forward(z, scratch);
  for (size_t k = 0; k < n; ++k) z[k] = mul(bhat[k], z[k]);
  P.inverse(z, scratch);
  for (size_t j = 0; j < n; ++j) {
    const c64 t = mul(P.itw[j], z[j]);
    out[j] = round_half_up_mod64(t.re);
    out[j + n] = round_half_up_mod64(t.im);
  }
}

struct U128Pipeline {
  size_t N, n;
  std::vector<double> t_re0, t_re1, t_im0, t_im1;
  explicit U128Pipeline(size_t N_) : N(N_), n(N_ / 2), t_re0(N_ / 2), t_re1(N_ / 2), t_im0(N_ / 2), t_im1(N_ / 2) {
    f128_twiddles(n, t_re0.data(), t_re1.data(), t_im0.data(), t_im1.data());
  }
};

// The u128 product around fft128::Plan, following the reference's own product
// test (src/fft128/mod.rs:1998-2058): fold re = x[i], im = x[i + N/2], forward,
// cplx_mul, scale both words by 2/N, inverse; then round hi+lo mod 2^128.
void u128_product_one(const U128Pipeline& P, const uint64_t* a, const double* bhat4, uint64_t* out,
                      double* ws /* 4n */) {
  const size_t n = P.n;
  double* re0 = ws;
  double* re1 = ws + n;
  double* im0 = ws + 2 * n;
  double* im1 = ws + 3 * n;
  for (size_t j = 0; j < n; ++j) {
    const u128 lo = (u128)a[2 * j] | ((u128)a[2 * j + 1] << 64);
    const u128 hi = (u128)a[2 * (j + n)] | ((u128)a[2 * (j + n) + 1] << 64);
    const f128 x = i128_to_f128(lo), y = i128_to_f128(hi);
    re0[j] = x.hi; re1[j] = x.lo; im0[j] = y.hi; im1[j] = y.lo;
  }
  f128_fwd(n, re0, re1, im0, im1, P.t_re0.data(), P.t_re1.data(), P.t_im0.data(), P.t_im1.data());
  const double factor = 2.0 / (double)P.N;
  const double* b_re0 = bhat4;
  const double* b_re1 = bhat4 + n;
  const double* b_im0 = bhat4 + 2 * n;
  const double* b_im1 = bhat4 + 3 * n;
  for (size_t k = 0; k < n; ++k) {
    f128 pr, pi;
    cplx_mul(f128{re0[k], re1[k]}, f128{im0[k], im1[k]}, f128{b_re0[k], b_re1[k]}, f128{b_im0[k], b_im1[k]}, &pr,
             &pi);
    re0[k] = pr.hi * factor;
    re1[k] = pr.lo * factor;
    im0[k] = pi.hi * factor;
    im1[k] = pi.lo * factor;
  }
  f128_inv(n, re0, re1, im0, im1, P.t_re0.data(), P.t_re1.data(), P.t_im0.data(), P.t_im1.data());
  for (size_t j = 0; j < n; ++j) {
    const u128 x = round_half_up_mod128(re0[j], re1[j]);
    const u128 y = round_half_up_mod128(im0[j], im1[j]);
    out[2 * j] = (uint64_t)x;
    out[2 * j + 1] = (uint64_t)(x >> 64);
    out[2 * (j + n)] = (uint64_t)y;
    out[2 * (j + n) + 1] = (uint64_t)(y >> 64);
  }
}

// A persistent pool of host threads for the batched calls (the CPU baseline runs
// many short batches; starting threads per call cost milliseconds).  One parallel
// region at a time: concurrent callers wait for the pool.  The work is cut into
// chunks that the caller and the workers take from a shared counter.
class HostPool {
 public:
  static HostPool& get() {
    static HostPool pool;
    return pool;
  }
  void run(size_t count, int nthreads, const std::function<void(size_t, size_t)>& f) {
    std::lock_guard<std::mutex> region(region_mu_);
    ensure_workers(nthreads - 1);
    const size_t nchunks = std::min<size_t>(count, (size_t)nthreads * 4);
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &f;
      count_ = count;
      nchunks_ = nchunks;
      next_.store(0);
      active_ = (int)std::min<size_t>(workers_.size(), (size_t)nthreads - 1);
      pending_ = active_;
      ++generation_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return pending_ == 0; });
    fn_ = nullptr;
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      quit_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  void work() {
    for (;;) {
      const size_t c = next_.fetch_add(1);
      if (c >= nchunks_) return;
      const size_t b = count_ * c / nchunks_, e = count_ * (c + 1) / nchunks_;
      if (b < e) (*fn_)(b, e);
    }
  }
  void ensure_workers(int n) {
    while ((int)workers_.size() < n) {
      const int id = (int)workers_.size();
      workers_.emplace_back([this, id] {
        uint64_t seen = 0;
        for (;;) {
          {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return quit_ || generation_ != seen; });
            if (quit_) return;
            seen = generation_;
            if (id >= active_) continue;
          }
          work();
          std::lock_guard<std::mutex> lk(mu_);
          if (--pending_ == 0) done_cv_.notify_all();
        }
      });
    }
  }
  std::mutex region_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  std::vector<std::thread> workers_;
  const std::function<void(size_t, size_t)>* fn_ = nullptr;
  size_t count_ = 0, nchunks_ = 0;
  std::atomic<size_t> next_{0};
  int active_ = 0, pending_ = 0;
  uint64_t generation_ = 0;
  bool quit_ = false;
};

template <class F>
void parallel_for(size_t count, int nthreads, F f) {
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  nthreads = (int)std::min<size_t>((size_t)nthreads, std::max<size_t>(count, 1));
  if (nthreads <= 1) {
    f(0, count);
    return;
  }
  const std::function<void(size_t, size_t)> fn = f;
  HostPool::get().run(count, nthreads, fn);
}

// ------------------------------------------------ rand 0.8 StdRng restatement
// StdRng = ChaCha12Rng (rand_chacha 0.3): 64-bit block counter in words 12-13,
// stream id 0 in words 14-15, keystream words consumed in order; next_u64 is
// (word[2i+1] << 32) | word[2i].  seed_from_u64 (rand_core 0.6) fills the
// 32-byte key with eight PCG32 outputs.  gen_range(0.0..1.0) for f64 is
// ((u64 >> 12) | 0x3FF0000000000000) as f64 - 1.0, times 1.0, plus 0.0.
inline uint32_t rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }
void chacha12_block(const uint32_t key[8], uint64_t counter, uint32_t out[16]) {
  uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                     key[4],      key[5],      key[6],      key[7],      (uint32_t)counter, (uint32_t)(counter >> 32),
                     0u,          0u};
  uint32_t x[16];
  std::memcpy(x, st, sizeof(x));
  auto qr = [&](int a, int b, int c, int d) {
    x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 16);
    x[c] += x[d]; x[b] ^= x[c]; x[b] = rotl32(x[b], 12);
    x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 8);
    x[c] += x[d]; x[b] ^= x[c]; x[b] = rotl32(x[b], 7);
  };
  for (int i = 0; i < 6; ++i) {
    qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15);
    qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14);
  }
  for (int i = 0; i < 16; ++i) out[i] = x[i] + st[i];
}

}  // namespace

// ============================================================== C ABI
extern "C" {

void oracle_sincospi64(double a, double* s, double* c) { sincospi64(a, s, c); }

int oracle_init_wt(int r, size_t n, double* w, double* w_inv) {
  if (!is_pow2(n) || (r != 2 && r != 4 && r != 8 && r != 16)) return -1;
  init_wt(r, n, (c64*)w, (c64*)w_inv);
  return 0;
}

int oracle_algo_radix(int algo) { return (algo < 0 || algo > 7) ? -1 : radix_of(algo); }

static int ordered_run(int algo, size_t n, double* buf, const double* tw, bool fwd) {
  if (algo < 0 || algo > 7 || !is_pow2(n) || log2u(n) > 16) return -1;
  std::vector<c64> scratch(n);
  ordered_transform(algo, fwd, n, (c64*)buf, scratch.data(), ((const c64*)tw) + n);
  return 0;
}
int oracle_ordered_fwd(int algo, size_t n, double* buf, const double* tw) { return ordered_run(algo, n, buf, tw, true); }
int oracle_ordered_inv(int algo, size_t n, double* buf, const double* tw) { return ordered_run(algo, n, buf, tw, false); }

int oracle_unordered_twiddles(size_t n, size_t base_n, int base_algo, double* w, double* w_inv) {
  if (!unordered_args_ok(n, base_n) || base_algo < 0 || base_algo > 7) return -1;
  const double nan = std::nan("");
  for (size_t i = 0; i < 2 * (n + base_n); ++i) w[i] = w_inv[i] = nan;
  unordered_twiddles(n, base_n, radix_of(base_algo), (c64*)w, (c64*)w_inv, n + base_n);
  return 0;
}

int oracle_unordered_fwd(int base_algo, size_t n, size_t base_n, double* buf, const double* w) {
  if (!unordered_args_ok(n, base_n) || base_algo < 0 || base_algo > 7) return -1;
  std::vector<c64> scratch(base_n);
  fwd_depth(n, (c64*)buf, (const c64*)w, base_algo, base_n, scratch.data());
  return 0;
}

int oracle_unordered_inv(int base_algo, size_t n, size_t base_n, double* buf, const double* w_inv) {
  if (!unordered_args_ok(n, base_n) || base_algo < 0 || base_algo > 7) return -1;
  std::vector<c64> scratch(base_n);
  inv_depth(n, (c64*)buf, (const c64*)w_inv, n + base_n, base_algo, base_n, scratch.data());
  return 0;
}

size_t oracle_bit_rev_twice(unsigned nbits, unsigned base_nbits, size_t i) {
  const size_t i_rev = bit_rev(nbits, i);
  const size_t bottom_mask = (size_t(1) << base_nbits) - 1;
  const size_t bottom_bits = bit_rev(base_nbits, i_rev);
  return (i_rev & ~bottom_mask) | bottom_bits;
}

size_t oracle_bit_rev_twice_inv(unsigned nbits, unsigned base_nbits, size_t i) {
  const size_t bottom_mask = (size_t(1) << base_nbits) - 1;
  const size_t bottom_bits = bit_rev(base_nbits, i);
  const size_t i_rev = (i & ~bottom_mask) | bottom_bits;
  return bit_rev(nbits, i_rev);
}

// src/unordered.rs:844-900
int oracle_unordered_fwd_monomial(size_t n, size_t base_n, size_t degree, double* buf) {
  if (!unordered_args_ok(n, base_n) || degree >= n) return -1;
  c64* z = (c64*)buf;
  const size_t mask = n - 1;
  const double theta = -2.0 / (double)n;
  std::vector<c64> tw(n);
  for (size_t i = 0; i < n; ++i) {
    double s, c;
    sincospi64(theta * (double)i, &s, &c);
    tw[i] = c64{c, s};
  }
  const unsigned nbits = log2u(n), base_nbits = log2u(base_n);
  const size_t ratio = n / base_n;
  if (ratio == 1) {
    for (size_t i = 0; i < n; ++i) z[i] = tw[(i * degree) & mask];
  } else if (ratio == 2) {
    for (size_t i = 0; i < n / 2; ++i) {
      z[i] = tw[((2 * i) * degree) & mask];
      z[i + n / 2] = tw[((2 * i + 1) * degree) & mask];
    }
  } else {
    for (size_t j = 0; j < n; ++j) z[j] = tw[(oracle_bit_rev_twice_inv(nbits, base_nbits, j) * degree) & mask];
  }
  return 0;
}

// src/unordered.rs:951-970 and :1019-1025
int oracle_unordered_to_standard(size_t n, size_t base_n, const double* permuted, double* standard) {
  if (!unordered_args_ok(n, base_n)) return -1;
  const unsigned nbits = log2u(n), bb = log2u(base_n);
  for (size_t i = 0; i < n; ++i) ((c64*)standard)[i] = ((const c64*)permuted)[oracle_bit_rev_twice(nbits, bb, i)];
  return 0;
}
int oracle_unordered_from_standard(size_t n, size_t base_n, const double* standard, double* permuted) {
  if (!unordered_args_ok(n, base_n)) return -1;
  const unsigned nbits = log2u(n), bb = log2u(base_n);
  for (size_t i = 0; i < n; ++i) ((c64*)permuted)[oracle_bit_rev_twice(nbits, bb, i)] = ((const c64*)standard)[i];
  return 0;
}

int oracle_f128_binop(int op, double a0, double a1, double b0, double b1, double* out2) {
  const f128 a{a0, a1}, b{b0, b1};
  f128 r;
  switch (op) {
    case 0: r = add_f128(a, b); break;
    case 1: r = sub_f128(a, b); break;
    case 2: r = mul_f128(a, b); break;
    case 3: r = add_estimate(a, b); break;
    case 4: r = sub_estimate(a, b); break;
    case 5: r = div_f128(a, b); break;
    case 6: r = sqr_f128(a); break;
    default: return -1;
  }
  out2[0] = r.hi;
  out2[1] = r.lo;
  return 0;
}

int oracle_f128_sincospi(double x0, double x1, double* s2, double* c2) {
  f128 s, c;
  if (f128_sincospi(f128{x0, x1}, &s, &c) != 0) return -1;
  s2[0] = s.hi; s2[1] = s.lo; c2[0] = c.hi; c2[1] = c.lo;
  return 0;
}

// Plan::new requires n >= 32 (src/fft128/mod.rs:1865-1866); the free functions
// init_negacyclic_twiddles and negacyclic_{fwd,inv}_fft_scalar (:1805, :352,
// :1105) take any power of two, as these entry points do.
int oracle_f128_twiddles(size_t n, double* re0, double* re1, double* im0, double* im1) {
  if (!is_pow2(n) || n < 2) return -1;
  f128_twiddles(n, re0, re1, im0, im1);
  return 0;
}

int oracle_f128_fwd(size_t n, double* re0, double* re1, double* im0, double* im1, const double* a, const double* b,
                    const double* c, const double* d) {
  if (!is_pow2(n) || n < 2) return -1;
  f128_fwd(n, re0, re1, im0, im1, a, b, c, d);
  return 0;
}
int oracle_f128_inv(size_t n, double* re0, double* re1, double* im0, double* im1, const double* a, const double* b,
                    const double* c, const double* d) {
  if (!is_pow2(n) || n < 2) return -1;
  f128_inv(n, re0, re1, im0, im1, a, b, c, d);
  return 0;
}

int oracle_negacyclic_u64_schoolbook(size_t N, const uint64_t* a, const int64_t* b, uint64_t* out) {
  if (!is_pow2(N)) return -1;
  std::vector<uint64_t> acc(N, 0);
  for (size_t i = 0; i < N; ++i) {
    const uint64_t ai = a[i];
    for (size_t j = 0; j < N; ++j) {
      const uint64_t p = ai * (uint64_t)b[j];
      const size_t k = i + j;
      if (k < N) acc[k] += p;
      else acc[k - N] -= p;
    }
  }
  std::memcpy(out, acc.data(), N * 8);
  return 0;
}

int oracle_negacyclic_u128_schoolbook(size_t N, const uint64_t* a, const int64_t* b, uint64_t* out) {
  if (!is_pow2(N)) return -1;
  std::vector<u128> acc(N, 0);
  for (size_t i = 0; i < N; ++i) {
    const u128 ai = (u128)a[2 * i] | ((u128)a[2 * i + 1] << 64);
    for (size_t j = 0; j < N; ++j) {
      const u128 p = ai * (u128)(i128)b[j];
      const size_t k = i + j;
      if (k < N) acc[k] += p;
      else acc[k - N] -= p;
    }
  }
  for (size_t k = 0; k < N; ++k) {
    out[2 * k] = (uint64_t)acc[k];
    out[2 * k + 1] = (uint64_t)(acc[k] >> 64);
  }
  return 0;
}

uint64_t oracle_round_mod64(double x) { return round_half_up_mod64(x); }

int oracle_u64_prepare_b(size_t N, int base_algo, size_t base_n, const int64_t* b, double* bhat) {
  if (!is_pow2(N) || N < 4 || !unordered_args_ok(N / 2, base_n) || base_algo < 0 || base_algo > 7) return -1;
  U64Pipeline P(N, base_algo, base_n);
  const size_t n = N / 2;
  c64* z = (c64*)bhat;
  for (size_t j = 0; j < n; ++j) z[j] = mul(P.tw[j], c64{(double)b[j], (double)b[j + n]});
  std::vector<c64> scratch(base_n);
  P.forward(z, scratch.data());
  return 0;
}

void oracle_c64_pointwise(size_t n, size_t count, const double* bhat, double* z) {
  const c64* b = (const c64*)bhat;
  c64* v = (c64*)z;
  for (size_t p = 0; p < count; ++p)
    for (size_t k = 0; k < n; ++k) v[p * n + k] = mul(b[k], v[p * n + k]);
}

int oracle_u64_product(size_t N, int base_algo, size_t base_n, const uint64_t* a, const double* bhat, uint64_t* out) {
  return oracle_u64_product_batch(N, base_algo, base_n, 1, a, bhat, out, 1);
}

int oracle_u64_product_batch(size_t N, int base_algo, size_t base_n, size_t count, const uint64_t* a,
                             const double* bhat, uint64_t* out, int nthreads) {
  if (!is_pow2(N) || N < 4 || !unordered_args_ok(N / 2, base_n) || base_algo < 0 || base_algo > 7) return -1;
  const U64Pipeline P(N, base_algo, base_n);
  const size_t n = N / 2;
  parallel_for(count, nthreads, [&](size_t b, size_t e) {
    std::vector<c64> z(n), scratch(base_n);
    for (size_t i = b; i < e; ++i)
      u64_product_one(P, a + i * N, ((const c64*)bhat) + i * n, out + i * N, z.data(), scratch.data());
  });
  return 0;
}

// Sum of `terms` products accumulated in the Fourier domain (the external
// product shape): acc = sum_t Bhat_t * fwd(twist(a_t)) in term order, then one
// inverse, untwist and rounding.  Groups are independent.
int oracle_u64_product_sum(size_t N, int base_algo, size_t base_n, size_t terms, size_t count, const uint64_t* a,
                           const double* bhat, uint64_t* out, int nthreads) {
  if (!is_pow2(N) || N < 4 || !unordered_args_ok(N / 2, base_n) || base_algo < 0 || base_algo > 7 || terms == 0)
    return -1;
  const U64Pipeline P(N, base_algo, base_n);
  const size_t n = N / 2;
  parallel_for(count, nthreads, [&](size_t b, size_t e) {
    std::vector<c64> z(n), acc(n), scratch(base_n);
    for (size_t g = b; g < e; ++g) {
      for (size_t t = 0; t < terms; ++t) {
        const uint64_t* at = a + (g * terms + t) * N;
        const c64* bt = ((const c64*)bhat) + (g * terms + t) * n;
        for (size_t j = 0; j < n; ++j) z[j] = mul(P.tw[j], c64{(double)(int64_t)at[j], (double)(int64_t)at[j + n]});
        P.forward(z.data(), scratch.data());
        for (size_t k = 0; k < n; ++k) {
          const c64 p = mul(bt[k], z[k]);
          acc[k] = t == 0 ? p : add(acc[k], p);
        }
      }
      P.inverse(acc.data(), scratch.data());
      uint64_t* og = out + g * N;
      for (size_t j = 0; j < n; ++j) {
        const c64 t = mul(P.itw[j], acc[j]);
        og[j] = round_half_up_mod64(t.re);
        og[j + n] = round_half_up_mod64(t.im);
      }
    }
  });
  return 0;
}

int oracle_u128_prepare_b(size_t N, const int64_t* b, double* bhat4) {
  if (!is_pow2(N) || N < 64) return -1;
  const U128Pipeline P(N);
  const size_t n = N / 2;
  double* re0 = bhat4;
  double* re1 = bhat4 + n;
  double* im0 = bhat4 + 2 * n;
  double* im1 = bhat4 + 3 * n;
  for (size_t j = 0; j < n; ++j) {
    re0[j] = (double)b[j]; re1[j] = 0.0; im0[j] = (double)b[j + n]; im1[j] = 0.0;
  }
  f128_fwd(n, re0, re1, im0, im1, P.t_re0.data(), P.t_re1.data(), P.t_im0.data(), P.t_im1.data());
  return 0;
}

int oracle_u128_product(size_t N, const uint64_t* a, const double* bhat4, uint64_t* out) {
  return oracle_u128_product_batch(N, 1, a, bhat4, out, 1);
}

int oracle_u128_product_batch(size_t N, size_t count, const uint64_t* a, const double* bhat4, uint64_t* out,
                              int nthreads) {
  if (!is_pow2(N) || N < 64) return -1;
  const U128Pipeline P(N);
  parallel_for(count, nthreads, [&](size_t b, size_t e) {
    std::vector<double> ws(2 * N);
    for (size_t i = b; i < e; ++i) u128_product_one(P, a + 2 * i * N, bhat4 + i * 2 * N, out + 2 * i * N, ws.data());
  });
  return 0;
}

int oracle_stdrng_uniform01(uint64_t seed, size_t count, double* out) {
  // rand_core 0.6 SeedableRng::seed_from_u64: PCG32 expansion of the seed.
  uint32_t key[8];
  uint64_t state = seed;
  for (int i = 0; i < 8; ++i) {
    state = state * 6364136223846793005ull + 11634580027462260723ull;
    const uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
    const uint32_t rot = (uint32_t)(state >> 59);
    key[i] = (xorshifted >> rot) | (xorshifted << ((32 - rot) & 31));
  }
  uint32_t block[16];
  uint64_t counter = 0;
  int idx = 16;
  for (size_t i = 0; i < count; ++i) {
    if (idx >= 16) {
      chacha12_block(key, counter++, block);
      idx = 0;
    }
    const uint64_t v = ((uint64_t)block[idx + 1] << 32) | block[idx];
    idx += 2;
    const uint64_t fbits = (v >> 12) | 0x3FF0000000000000ull;
    double f;
    std::memcpy(&f, &fbits, 8);
    out[i] = (f - 1.0) * 1.0 + 0.0;
  }
  return 0;
}

int oracle_ordered_batch(int fwd, int algo, size_t n, size_t count, double* bufs, const double* tw, int nthreads) {
  if (algo < 0 || algo > 7 || !is_pow2(n)) return -1;
  parallel_for(count, nthreads, [&](size_t b, size_t e) {
    std::vector<c64> scratch(n);
    for (size_t i = b; i < e; ++i)
      ordered_transform(algo, fwd != 0, n, ((c64*)bufs) + i * n, scratch.data(), ((const c64*)tw) + n);
  });
  return 0;
}

int oracle_unordered_batch(int fwd, int base_algo, size_t n, size_t base_n, size_t count, double* bufs,
                           const double* tw, int nthreads) {
  if (!unordered_args_ok(n, base_n) || base_algo < 0 || base_algo > 7) return -1;
  parallel_for(count, nthreads, [&](size_t b, size_t e) {
    std::vector<c64> scratch(base_n);
    for (size_t i = b; i < e; ++i) {
      c64* z = ((c64*)bufs) + i * n;
      if (fwd)
        fwd_depth(n, z, (const c64*)tw, base_algo, base_n, scratch.data());
      else
        inv_depth(n, z, (const c64*)tw, n + base_n, base_algo, base_n, scratch.data());
    }
  });
  return 0;
}

int oracle_f128_batch(int fwd, size_t n, size_t count, double* re0, double* re1, double* im0, double* im1,
                      const double* t_re0, const double* t_re1, const double* t_im0, const double* t_im1,
                      int nthreads) {
  if (!is_pow2(n) || n < 2) return -1;
  parallel_for(count, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      const size_t o = i * n;
      if (fwd)
        f128_fwd(n, re0 + o, re1 + o, im0 + o, im1 + o, t_re0, t_re1, t_im0, t_im1);
      else
        f128_inv(n, re0 + o, re1 + o, im0 + o, im1 + o, t_re0, t_re1, t_im0, t_im1);
    }
  });
  return 0;
}

int oracle_schoolbook_batch(int words, size_t N, size_t count, const uint64_t* a, const int64_t* b, uint64_t* out,
                            int nthreads) {
  if (!is_pow2(N) || (words != 1 && words != 2)) return -1;
  int bad = 0;
  parallel_for(count, nthreads, [&](size_t lo, size_t hi) {
    for (size_t i = lo; i < hi; ++i) {
      const int rc = words == 1
                         ? oracle_negacyclic_u64_schoolbook(N, a + i * N, b + i * N, out + i * N)
                         : oracle_negacyclic_u128_schoolbook(N, a + 2 * i * N, b + i * N, out + 2 * i * N);
      if (rc) bad = 1;
    }
  });
  return bad ? -1 : 0;
}

// Per-call CPU time of the restated reference, single-threaded, for the timed
// CPU baseline of the reference's own benchmark cases (benches/fft.rs): the
// call repeated `reps` times on one buffer, as a criterion loop does.
//   kind 0: ordered fwd (algo), 1: unordered fwd, 2: unordered inv (algo, base_n),
//   3: fwd_monomial (base_n; degree cycling as in the reference bench),
//   4: fft128 negacyclic fwd, 5: fft128 negacyclic inv.
int oracle_bench_call(int kind, int algo, size_t n, size_t base_n, size_t reps, double* ns_per_call) {
  if (!ns_per_call || !is_pow2(n) || reps == 0) return -1;
  if ((kind == 1 || kind == 2 || kind == 3) && !unordered_args_ok(n, base_n)) return -1;
  if (kind <= 2 && (algo < 0 || algo > 7)) return -1;
  if (kind == 0 && log2u(n) > 10) return -1;
  if (kind >= 4 && n < 2) return -1;
  std::vector<c64> buf(n, c64{0.0, 0.0}), scratch(std::max(n, base_n) + 1);
  for (size_t i = 0; i < n; ++i) buf[i] = c64{std::sin(0.1 * (double)i), std::cos(0.3 * (double)i)};
  std::vector<c64> w, wi;
  std::vector<double> f[4], t[4];
  std::vector<size_t> indices;
  std::vector<c64> mono;
  if (kind == 0) {
    w.assign(2 * n, c64{0, 0});
    wi.assign(2 * n, c64{0, 0});
    init_wt(radix_of(algo), n, w.data(), wi.data());
  } else if (kind <= 2) {
    w.assign(n + base_n, c64{0, 0});
    wi.assign(n + base_n, c64{0, 0});
    unordered_twiddles(n, base_n, radix_of(algo), w.data(), wi.data(), n + base_n);
  } else if (kind == 3) {
    mono.resize(n);
    const double theta = -2.0 / (double)n;
    for (size_t i = 0; i < n; ++i) {
      double sn, cs;
      sincospi64(theta * (double)i, &sn, &cs);
      mono[i] = c64{cs, sn};
    }
    indices.resize(n);
    for (size_t j = 0; j < n; ++j) indices[j] = oracle_bit_rev_twice_inv(log2u(n), log2u(base_n), j);
  } else {
    for (int k = 0; k < 4; ++k) {
      f[k].assign(n, 0.0);
      t[k].assign(n, 0.0);
    }
    for (size_t i = 0; i < n; ++i) {
      f[0][i] = std::sin(0.1 * (double)i);
      f[2][i] = std::cos(0.3 * (double)i);
    }
    f128_twiddles(n, t[0].data(), t[1].data(), t[2].data(), t[3].data());
  }
  const size_t mask = n - 1, ratio = n / (base_n ? base_n : n);
  size_t degree = 0;
  const auto t0 = std::chrono::steady_clock::now();
  for (size_t r = 0; r < reps; ++r) {
    switch (kind) {
      case 0: ordered_transform(algo, true, n, buf.data(), scratch.data(), w.data() + n); break;
      case 1: fwd_depth(n, buf.data(), w.data(), algo, base_n, scratch.data()); break;
      case 2: inv_depth(n, buf.data(), wi.data(), n + base_n, algo, base_n, scratch.data()); break;
      case 3:
        degree = degree + 1 == n ? 0 : degree + 1;
        if (ratio == 1) {
          for (size_t i = 0; i < n; ++i) buf[i] = mono[(i * degree) & mask];
        } else if (ratio == 2) {
          for (size_t i = 0; i < n / 2; ++i) {
            buf[i] = mono[((2 * i) * degree) & mask];
            buf[i + n / 2] = mono[((2 * i + 1) * degree) & mask];
          }
        } else {
          for (size_t j = 0; j < n; ++j) buf[j] = mono[(indices[j] * degree) & mask];
        }
        break;
      case 4: f128_fwd(n, f[0].data(), f[1].data(), f[2].data(), f[3].data(), t[0].data(), t[1].data(), t[2].data(), t[3].data()); break;
      default: f128_inv(n, f[0].data(), f[1].data(), f[2].data(), f[3].data(), t[0].data(), t[1].data(), t[2].data(), t[3].data()); break;
    }
    // every 16 calls, bring the values back to magnitude ~1 (an exact power-of-two
    // scaling): repeated unnormalised transforms would otherwise overflow
    if (kind <= 2 && (r & 15) == 15) {
      double m = 0.0;
      for (size_t i = 0; i < n; ++i) m = std::max(m, std::max(std::fabs(buf[i].re), std::fabs(buf[i].im)));
      if (m > 0.0 && std::isfinite(m)) {
        int e = 0;
        std::frexp(m, &e);
        for (size_t i = 0; i < n; ++i) buf[i] = c64{std::ldexp(buf[i].re, -e), std::ldexp(buf[i].im, -e)};
      }
    }
  }
  const auto t1 = std::chrono::steady_clock::now();
  *ns_per_call = std::chrono::duration<double, std::nano>(t1 - t0).count() / (double)reps;
  return 0;
}

}  // extern "C"
