// twiddles.cpp -- host twiddle tables, restated from concrete-fft v0.5.1.
//
// Plans compute their tables once on the host, exactly as the reference does
// at plan construction, and upload them; no CUDA math routine is involved, so
// every table entry has the bits of the reference's.  Built with
// -ffp-contract=off: std::fma appears only where the reference calls mul_add.
#include <cmath>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cfft_internal.h"
#include "tune_cache.h"

namespace cfft {

// src/fft_simd.rs:236-296 (the sincospi of StackOverflow answer 42792940, which
// the reference cites): reduce to (-1/4, 1/4], minimax polynomials for
// cos(pi t) and sin(pi t), then quadrant mapping.
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
  double c = std::fma(r, s, 1.0);
  r = 4.6151442520157035e-4;
  r = std::fma(r, s, -7.3700183130883555e-3);
  r = std::fma(r, s, 8.2145868949323936e-2);
  r = std::fma(r, s, -5.9926452893214921e-1);
  r = std::fma(r, s, 2.5501640398732688e+0);
  r = std::fma(r, s, -5.1677127800499516e+0);
  r *= s * t;
  double sn = std::fma(t, 3.1415926535897931e+0, r);
  if (i & 2) {
    sn = 0.0 - sn;
    c = 0.0 - c;
  }
  if (i & 1) {
    const double tt = 0.0 - sn;
    sn = c;
    c = tt;
  }
  if (a == std::floor(a)) sn = az;
  *sp = sn;
  *cp = c;
}

void init_wt(int r, size_t n, c64h* w, c64h* w_inv) {
  const double nan = std::nan("");
  for (size_t i = 0; i < 2 * n; ++i) w[i] = w_inv[i] = c64h{nan, nan};
  if (n < (size_t)r) return;
  const size_t nr = n / (size_t)r;
  const double theta = -2.0 / (double)n;
  for (size_t p = 0; p < nr; ++p) {
    for (int k = 1; k < r; ++k) {
      double s, c;
      sincospi64(theta * (double)((size_t)k * p), &s, &c);
      w[p + (size_t)k * nr] = w[n + (size_t)r * p + (size_t)k] = c64h{c, s};
      w_inv[p + (size_t)k * nr] = w_inv[n + (size_t)r * p + (size_t)k] = c64h{c, -s};
    }
  }
}

void parallel_range(size_t count, void (*f)(size_t, size_t, void*), void* ctx) {
  const size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>({hw, 16, count >> 16});  // below 2^17 entries: this thread
  if (nt <= 1) {
    f(0, count, ctx);
    return;
  }
  std::vector<std::thread> ts;
  for (size_t t = 0; t < nt; ++t) ts.emplace_back(f, count * t / nt, count * (t + 1) / nt, ctx);
  for (auto& t : ts) t.join();
}

namespace {
template <class F>
void for_range(size_t count, F&& body) {
  parallel_range(
      count, [](size_t b, size_t e, void* c) { (*(F*)c)(b, e); }, (void*)&body);
}
}  // namespace

static void unordered_rec(size_t n, size_t base_n, int base_r, c64h* w, c64h* w_inv, size_t len) {
  if (n <= base_n) {
    init_wt(base_r, n, w, w_inv);
    return;
  }
  const int r = outer_radix(n, base_n);
  const size_t m = n / (size_t)r;
  const size_t head = (size_t)(r - 1) * m;
  const double theta = 2.0 / (double)n;
  c64h* w_inv_cur = w_inv + (len - head);
  for_range(m, [&](size_t b, size_t e) {
    for (size_t p = b; p < e; ++p) {
      for (int k = 1; k < r; ++k) {
        double sk, ck;
        sincospi64(theta * (double)((size_t)k * p), &sk, &ck);
        const size_t idx = (size_t)(r - 1) * p + (size_t)(k - 1);
        w[idx] = c64h{ck, -sk};
        w_inv_cur[idx] = c64h{ck, sk};
      }
    }
  });
  unordered_rec(n / (size_t)r, base_n, base_r, w + head, w_inv, len - head);
}

void unordered_twiddles(size_t n, size_t base_n, int base_r, c64h* w, c64h* w_inv) {
  unordered_rec(n, base_n, base_r, w, w_inv, n + base_n);
}

void monomial_twiddles(size_t n, c64h* tw) {
  const double theta = -2.0 / (double)n;
  for_range(n, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      double s, c;
      sincospi64(theta * (double)i, &s, &c);
      tw[i] = c64h{c, s};
    }
  });
}

void product_twist_tables(size_t N, c64h* tw, c64h* itw) {
  const size_t n = N / 2;
  const double inv_n = 1.0 / (double)n;
  for_range(n, [&](size_t b, size_t e) {
    for (size_t j = b; j < e; ++j) {
      double s, c;
      sincospi64((double)j / (double)N, &s, &c);
      tw[j] = c64h{c, s};
      itw[j] = c64h{c * inv_n, -s * inv_n};  // exact: inv_n is a power of two
    }
  });
}

LevelDesc make_levels(size_t n, size_t base_n) {
  LevelDesc d;
  std::memset(&d, 0, sizeof(d));
  size_t cur = n;
  int l = 0, off = 0;
  while (cur > base_n) {
    const int r = outer_radix(cur, base_n);
    d.log2n[l] = ilog2(cur);
    d.log2r[l] = ilog2((size_t)r);
    d.w_off[l] = off;
    off += (int)((size_t)(r - 1) * (cur / (size_t)r));
    d.winv_off[l] = (int)(cur / (size_t)r + base_n);
    cur /= (size_t)r;
    ++l;
  }
  d.nlevels = l;
  d.log2n[l] = ilog2(cur);
  d.w_off[l] = off;
  return d;
}

// ---------------------------------------------------------------- fft128
namespace {
struct f128 {
  double hi, lo;
};
// src/fft128/f128_ops.rs:3-40, 290-400 (no contraction: only two_prod uses fma)
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
inline f128 add(f128 a, f128 b) {
  double s1, s2, t1, t2;
  two_sum(a.hi, b.hi, &s1, &s2);
  two_sum(a.lo, b.lo, &t1, &t2);
  s2 = s2 + t1;
  quick_two_sum(s1, s2, &s1, &s2);
  s2 = s2 + t2;
  quick_two_sum(s1, s2, &s1, &s2);
  return {s1, s2};
}
inline f128 sub(f128 a, f128 b) {
  double s1, s2, t1, t2;
  two_diff(a.hi, b.hi, &s1, &s2);
  two_diff(a.lo, b.lo, &t1, &t2);
  s2 = s2 + t1;
  quick_two_sum(s1, s2, &s1, &s2);
  s2 = s2 + t2;
  quick_two_sum(s1, s2, &s1, &s2);
  return {s1, s2};
}
inline f128 sub_f64(f128 a, double b) {
  double s1, s2;
  two_diff(a.hi, b, &s1, &s2);
  s2 = s2 + a.lo;
  quick_two_sum(s1, s2, &s1, &s2);
  return {s1, s2};
}
inline f128 mul(f128 a, f128 b) {
  const double p = a.hi * b.hi;
  double e = std::fma(a.hi, b.hi, -p);
  e = e + (a.hi * b.lo + a.lo * b.hi);
  double s1, s2;
  quick_two_sum(p, e, &s1, &s2);
  return {s1, s2};
}
inline f128 sqr(f128 a) {
  const double p = a.hi * a.hi;
  double e = std::fma(a.hi, a.hi, -p);
  e = e + 2.0 * (a.hi * a.lo);
  double s1, s2;
  quick_two_sum(p, e, &s1, &s2);
  return {s1, s2};
}
inline f128 neg(f128 a) { return {-a.hi, -a.lo}; }

#include "f128_constants.inc"

// src/fft128/f128_ops.rs:504-575
void f128_sincospi(f128 x, f128* s_out, f128* c_out) {
  const double pd = std::round(x.hi * 2.0);
  f128 r = sub_f64(x, pd * 0.5);
  const double qd = std::round(r.hi * 16.0);
  r = sub_f64(r, qd * (1.0 / 16.0));
  const long p = (long)pd, q = (long)qd;
  const long qa = q < 0 ? -q : q;
  f128 sinc = kF128Pi, cs = {1.0, 0.0}, pw = {1.0, 0.0};
  const f128 sq = sqr(r);
  for (int i = 0; i < 9; ++i) {
    pw = mul(pw, sq);
    sinc = add(sinc, mul(kSinPiTaylor[i], pw));
    cs = add(cs, mul(kCosPiTaylor[i], pw));
  }
  const f128 sin_r = mul(sinc, r), cos_r = cs;
  f128 s, c;
  if (q == 0) {
    s = sin_r;
    c = cos_r;
  } else {
    const f128 u = kCosKPiOver16[qa - 1], v = kSinKPiOver16[qa - 1];
    if (q > 0) {
      s = add(mul(u, sin_r), mul(v, cos_r));
      c = sub(mul(u, cos_r), mul(v, sin_r));
    } else {
      s = sub(mul(u, sin_r), mul(v, cos_r));
      c = add(mul(u, cos_r), mul(v, sin_r));
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
}
}  // namespace

void f128_twiddles(size_t n, double* re0, double* re1, double* im0, double* im1) {
  re0[0] = re1[0] = im0[0] = im1[0] = 0.0;
  const int logn2 = ilog2(2 * n);
  // entry m + i (m a power of two, i < m) holds the twiddle of k = 2m + i
  for_range(n, [&](size_t b, size_t e) {
    for (size_t pos = std::max<size_t>(b, 1); pos < e; ++pos) {
      size_t m = 1;
      while (2 * m <= pos) m *= 2;
      const size_t k = pos + m;
      size_t br = 0;
      for (int bit = 0; bit < logn2; ++bit) br |= ((k >> bit) & 1u) << (logn2 - 1 - bit);
      f128 s, c;
      f128_sincospi(f128{(double)br / (double)(2 * n), 0.0}, &s, &c);
      re0[pos] = c.hi;
      re1[pos] = c.lo;
      im0[pos] = s.hi;
      im1[pos] = s.lo;
    }
  });
}

// ---------------------------------------------------------------- f128::sincospi on the host
// src/fft128/f128_ops.rs:534-575: panics for inputs above 1 or below -1 in
// f128's lexicographic order (NaN compares as unordered and goes through).
extern "C" cfft_status cfft_f128_sincospi(double x_hi, double x_lo, double* sin_out, double* cos_out) {
  if (!sin_out || !cos_out) return fail_status(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  const bool above = x_hi > 1.0 || (x_hi == 1.0 && x_lo > 0.0);
  const bool below = x_hi < -1.0 || (x_hi == -1.0 && x_lo < 0.0);
  if (above || below) return fail_status(CFFT_ERR_INVALID_ARGUMENT, "f128::sincospi: input outside [-1, 1]");
  f128 s, c;
  f128_sincospi(f128{x_hi, x_lo}, &s, &c);
  sin_out[0] = s.hi;
  sin_out[1] = s.lo;
  cos_out[0] = c.hi;
  cos_out[1] = c.lo;
  return CFFT_OK;
}

// ---------------------------------------------------------------- errors
static std::mutex g_err_mu;
static std::string g_err;
void set_error(const std::string& msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err = msg;
}
cfft_status fail_status(cfft_status s, const std::string& msg) {
  set_error(msg);
  return s;
}
std::string get_error() {
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_err;
}

}  // namespace cfft
