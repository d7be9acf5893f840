// f128.hpp -- host double-double arithmetic, the C++ counterpart of
// concrete_fft::fft128::f128 (src/fft128/f128_ops.rs of concrete-fft v0.5.1).
//
// A value is the unevaluated sum hi + lo of two f64 (the crate's `.0` and
// `.1`).  The operations are the crate's: error-free two_sum / two_diff /
// quick_two_sum / two_prod (FMA) building blocks, "ieee" and "estimate" adds
// and subtractions, products, squares, Newton-step divisions, and sincospi by
// argument reduction mod 1/2 and 1/16 plus a Taylor series.  Results are
// bit-identical to the crate's, which requires that the compiler does not
// contract a*b + c into an FMA: build with -ffp-contract=off (the library
// itself is built that way); every step below is a separate statement so that
// compilers contracting only within an expression keep them apart as well.
#pragma once
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <utility>

namespace concrete_fft {
namespace fft128 {

struct f128 {
  double hi = 0.0, lo = 0.0;
  constexpr f128() = default;
  constexpr f128(double h, double l) : hi(h), lo(l) {}
  constexpr f128(double v) : hi(v), lo(0.0) {}  // From<f64>  (src/fft128/f128_ops.rs:48)

  // ---- error-free transformations (src/fft128/f128_ops.rs:3-40)
  static std::pair<double, double> quick_two_sum(double a, double b) {
    const double s = a + b;
    const double t = s - a;
    return {s, b - t};
  }
  static std::pair<double, double> two_sum(double a, double b) {
    const double s = a + b;
    const double bb = s - a;
    const double t = s - bb;
    const double u = a - t;
    const double v = b - bb;
    return {s, u + v};
  }
  static std::pair<double, double> two_diff(double a, double b) {
    const double s = a - b;
    const double bb = s - a;
    const double t = s - bb;
    const double u = a - t;
    const double v = b + bb;
    return {s, u - v};
  }
  static std::pair<double, double> two_prod(double a, double b) {
    const double p = a * b;
    return {p, std::fma(a, b, -p)};
  }

  // ---- additions (src/fft128/f128_ops.rs:279-322)
  static f128 add_f64_f64(double a, double b) {
    const auto se = two_sum(a, b);
    return {se.first, se.second};
  }
  static f128 add_f128_f64(f128 a, double b) {
    auto s = two_sum(a.hi, b);
    const double s2 = s.second + a.lo;
    s = quick_two_sum(s.first, s2);
    return {s.first, s.second};
  }
  static f128 add_f64_f128(double a, f128 b) { return add_f128_f64(b, a); }
  static f128 add_estimate_f128_f128(f128 a, f128 b) {
    const auto s = two_sum(a.hi, b.hi);
    const double l = a.lo + b.lo;
    const double e = s.second + l;
    const auto r = quick_two_sum(s.first, e);
    return {r.first, r.second};
  }
  static f128 add_f128_f128(f128 a, f128 b) {
    auto s = two_sum(a.hi, b.hi);
    const auto t = two_sum(a.lo, b.lo);
    double s2 = s.second + t.first;
    s = quick_two_sum(s.first, s2);
    s2 = s.second + t.second;
    s = quick_two_sum(s.first, s2);
    return {s.first, s.second};
  }

  // ---- subtractions (src/fft128/f128_ops.rs:324-371)
  static f128 sub_f64_f64(double a, double b) {
    const auto se = two_diff(a, b);
    return {se.first, se.second};
  }
  static f128 sub_f128_f64(f128 a, double b) {
    auto s = two_diff(a.hi, b);
    const double s2 = s.second + a.lo;
    s = quick_two_sum(s.first, s2);
    return {s.first, s.second};
  }
  static f128 sub_f64_f128(double a, f128 b) {
    auto s = two_diff(a, b.hi);
    const double s2 = s.second - b.lo;
    s = quick_two_sum(s.first, s2);
    return {s.first, s.second};
  }
  static f128 sub_estimate_f128_f128(f128 a, f128 b) {
    const auto s = two_diff(a.hi, b.hi);
    double e = s.second + a.lo;
    e = e - b.lo;
    const auto r = quick_two_sum(s.first, e);
    return {r.first, r.second};
  }
  static f128 sub_f128_f128(f128 a, f128 b) {
    auto s = two_diff(a.hi, b.hi);
    const auto t = two_diff(a.lo, b.lo);
    double s2 = s.second + t.first;
    s = quick_two_sum(s.first, s2);
    s2 = s.second + t.second;
    s = quick_two_sum(s.first, s2);
    return {s.first, s.second};
  }

  // ---- products (src/fft128/f128_ops.rs:373-410)
  static f128 mul_f64_f64(double a, double b) {
    const auto pe = two_prod(a, b);
    return {pe.first, pe.second};
  }
  static f128 mul_f128_f64(f128 a, double b) {
    auto p = two_prod(a.hi, b);
    const double c = a.lo * b;
    const double p2 = p.second + c;
    p = quick_two_sum(p.first, p2);
    return {p.first, p.second};
  }
  static f128 mul_f64_f128(double a, f128 b) { return mul_f128_f64(b, a); }
  static f128 mul_f128_f128(f128 a, f128 b) {
    auto p = two_prod(a.hi, b.hi);
    const double c1 = a.hi * b.lo;
    const double c2 = a.lo * b.hi;
    const double c = c1 + c2;
    const double p2 = p.second + c;
    p = quick_two_sum(p.first, p2);
    return {p.first, p.second};
  }
  f128 sqr() const {
    auto p = two_prod(hi, hi);
    const double c = hi * lo;
    const double c2 = 2.0 * c;
    const double p2 = p.second + c2;
    p = quick_two_sum(p.first, p2);
    return {p.first, p.second};
  }

  // ---- divisions (src/fft128/f128_ops.rs:411-492)
  static f128 div_f64_f64(double a, double b) {
    const double q1 = a / b;
    const auto p = two_prod(q1, b);
    const auto s = two_diff(a, p.first);
    const double e = s.second - p.second;
    const double t = s.first + e;
    const double q2 = t / b;
    const auto r = quick_two_sum(q1, q2);
    return {r.first, r.second};
  }
  static f128 div_f128_f64(f128 a, double b) {
    const double q1 = a.hi / b;
    const auto p = two_prod(q1, b);
    const auto s = two_diff(a.hi, p.first);
    double e = s.second + a.lo;
    e = e - p.second;
    const double t = s.first + e;
    const double q2 = t / b;
    const auto r = quick_two_sum(q1, q2);
    return {r.first, r.second};
  }
  static f128 div_f128_f128(f128 a, f128 b) {
    const double q1 = a.hi / b.hi;
    f128 r = sub_f128_f128(a, mul_f128_f64(b, q1));
    const double q2 = r.hi / b.hi;
    r = sub_f128_f128(r, mul_f64_f128(q2, b));
    const double q3 = r.hi / b.hi;
    const auto q = quick_two_sum(q1, q2);
    return add_f128_f64(f128{q.first, q.second}, q3);
  }
  static f128 div_f64_f128(double a, f128 b) { return div_f128_f128(f128{a, 0.0}, b); }
  static f128 div_estimate_f128_f128(f128 a, f128 b) {
    const double q1 = a.hi / b.hi;
    const f128 r = mul_f128_f64(b, q1);
    const auto s = two_diff(a.hi, r.hi);
    double s2 = s.second - r.lo;
    s2 = s2 + a.lo;
    const double t = s.first + s2;
    const double q2 = t / b.hi;
    const auto q = quick_two_sum(q1, q2);
    return {q.first, q.second};
  }

  // ---- misc (src/fft128/f128_ops.rs:494-515)
  double to_f64() const { return hi; }
  bool is_nan() const { return std::isnan(hi) || std::isnan(lo); }
  f128 abs() const { return hi < 0.0 ? f128{-hi, -lo} : *this; }

  // sin(pi x), cos(pi x) for x in [-1, 1] (src/fft128/f128_ops.rs:517-577)
  std::pair<f128, f128> sincospi() const;

  // constants (src/fft128/f128_ops.rs:579-619), defined below
  static const f128 PI;
};

// ---- operators (src/fft128/f128_ops.rs:55-275)
inline f128 operator-(f128 a) { return {-a.hi, -a.lo}; }
inline f128 operator+(f128 a, f128 b) { return f128::add_f128_f128(a, b); }
inline f128 operator+(f128 a, double b) { return f128::add_f128_f64(a, b); }
inline f128 operator+(double a, f128 b) { return f128::add_f64_f128(a, b); }
inline f128 operator-(f128 a, f128 b) { return f128::sub_f128_f128(a, b); }
inline f128 operator-(f128 a, double b) { return f128::sub_f128_f64(a, b); }
inline f128 operator-(double a, f128 b) { return f128::sub_f64_f128(a, b); }
inline f128 operator*(f128 a, f128 b) { return f128::mul_f128_f128(a, b); }
inline f128 operator*(f128 a, double b) { return f128::mul_f128_f64(a, b); }
inline f128 operator*(double a, f128 b) { return f128::mul_f64_f128(a, b); }
inline f128 operator/(f128 a, f128 b) { return f128::div_f128_f128(a, b); }
inline f128 operator/(f128 a, double b) { return f128::div_f128_f64(a, b); }
inline f128 operator/(double a, f128 b) { return f128::div_f64_f128(a, b); }
inline f128& operator+=(f128& a, f128 b) { return a = a + b; }
inline f128& operator+=(f128& a, double b) { return a = a + b; }
inline f128& operator-=(f128& a, f128 b) { return a = a - b; }
inline f128& operator-=(f128& a, double b) { return a = a - b; }
inline f128& operator*=(f128& a, f128 b) { return a = a * b; }
inline f128& operator*=(f128& a, double b) { return a = a * b; }
inline f128& operator/=(f128& a, f128 b) { return a = a / b; }
inline f128& operator/=(f128& a, double b) { return a = a / b; }
inline bool operator==(f128 a, f128 b) { return a.hi == b.hi && a.lo == b.lo; }
inline bool operator!=(f128 a, f128 b) { return !(a == b); }
// lexicographic on (hi, lo), false when either part is unordered (NaN)
inline bool operator<(f128 a, f128 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
inline bool operator>(f128 a, f128 b) { return b < a; }
inline bool operator<=(f128 a, f128 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
inline bool operator>=(f128 a, f128 b) { return b <= a; }

namespace detail {
using f128 = ::concrete_fft::fft128::f128;
#include "../csrc/f128_constants.inc"
}  // namespace detail

inline const f128 f128::PI = detail::kF128Pi;

inline std::pair<f128, f128> f128::sincospi() const {
  const f128 x = *this;
  if (x > f128{1.0} || x < f128{-1.0}) throw std::domain_error("f128::sincospi: input outside [-1, 1]");
  // reduce mod 1/2, then mod 1/16
  const double p = std::round(x.hi * 2.0);
  f128 r = x - p * 0.5;
  const double q = std::round(r.hi * 16.0);
  r = r - q * (1.0 / 16.0);
  const long pi_ = (long)p, qi = (long)q;
  const long qa = qi < 0 ? -qi : qi;
  // Taylor series of sin(pi r)/r and cos(pi r)
  f128 sinc = detail::kF128Pi, cosr{1.0, 0.0}, pw{1.0, 0.0};
  const f128 sq = r.sqr();
  for (int i = 0; i < 9; ++i) {
    pw *= sq;
    sinc += detail::kSinPiTaylor[i] * pw;
    cosr += detail::kCosPiTaylor[i] * pw;
  }
  const f128 sin_r = sinc * r;
  f128 s = sin_r, c = cosr;
  if (qi != 0) {
    const f128 u = detail::kCosKPiOver16[qa - 1], v = detail::kSinKPiOver16[qa - 1];
    if (qi > 0) {
      s = u * sin_r + v * cosr;
      c = u * cosr - v * sin_r;
    } else {
      s = u * sin_r - v * cosr;
      c = u * cosr + v * sin_r;
    }
  }
  if (pi_ == 0) return {s, c};
  if (pi_ == 1) return {c, -s};
  if (pi_ == -1) return {-c, s};
  return {-s, -c};
}

}  // namespace fft128
}  // namespace concrete_fft
