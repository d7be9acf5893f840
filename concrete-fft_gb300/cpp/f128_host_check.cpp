// f128_host_check.cpp -- evaluates the host f128 of f128.hpp on operand pairs
// read from stdin ("op a.hi a.lo b.hi b.lo", bit patterns in hex) and prints
// the results' bit patterns, for comparison with other implementations.
// op: 0 add, 1 sub, 2 mul, 3 add_estimate, 4 sub_estimate, 5 div, 6 sqr (of a),
// 7 sincospi (of a; prints sin then cos), 8 add_f128_f64, 9 sub_f128_f64,
// 10 mul_f128_f64, 11 div_f128_f64, 12 div_f64_f64, 13 div_estimate.
#include <cinttypes>
#include <cstdio>
#include <cstring>

#include "f128.hpp"

using concrete_fft::fft128::f128;

static double d(uint64_t u) {
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}
static uint64_t u(double x) {
  uint64_t v;
  std::memcpy(&v, &x, 8);
  return v;
}

int main() {
  int op;
  uint64_t a0, a1, b0, b1;
  while (std::scanf("%d %" SCNx64 " %" SCNx64 " %" SCNx64 " %" SCNx64, &op, &a0, &a1, &b0, &b1) == 5) {
    const f128 a{d(a0), d(a1)}, b{d(b0), d(b1)};
    f128 r, r2;
    switch (op) {
      case 0: r = a + b; break;
      case 1: r = a - b; break;
      case 2: r = a * b; break;
      case 3: r = f128::add_estimate_f128_f128(a, b); break;
      case 4: r = f128::sub_estimate_f128_f128(a, b); break;
      case 5: r = a / b; break;
      case 6: r = a.sqr(); break;
      case 7: {
        const auto sc = a.sincospi();
        r = sc.first;
        r2 = sc.second;
        break;
      }
      case 8: r = a + b.hi; break;
      case 9: r = a - b.hi; break;
      case 10: r = a * b.hi; break;
      case 11: r = a / b.hi; break;
      case 12: r = f128::div_f64_f64(a.hi, b.hi); break;
      case 13: r = f128::div_estimate_f128_f128(a, b); break;
      default: return 2;
    }
    std::printf("%016" PRIx64 " %016" PRIx64 " %016" PRIx64 " %016" PRIx64 "\n", u(r.hi), u(r.lo), u(r2.hi),
                u(r2.lo));
  }
  return 0;
}
