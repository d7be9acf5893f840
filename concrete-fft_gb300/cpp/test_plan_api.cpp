// test_plan_api.cpp -- the reference crate's own tests, through the C++ API.
//
// Each test restates one #[test] of concrete-fft v0.5.1 with its tolerance;
// rustfft is replaced by a long-double DFT, rug/f128 schoolbook products by
// quad precision (long double on aarch64, __float128 elsewhere).
//   ordered::tests::test_fft            src/ordered.rs:389-467
//   unordered::tests::test_fwd          src/unordered.rs:1073-1104
//   unordered::tests::test_fwd_monomial src/unordered.rs:1108-1137
//   unordered::tests::test_roundtrip    src/unordered.rs:1141-1172
//   unordered::tests::test_equivalency  src/unordered.rs:1176-9395 (golden vector)
//   unordered::tests_serde::test_serde  src/unordered.rs:9399-9466
//   fft128::tests::test_wrapper         src/fft128/mod.rs:1972-2065
// Usage: test_plan_api <dir with the golden .npy fixtures>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <string>

#include "concrete_fft.hpp"

using concrete_fft::c64;
using concrete_fft::FftAlgo;
namespace ordered = concrete_fft::ordered;
namespace unordered = concrete_fft::unordered;

#if defined(__aarch64__)
typedef long double quad;
#else
typedef __float128 quad;
#endif

static int g_fail = 0;
#define EXPECT(cond, ...)                      \
  do {                                         \
    if (!(cond)) {                             \
      std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);                \
      std::printf("\n");                       \
      ++g_fail;                                \
    }                                          \
  } while (0)

static std::mt19937_64 rng(42);
static double random01() { return std::uniform_real_distribution<double>(0.0, 1.0)(rng); }

static std::vector<std::complex<long double>> dft(const std::vector<c64>& x) {
  const size_t n = x.size();
  std::vector<std::complex<long double>> y(n);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (size_t p = 0; p < n; ++p) {
    std::complex<long double> acc = 0;
    for (size_t q = 0; q < n; ++q) {
      const long double ang = -2.0L * pi * (long double)((p * q) % n) / (long double)n;
      acc += std::complex<long double>(x[q].real(), x[q].imag()) * std::complex<long double>(cosl(ang), sinl(ang));
    }
    y[p] = acc;
  }
  return y;
}

static double dist(c64 a, std::complex<long double> b) {
  return (double)std::abs(std::complex<long double>(a.real(), a.imag()) - b);
}

static size_t bit_rev(unsigned nbits, size_t i) {
  size_t r = 0;
  for (unsigned b = 0; b < nbits; ++b) r |= ((i >> b) & 1u) << (nbits - 1 - b);
  return r;
}
static size_t bit_rev_twice(unsigned nbits, unsigned base_nbits, size_t i) {
  const size_t i_rev = bit_rev(nbits, i);
  const size_t mask = (size_t(1) << base_nbits) - 1;
  return (i_rev & ~mask) | bit_rev(base_nbits, i_rev & mask);
}
static unsigned lg(size_t n) {
  unsigned l = 0;
  while ((size_t(1) << l) < n) ++l;
  return l;
}

static void test_fft() {
  const FftAlgo algos[] = {FftAlgo::Dif2, FftAlgo::Dit2, FftAlgo::Dif4, FftAlgo::Dit4,
                           FftAlgo::Dif8, FftAlgo::Dit8, FftAlgo::Dif16, FftAlgo::Dit16};
  for (FftAlgo a : algos)
    for (int e = 1; e <= 10; ++e) {
      const size_t n = size_t(1) << e;
      ordered::Plan plan(n, ordered::Method::UserProvided(a));
      std::vector<c64> x(n);
      for (auto& z : x) z = c64(random01(), random01());
      const auto orig = x;
      plan.fwd(x);
      const auto want = dft(orig);
      double err = 0;
      for (size_t i = 0; i < n; ++i) err = std::max(err, dist(x[i], want[i]));
      EXPECT(err < 1e-12, "ordered fwd algo %d n %zu err %g", (int)a, n, err);
      plan.inv(x);
      double rt = 0;
      for (size_t i = 0; i < n; ++i) rt = std::max(rt, std::abs(x[i] / (double)n - orig[i]));
      EXPECT(rt < 1e-14, "ordered roundtrip algo %d n %zu err %g", (int)a, n, rt);
    }
}

static void test_fwd() {
  for (size_t n : {128, 256, 512, 1024}) {
    std::vector<c64> z(n);
    for (auto& v : z) v = c64(random01(), random01());
    const auto target = dft(z);
    unordered::Plan plan(n, unordered::Method::UserProvided(FftAlgo::Dif4, 32));
    plan.fwd(z);
    for (size_t i = 0; i < n; ++i)
      EXPECT(dist(z[bit_rev_twice(lg(n), lg(32), i)], target[i]) < 1e-12, "unordered fwd n %zu i %zu", n, i);
  }
}

static void test_fwd_monomial() {
  for (size_t n : {256, 512, 1024})
    for (size_t base : {size_t(32), n, n / 2, n / 4, n / 8})
      for (int t = 0; t < 10; ++t) {
        unordered::Plan plan(n, unordered::Method::UserProvided(FftAlgo::Dif4, base));
        const size_t degree = rng() % n;
        std::vector<c64> z(n, 0.0), target(n, 0.0);
        target[degree] = 1.0;
        plan.fwd(target);
        plan.fwd_monomial(degree, z.data(), n);
        double err = 0;
        for (size_t i = 0; i < n; ++i) err = std::max(err, std::abs(z[i] - target[i]));
        EXPECT(err < 1e-12, "monomial n %zu base %zu degree %zu err %g", n, base, degree, err);
      }
}

static void test_roundtrip() {
  for (size_t n : {32, 64, 256, 512, 1024}) {
    std::vector<c64> z(n);
    for (auto& v : z) v = c64(random01(), random01());
    const auto orig = z;
    unordered::Plan plan(n, unordered::Method::UserProvided(FftAlgo::Dif4, 32));
    plan.fwd(z);
    plan.inv(z);
    double err = 0;
    for (size_t i = 0; i < n; ++i) err = std::max(err, std::abs(z[i] / (double)n - orig[i]));
    EXPECT(err < 1e-12, "unordered roundtrip n %zu err %g", n, err);
  }
}

// minimal .npy reader for (2048, 2) float64 fixtures
static bool read_npy(const std::string& path, std::vector<double>& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  char magic[6];
  f.read(magic, 6);
  unsigned char ver[2];
  f.read((char*)ver, 2);
  uint32_t hlen = 0;
  if (ver[0] == 1) {
    uint16_t h16;
    f.read((char*)&h16, 2);
    hlen = h16;
  } else {
    f.read((char*)&hlen, 4);
  }
  std::string header(hlen, ' ');
  f.read(&header[0], hlen);
  out.resize(4096);
  f.read((char*)out.data(), 4096 * 8);
  return (bool)f;
}

static void test_equivalency(const std::string& dir) {
  std::vector<double> in, want;
  if (!read_npy(dir + "/unordered_fwd_n2048_dif4_base32_input.npy", in) ||
      !read_npy(dir + "/unordered_fwd_n2048_dif4_base32_expected.npy", want)) {
    EXPECT(false, "golden fixtures not found in %s", dir.c_str());
    return;
  }
  std::vector<c64> z(2048);
  for (size_t i = 0; i < 2048; ++i) z[i] = c64(in[2 * i], in[2 * i + 1]);
  unordered::Plan plan(2048, unordered::Method::UserProvided(FftAlgo::Dif4, 32));
  plan.fwd(z);
  size_t bad = 0;
  for (size_t i = 0; i < 2048; ++i)
    if (z[i].real() != want[2 * i] || z[i].imag() != want[2 * i + 1]) ++bad;  // assert_eq!
  EXPECT(bad == 0, "golden vector: %zu of 2048 differ", bad);
}

static void test_serde() {
  for (size_t n : {64, 128, 256, 512, 1024}) {
    std::vector<c64> z(n);
    for (auto& v : z) v = c64(random01(), random01());
    const auto orig = z;
    unordered::Plan plan1(n, unordered::Method::UserProvided(FftAlgo::Dif4, 32));
    unordered::Plan plan2(n, unordered::Method::UserProvided(FftAlgo::Dif4, 64));
    plan1.fwd(z);
    const auto wire = plan1.serialize_fourier_buffer(z.data(), n);
    plan2.deserialize_fourier_buffer(wire, z.data(), n);
    plan2.inv(z);
    double err = 0;
    for (size_t i = 0; i < n; ++i) err = std::max(err, std::abs(z[i] / (double)n - orig[i]));
    EXPECT(err < 1e-12, "serde n %zu err %g", n, err);
    bool threw = false;
    try {
      plan2.deserialize_fourier_buffer(std::vector<c64>(n - 1), z.data(), n);
    } catch (const concrete_fft::Error& e) {
      threw = e.status() == CFFT_ERR_LENGTH_MISMATCH;
    }
    EXPECT(threw, "serde invalid_length not reported");
  }
}

static void test_wrapper() {
  for (size_t n : {64, 128, 256, 512, 1024, 2048}) {
    std::vector<double> lhs(n), rhs(n);
    for (auto& v : lhs) v = random01();
    for (auto& v : rhs) v = random01();
    std::vector<quad> full(2 * n, 0), nega(n);
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j) full[i + j] += (quad)lhs[i] * (quad)rhs[j];
    for (size_t i = 0; i < n; ++i) nega[i] = full[i] - full[i + n];
    const size_t h = n / 2;
    std::vector<double> l0(h), l1(h, 0.0), l2(h), l3(h, 0.0), r0(h), r1(h, 0.0), r2(h), r3(h, 0.0);
    for (size_t i = 0; i < h; ++i) {
      l0[i] = lhs[i];
      l2[i] = lhs[i + h];
      r0[i] = rhs[i];
      r2[i] = rhs[i + h];
    }
    concrete_fft::fft128::Plan plan(h);
    plan.fwd(l0.data(), l1.data(), l2.data(), l3.data(), h);
    plan.fwd(r0.data(), r1.data(), r2.data(), r3.data(), h);
    // cplx_mul and the 2/n scale in quad, split back to double-double
    const quad factor = (quad)2.0 / (quad)n;
    for (size_t i = 0; i < h; ++i) {
      const quad ar = (quad)l0[i] + (quad)l1[i], ai = (quad)l2[i] + (quad)l3[i];
      const quad br = (quad)r0[i] + (quad)r1[i], bi = (quad)r2[i] + (quad)r3[i];
      const quad pr = (ar * br - ai * bi) * factor, pi = (ar * bi + ai * br) * factor;
      l0[i] = (double)pr;
      l1[i] = (double)(pr - (quad)l0[i]);
      l2[i] = (double)pi;
      l3[i] = (double)(pi - (quad)l2[i]);
    }
    plan.inv(l0.data(), l1.data(), l2.data(), l3.data(), h);
    double err = 0;
    for (size_t i = 0; i < h; ++i) {
      err = std::max(err, (double)fabsl((long double)(((quad)l0[i] + (quad)l1[i]) - nega[i])));
      err = std::max(err, (double)fabsl((long double)(((quad)l2[i] + (quad)l3[i]) - nega[i + h])));
    }
    EXPECT(err < 1e-30 * (double)n, "fft128 product n %zu err %g", n, err);
  }
}

static void test_errors() {
  bool threw = false;
  try {
    ordered::Plan p(2048, ordered::Method::UserProvided(FftAlgo::Dif2));  // src/ordered.rs:244
  } catch (const concrete_fft::Error& e) {
    threw = e.status() == CFFT_ERR_INVALID_SIZE;
  }
  EXPECT(threw, "ordered n = 2048 accepted");
  threw = false;
  try {
    ordered::Plan p(64, ordered::Method::UserProvided(FftAlgo::Dif4));
    std::vector<c64> x(63);
    p.fwd(x);
  } catch (const concrete_fft::Error& e) {
    threw = e.status() == CFFT_ERR_LENGTH_MISMATCH;
  }
  EXPECT(threw, "wrong buffer length accepted");
}

int main(int argc, char** argv) {
  const std::string dir = argc > 1 ? argv[1] : "tests/golden";
  try {
    test_fft();
    test_fwd();
    test_fwd_monomial();
    test_roundtrip();
    test_equivalency(dir);
    test_serde();
    test_wrapper();
    test_errors();
  } catch (const std::exception& e) {
    std::printf("FAIL exception: %s\n", e.what());
    return 1;
  }
  std::printf(g_fail ? "FAILED (%d)\n" : "ALL OK\n", g_fail);
  return g_fail ? 1 : 0;
}
