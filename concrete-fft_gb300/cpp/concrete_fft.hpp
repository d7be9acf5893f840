// concrete_fft.hpp -- C++ mirror of concrete-fft's public API over the C ABI
// of libcfft_gb300.so (include/cfft.h).
//
// Same module and method names as the Rust crate (zama-ai/concrete-fft v0.5.1):
//   concrete_fft::ordered::{FftAlgo, Method, Plan}      (src/ordered.rs)
//   concrete_fft::unordered::{Method, Plan}             (src/unordered.rs)
//   concrete_fft::fft128::{Plan, f128}                  (src/fft128/mod.rs, f128_ops.rs)
// Where the crate panics (assert! on sizes, base sizes, buffer lengths), these
// classes throw concrete_fft::Error carrying the cfft_status.  Slices become
// (pointer, length) pairs; host buffers go through the *_host entry points,
// device buffers (with a CUDA stream) through the device entry points.
#pragma once
#include <chrono>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/cfft.h"
#include "f128.hpp"

namespace concrete_fft {

using c64 = std::complex<double>;  // layout of num_complex::Complex64

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(cfft_status s) {
  if (s != CFFT_OK) throw Error((int)s, std::string("concrete-fft (gb300): ") + cfft_last_error());
}

// src/ordered.rs:28-45
enum class FftAlgo { Dif2 = 0, Dit2, Dif4, Dit4, Dif8, Dit8, Dif16, Dit16 };

namespace ordered {

using concrete_fft::FftAlgo;

// src/ordered.rs:50-59
struct Method {
  enum class Kind { UserProvided, Measure } kind;
  FftAlgo algo = FftAlgo::Dif2;
  double seconds = 0.0;
  static Method UserProvided(FftAlgo a) { return Method{Kind::UserProvided, a, 0.0}; }
  static Method Measure(std::chrono::duration<double> d) { return Method{Kind::Measure, FftAlgo::Dif2, d.count()}; }
};

class Plan {
 public:
  // Plan::new -- src/ordered.rs:242-278
  Plan(std::size_t n, Method m) {
    cfft_ordered_plan* p = nullptr;
    if (m.kind == Method::Kind::UserProvided) check(cfft_ordered_plan_create(n, (cfft_algo)m.algo, &p));
    else check(cfft_ordered_plan_create_measure(n, m.seconds, &p));
    raw_ = p;
  }
  ~Plan() { cfft_ordered_plan_destroy(raw_); }
  Plan(const Plan&) = delete;
  Plan& operator=(const Plan&) = delete;
  Plan(Plan&& o) noexcept : raw_(std::exchange(o.raw_, nullptr)) {}

  std::size_t fft_size() const { return cfft_ordered_fft_size(raw_); }   // src/ordered.rs:291
  FftAlgo algo() const { return (FftAlgo)cfft_ordered_algo(raw_); }       // src/ordered.rs:305
  std::size_t fft_scratch() const { return cfft_ordered_scratch_bytes(raw_); }  // src/ordered.rs:320

  // Plan::fwd / Plan::inv -- src/ordered.rs:342-373 (host slice, in place)
  void fwd(c64* buf, std::size_t len) const { run(buf, len, true); }
  void inv(c64* buf, std::size_t len) const { run(buf, len, false); }
  void fwd(std::vector<c64>& v) const { fwd(v.data(), v.size()); }
  void inv(std::vector<c64>& v) const { inv(v.data(), v.size()); }
  // device buffers: `batch` transforms back to back
  void fwd_device(double* d, std::size_t batch, void* stream) const { check(cfft_ordered_fwd(raw_, d, batch, stream)); }
  void inv_device(double* d, std::size_t batch, void* stream) const { check(cfft_ordered_inv(raw_, d, batch, stream)); }

 private:
  void run(c64* buf, std::size_t len, bool f) const {
    const std::size_t n = fft_size();
    if (len != n) throw Error(CFFT_ERR_LENGTH_MISMATCH, "buffer length differs from fft_size");
    check(f ? cfft_ordered_fwd_host(raw_, (double*)buf, 1) : cfft_ordered_inv_host(raw_, (double*)buf, 1));
  }
  cfft_ordered_plan* raw_ = nullptr;
};

}  // namespace ordered

namespace unordered {

using concrete_fft::FftAlgo;

// src/unordered.rs:526-537
struct Method {
  enum class Kind { UserProvided, Measure } kind;
  FftAlgo base_algo = FftAlgo::Dif4;
  std::size_t base_n = 0;
  double seconds = 0.0;
  static Method UserProvided(FftAlgo a, std::size_t base_n) { return Method{Kind::UserProvided, a, base_n, 0.0}; }
  static Method Measure(std::chrono::duration<double> d) { return Method{Kind::Measure, FftAlgo::Dif4, 0, d.count()}; }
};

class Plan {
 public:
  // Plan::new -- src/unordered.rs:659-747
  Plan(std::size_t n, Method m) {
    cfft_unordered_plan* p = nullptr;
    if (m.kind == Method::Kind::UserProvided)
      check(cfft_unordered_plan_create(n, (cfft_algo)m.base_algo, m.base_n, &p));
    else
      check(cfft_unordered_plan_create_measure(n, m.seconds, &p));
    raw_ = p;
  }
  ~Plan() { cfft_unordered_plan_destroy(raw_); }
  Plan(const Plan&) = delete;
  Plan& operator=(const Plan&) = delete;
  Plan(Plan&& o) noexcept : raw_(std::exchange(o.raw_, nullptr)) {}

  std::size_t fft_size() const { return cfft_unordered_fft_size(raw_); }
  std::pair<FftAlgo, std::size_t> algo() const {
    cfft_algo a;
    std::size_t b;
    cfft_unordered_algo(raw_, &a, &b);
    return {(FftAlgo)a, b};
  }
  std::size_t fft_scratch() const { return cfft_unordered_scratch_bytes(raw_); }

  // src/unordered.rs:826-839, :927-940
  void fwd(c64* buf, std::size_t len) const {
    need(len);
    check(cfft_unordered_fwd_host(raw_, (double*)buf, 1));
  }
  void inv(c64* buf, std::size_t len) const {
    need(len);
    check(cfft_unordered_inv_host(raw_, (double*)buf, 1));
  }
  void fwd(std::vector<c64>& v) const { fwd(v.data(), v.size()); }
  void inv(std::vector<c64>& v) const { inv(v.data(), v.size()); }
  void fwd_device(double* d, std::size_t batch, void* s) const { check(cfft_unordered_fwd(raw_, d, batch, s)); }
  void inv_device(double* d, std::size_t batch, void* s) const { check(cfft_unordered_inv(raw_, d, batch, s)); }

  // src/unordered.rs:844-900
  void fwd_monomial(std::size_t degree, c64* buf, std::size_t len) const {
    need(len);
    check(cfft_unordered_fwd_monomial_host(raw_, degree, (double*)buf));
  }
  // serialize_fourier_buffer's element sequence (standard order), src/unordered.rs:951-970
  std::vector<c64> serialize_fourier_buffer(const c64* buf, std::size_t len) const {
    need(len);
    std::vector<c64> out(len);
    check(cfft_unordered_to_standard_host(raw_, (const double*)buf, (double*)out.data(), 1));
    return out;
  }
  // deserialize_fourier_buffer: a sequence of the wrong length is an
  // invalid_length error (src/unordered.rs:1027-1031)
  void deserialize_fourier_buffer(const std::vector<c64>& seq, c64* buf, std::size_t len) const {
    need(len);
    if (seq.size() != len)
      throw Error(CFFT_ERR_LENGTH_MISMATCH, "invalid length " + std::to_string(seq.size()) + ", expected a sequence of " +
                                               std::to_string(len) + " 64-bit complex numbers");
    check(cfft_unordered_from_standard_host(raw_, (const double*)seq.data(), (double*)buf, 1));
  }

 private:
  void need(std::size_t len) const {
    if (len != fft_size()) throw Error(CFFT_ERR_LENGTH_MISMATCH, "buffer length differs from fft_size");
  }
  cfft_unordered_plan* raw_ = nullptr;
};

}  // namespace unordered

namespace fft128 {

// f128 (src/fft128/mod.rs:7, src/fft128/f128_ops.rs): see f128.hpp

class Plan {
 public:
  explicit Plan(std::size_t n) {  // src/fft128/mod.rs:1864-1881
    cfft_f128_plan* p = nullptr;
    check(cfft_f128_plan_create(n, &p));
    raw_ = p;
  }
  ~Plan() { cfft_f128_plan_destroy(raw_); }
  Plan(const Plan&) = delete;
  Plan& operator=(const Plan&) = delete;
  std::size_t fft_size() const { return cfft_f128_fft_size(raw_); }
  // src/fft128/mod.rs:1905-1960: split re0/re1/im0/im1 slices of fft_size each
  void fwd(double* re0, double* re1, double* im0, double* im1, std::size_t len) const {
    need(len);
    check(cfft_f128_fwd_host(raw_, re0, re1, im0, im1, 1));
  }
  void inv(double* re0, double* re1, double* im0, double* im1, std::size_t len) const {
    need(len);
    check(cfft_f128_inv_host(raw_, re0, re1, im0, im1, 1));
  }

 private:
  void need(std::size_t len) const {
    if (len != fft_size()) throw Error(CFFT_ERR_LENGTH_MISMATCH, "buffer length differs from fft_size");
  }
  cfft_f128_plan* raw_ = nullptr;
};

// The crate's #[doc(hidden)] free functions (src/fft128/mod.rs:1041-1104, 1805-1828).
// init_negacyclic_twiddles fills positions 1..n-1 of four host slices of n; the
// transforms take DEVICE arrays (`batch` transforms of n back to back) and a stream.
inline void init_negacyclic_twiddles(double* re0, double* re1, double* im0, double* im1, std::size_t n) {
  check(cfft_f128_init_negacyclic_twiddles(n, re0, re1, im0, im1));
}
inline void negacyclic_fwd_fft(double* re0, double* re1, double* im0, double* im1, const double* twid_re0,
                               const double* twid_re1, const double* twid_im0, const double* twid_im1,
                               std::size_t n, std::size_t batch = 1, void* stream = nullptr) {
  check(cfft_f128_negacyclic_fwd(n, batch, re0, re1, im0, im1, twid_re0, twid_re1, twid_im0, twid_im1, stream));
}
inline void negacyclic_inv_fft(double* re0, double* re1, double* im0, double* im1, const double* twid_re0,
                               const double* twid_re1, const double* twid_im0, const double* twid_im1,
                               std::size_t n, std::size_t batch = 1, void* stream = nullptr) {
  check(cfft_f128_negacyclic_inv(n, batch, re0, re1, im0, im1, twid_re0, twid_re1, twid_im0, twid_im1, stream));
}

}  // namespace fft128

}  // namespace concrete_fft
