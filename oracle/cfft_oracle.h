/*
 * cfft_oracle.h -- CPU oracle for the concrete-fft hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a scalar C++ restatement of the
 * reference crate's algorithms (zama-ai/concrete-fft v0.5.1), used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.  The
 * product library (libcfft_gb300.so) never links, loads or calls it.
 *
 * Parity is pinned: the restated unordered forward FFT reproduces the
 * reference's exact golden vector (src/unordered.rs:1176-9395, compared with
 * assert_eq!) from the restated rand 0.8 StdRng stream, see
 * tests/test_oracle_golden.py.
 *
 * Conventions: a "c64" buffer is interleaved (re, im) doubles, 16 bytes per
 * point, exactly like num_complex::Complex64.  All functions return 0 on
 * success and a negative value on invalid arguments (the reference panics).
 */
#ifndef CFFT_ORACLE_H
#define CFFT_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- scalar primitives (src/fft_simd.rs:236-321) ---- */
void oracle_sincospi64(double a, double* s, double* c);
/* init_wt(r, n): w and w_inv each hold 2n c64 (src/fft_simd.rs:298-321). */
int oracle_init_wt(int r, size_t n, double* w, double* w_inv);

/* ---- ordered plan (src/ordered.rs, src/dif*.rs, src/dit*.rs) ----
 * algo: 0 Dif2, 1 Dit2, 2 Dif4, 3 Dit4, 4 Dif8, 5 Dit8, 6 Dif16, 7 Dit16
 * (the discriminant order of ordered::FftAlgo, src/ordered.rs:28-45). */
int oracle_algo_radix(int algo);
int oracle_ordered_fwd(int algo, size_t n, double* buf, const double* twiddles);
int oracle_ordered_inv(int algo, size_t n, double* buf, const double* twiddles_inv);

/* ---- unordered plan (src/unordered.rs) ---- */
/* twiddle tables hold n + base_n c64 each (src/unordered.rs:680-681). */
int oracle_unordered_twiddles(size_t n, size_t base_n, int base_algo, double* w, double* w_inv);
int oracle_unordered_fwd(int base_algo, size_t n, size_t base_n, double* buf, const double* w);
int oracle_unordered_inv(int base_algo, size_t n, size_t base_n, double* buf, const double* w_inv);
int oracle_unordered_fwd_monomial(size_t n, size_t base_n, size_t degree, double* buf);
size_t oracle_bit_rev_twice(unsigned nbits, unsigned base_nbits, size_t i);
size_t oracle_bit_rev_twice_inv(unsigned nbits, unsigned base_nbits, size_t i);
/* serialize_fourier_buffer's element order: standard[i] = permuted[bit_rev_twice(i)] */
int oracle_unordered_to_standard(size_t n, size_t base_n, const double* permuted, double* standard);
int oracle_unordered_from_standard(size_t n, size_t base_n, const double* standard, double* permuted);

/* ---- fft128 (src/fft128/f128_ops.rs, src/fft128/mod.rs) ---- */
/* op: 0 add, 1 sub, 2 mul, 3 add_estimate, 4 sub_estimate, 5 div, 6 sqr */
int oracle_f128_binop(int op, double a0, double a1, double b0, double b1, double* out2);
int oracle_f128_sincospi(double x0, double x1, double* s2, double* c2);
int oracle_f128_twiddles(size_t n, double* re0, double* re1, double* im0, double* im1);
int oracle_f128_fwd(size_t n, double* re0, double* re1, double* im0, double* im1,
                    const double* t_re0, const double* t_re1, const double* t_im0, const double* t_im1);
int oracle_f128_inv(size_t n, double* re0, double* re1, double* im0, double* im1,
                    const double* t_re0, const double* t_re1, const double* t_im0, const double* t_im1);

/* ---- negacyclic products ----
 * Exact wrapping schoolbook (the integer oracle): out = a * b mod (X^N + 1),
 * coefficients mod 2^64 (u64) or 2^128 (u128, little-endian lo/hi words). */
int oracle_negacyclic_u64_schoolbook(size_t N, const uint64_t* a, const int64_t* b, uint64_t* out);
int oracle_negacyclic_u128_schoolbook(size_t N, const uint64_t* a, const int64_t* b, uint64_t* out);

/* The FP64 product pipeline restated around the reference's unordered FFT
 * (fold, twist, fwd, pointwise, inv, untwist, exact round mod 2^64).
 * bhat: N/2 c64 in the plan's permuted order (from oracle_u64_prepare_b). */
int oracle_u64_prepare_b(size_t N, int base_algo, size_t base_n, const int64_t* b, double* bhat);
/* z[p][k] = bhat[k] * z[p][k] for count rows of n c64 (the product pipeline's
 * pointwise step: the reference's FMA complex product, src/fft_simd.rs:164-234). */
void oracle_c64_pointwise(size_t n, size_t count, const double* bhat, double* z);
int oracle_u64_product(size_t N, int base_algo, size_t base_n, const uint64_t* a,
                       const double* bhat, uint64_t* out);
/* batched + threaded version for the CPU baseline (nthreads <= 0: all cores) */
int oracle_u64_product_batch(size_t N, int base_algo, size_t base_n, size_t count,
                             const uint64_t* a, const double* bhat, uint64_t* out, int nthreads);
/* Fourier-domain accumulation: out[g] = sum_t a[g][t] * B[g][t] mod (X^N + 1),
 * the products summed in the Fourier domain in term order, one inverse. */
int oracle_u64_product_sum(size_t N, int base_algo, size_t base_n, size_t terms, size_t count, const uint64_t* a,
                           const double* bhat, uint64_t* out, int nthreads);
/* f64 -> integer mod 2^64, floor(x + 1/2), exact for any finite input */
uint64_t oracle_round_mod64(double x);

/* The double-double product pipeline around the reference's fft128 plan.
 * a: N u128 (lo, hi words); bhat: 4 arrays of N/2 f64 (re0, re1, im0, im1). */
int oracle_u128_prepare_b(size_t N, const int64_t* b, double* bhat4);
int oracle_u128_product(size_t N, const uint64_t* a, const double* bhat4, uint64_t* out);
int oracle_u128_product_batch(size_t N, size_t count, const uint64_t* a, const double* bhat4,
                              uint64_t* out, int nthreads);

/* ---- rand 0.8 StdRng (ChaCha12) restatement, for the golden vector ----
 * StdRng::seed_from_u64(seed), then `count` draws of gen_range(0.0..1.0). */
int oracle_stdrng_uniform01(uint64_t seed, size_t count, double* out);

/* batched c64 transforms over `count` contiguous buffers, threaded (CPU baseline) */
int oracle_ordered_batch(int fwd, int algo, size_t n, size_t count, double* bufs,
                         const double* twiddles, int nthreads);
int oracle_unordered_batch(int fwd, int base_algo, size_t n, size_t base_n, size_t count,
                           double* bufs, const double* tw, int nthreads);
/* batched fft128 transforms: re0/re1/im0/im1 each hold count x n doubles (SoA per word) */
int oracle_f128_batch(int fwd, size_t n, size_t count, double* re0, double* re1, double* im0, double* im1,
                      const double* t_re0, const double* t_re1, const double* t_im0, const double* t_im1,
                      int nthreads);
/* single-threaded per-call CPU time of the restated reference (the reference's own
 * benchmark cases): kind 0 ordered fwd, 1 unordered fwd, 2 unordered inv,
 * 3 fwd_monomial, 4 fft128 fwd, 5 fft128 inv; `reps` calls on one buffer */
int oracle_bench_call(int kind, int algo, size_t n, size_t base_n, size_t reps, double* ns_per_call);
/* exact schoolbook products over a batch (words = 1: u64, words = 2: u128 as lo/hi u64 pairs), threaded */
int oracle_schoolbook_batch(int words, size_t N, size_t count, const uint64_t* a, const int64_t* b, uint64_t* out,
                            int nthreads);

#ifdef __cplusplus
}
#endif
#endif
