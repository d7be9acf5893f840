// cfft_device.cuh -- device arithmetic of the GB300 FFT path.
//
// Every operation is written with an explicit IEEE intrinsic (__dadd_rn,
// __dsub_rn, __dmul_rn, __fma_rn) and the library is compiled with
// --fmad=false, so each value is computed by exactly the operation sequence of
// the reference's Scalar backend (src/fft_simd.rs:164-234 of concrete-fft):
// the GPU transforms are bit-identical to the reference for the same
// algorithm, size and twiddle table, not merely close to it.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "int_fp64.cuh"

namespace cfft {

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization is launched as soon as every CTA of the previous kernel of its
// stream has exited, without waiting for the end of that kernel;
// grid_dependency_wait() blocks until the previous kernel has completed and its
// memory is visible, so it comes before the kernel's first global access.  No
// kernel here signals its dependents earlier than at exit: the dependents' CTAs
// would be placed while few SMs are free, and a small grid would then run on a
// fraction of the SMs (256 one-CTA transforms of 1024 points: 96 instead of
// 50 us per forward and inverse).  Without the launch attribute the wait is a
// no-op.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

struct c64 {
  double re, im;
};

__device__ __forceinline__ c64 ld(const double2* p) {
  const double2 v = *p;
  return {v.x, v.y};
}
__device__ __forceinline__ c64 ldg(const double2* p) {
  const double2 v = __ldg(p);
  return {v.x, v.y};
}
__device__ __forceinline__ void st(double2* p, c64 v) { *p = make_double2(v.re, v.im); }

// src/fft_simd.rs:209-233
__device__ __forceinline__ c64 cadd(c64 a, c64 b) { return {__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im)}; }
__device__ __forceinline__ c64 csub(c64 a, c64 b) { return {__dsub_rn(a.re, b.re), __dsub_rn(a.im, b.im)}; }
// complex product: re = fma(a, x, -(b*y)), im = fma(a, y, b*x) with (a, b) = ab.
__device__ __forceinline__ c64 cmul(c64 ab, c64 xy) {
  return {__fma_rn(ab.re, xy.re, -__dmul_rn(ab.im, xy.im)), __fma_rn(ab.re, xy.im, __dmul_rn(ab.im, xy.re))};
}
__device__ __forceinline__ c64 real_mul(double r, c64 v) { return {__dmul_rn(r, v.re), __dmul_rn(r, v.im)}; }

// Selectable adders.  E (0..8) is the number of eighths of the butterfly's
// real additions that run on the integer pipe (dadd_int, bit-identical to the
// FP64 add); I is the complex operation's index inside its butterfly, so the
// choice is made at compile time and spread evenly over the butterfly.
template <int E, int I>
__device__ __forceinline__ double sel_add(double a, double b) {
  if constexpr ((I % 8) < E) return dadd_int(a, b);
  else return __dadd_rn(a, b);
}
template <int E, int I>
__device__ __forceinline__ double sel_sub(double a, double b) {
  if constexpr ((I % 8) < E) return dsub_int(a, b);
  else return __dsub_rn(a, b);
}
template <int E, int I>
__device__ __forceinline__ c64 cadd_e(c64 a, c64 b) {
  return {sel_add<E, 2 * I>(a.re, b.re), sel_add<E, 2 * I + 1>(a.im, b.im)};
}
template <int E, int I>
__device__ __forceinline__ c64 csub_e(c64 a, c64 b) {
  return {sel_sub<E, 2 * I>(a.re, b.re), sel_sub<E, 2 * I + 1>(a.im, b.im)};
}
// src/fft_simd.rs:106-119: multiplication by -i (forward) or +i (inverse) is a
// swap plus a sign flip, both exact.
template <bool FWD>
__device__ __forceinline__ c64 mul_j(c64 v) {
  return FWD ? c64{-v.im, v.re} : c64{v.im, -v.re};
}

constexpr double kFrac1Sqrt2 = 0.70710678118654752440;
constexpr double kH1X = 0.9238795325112867;    // cos(-pi/8)
constexpr double kH1Y = -0.38268343236508984;  // sin(-pi/8)

// src/fft_simd.rs:121-160
template <bool FWD, int E = 0, int I = 0>
__device__ __forceinline__ c64 mul_exp_pi_over_8(c64 v) {
  return real_mul(kFrac1Sqrt2, cadd_e<E, I>(v, mul_j<FWD>(v)));
}
template <bool FWD, int E = 0, int I = 0>
__device__ __forceinline__ c64 mul_exp_neg_pi_over_8(c64 v) {
  return mul_exp_pi_over_8<!FWD, E, I>(v);
}
template <bool FWD>
__device__ __forceinline__ c64 mul_exp_pi_over_16(c64 v) {
  return cmul(FWD ? c64{kH1X, kH1Y} : c64{kH1X, -kH1Y}, v);
}
template <bool FWD>
__device__ __forceinline__ c64 mul_exp_17pi_over_16(c64 v) {
  return cmul(FWD ? c64{-kH1Y, -kH1X} : c64{-kH1Y, kH1X}, v);
}

// ----------------------------------------------------------------------------
// Radix-R DFT cores (the "last_butterfly" of each reference file).  The DIF
// passes multiply output k by w_k afterwards, the DIT passes multiply input k
// by w_k beforehand, the end passes use the core alone.
template <int R, bool FWD, int E = 0>
struct Core;

template <bool FWD, int E>
struct Core<2, FWD, E> {  // src/dif2.rs:108-115
  __device__ __forceinline__ static void run(c64* x) {
    const c64 a = x[0], b = x[1];
    x[0] = cadd_e<E, 0>(a, b);
    x[1] = csub_e<E, 1>(a, b);
  }
};

template <bool FWD, int E>
struct Core<4, FWD, E> {  // src/dif4.rs:171-192
  __device__ __forceinline__ static void run(c64* x) {
    const c64 apc = cadd_e<E, 0>(x[0], x[2]);
    const c64 amc = csub_e<E, 1>(x[0], x[2]);
    const c64 bpd = cadd_e<E, 2>(x[1], x[3]);
    const c64 jbmd = mul_j<FWD>(csub_e<E, 3>(x[1], x[3]));
    x[0] = cadd_e<E, 4>(apc, bpd);
    x[1] = csub_e<E, 5>(amc, jbmd);
    x[2] = csub_e<E, 6>(apc, bpd);
    x[3] = cadd_e<E, 7>(amc, jbmd);
  }
};

template <bool FWD, int E>
struct Core<8, FWD, E> {  // src/dif8.rs:311-352
  __device__ __forceinline__ static void run(c64* x) {
    const c64 a04 = cadd_e<E, 0>(x[0], x[4]);
    const c64 s04 = csub_e<E, 1>(x[0], x[4]);
    const c64 a26 = cadd_e<E, 2>(x[2], x[6]);
    const c64 js26 = mul_j<FWD>(csub_e<E, 3>(x[2], x[6]));
    const c64 a15 = cadd_e<E, 4>(x[1], x[5]);
    const c64 s15 = csub_e<E, 5>(x[1], x[5]);
    const c64 a37 = cadd_e<E, 6>(x[3], x[7]);
    const c64 js37 = mul_j<FWD>(csub_e<E, 7>(x[3], x[7]));
    const c64 a04_p1_a26 = cadd_e<E, 8>(a04, a26);
    const c64 s04_mj_s26 = csub_e<E, 9>(s04, js26);
    const c64 a04_m1_a26 = csub_e<E, 10>(a04, a26);
    const c64 s04_pj_s26 = cadd_e<E, 11>(s04, js26);
    const c64 a15_p1_a37 = cadd_e<E, 12>(a15, a37);
    const c64 w8_s15_mj_s37 = mul_exp_neg_pi_over_8<FWD, E, 24>(csub_e<E, 13>(s15, js37));
    const c64 j_a15_m1_a37 = mul_j<FWD>(csub_e<E, 14>(a15, a37));
    const c64 v8_s15_pj_s37 = mul_exp_pi_over_8<FWD, E, 25>(cadd_e<E, 15>(s15, js37));
    x[0] = cadd_e<E, 16>(a04_p1_a26, a15_p1_a37);
    x[1] = cadd_e<E, 17>(s04_mj_s26, w8_s15_mj_s37);
    x[2] = csub_e<E, 18>(a04_m1_a26, j_a15_m1_a37);
    x[3] = csub_e<E, 19>(s04_pj_s26, v8_s15_pj_s37);
    x[4] = csub_e<E, 20>(a04_p1_a26, a15_p1_a37);
    x[5] = csub_e<E, 21>(s04_mj_s26, w8_s15_mj_s37);
    x[6] = cadd_e<E, 22>(a04_m1_a26, j_a15_m1_a37);
    x[7] = cadd_e<E, 23>(s04_pj_s26, v8_s15_pj_s37);
  }
};

template <bool FWD, int E>
struct Core<16, FWD, E> {  // src/dif16.rs:650-779
  __device__ __forceinline__ static void run(c64* x) {
    const c64 a08 = cadd_e<E, 0>(x[0], x[8]), s08 = csub_e<E, 1>(x[0], x[8]);
    const c64 a4c = cadd_e<E, 2>(x[4], x[12]), s4c = csub_e<E, 3>(x[4], x[12]);
    const c64 a2a = cadd_e<E, 4>(x[2], x[10]), s2a = csub_e<E, 5>(x[2], x[10]);
    const c64 a6e = cadd_e<E, 6>(x[6], x[14]), s6e = csub_e<E, 7>(x[6], x[14]);
    const c64 a19 = cadd_e<E, 8>(x[1], x[9]), s19 = csub_e<E, 9>(x[1], x[9]);
    const c64 a5d = cadd_e<E, 10>(x[5], x[13]), s5d = csub_e<E, 11>(x[5], x[13]);
    const c64 a3b = cadd_e<E, 12>(x[3], x[11]), s3b = csub_e<E, 13>(x[3], x[11]);
    const c64 a7f = cadd_e<E, 14>(x[7], x[15]), s7f = csub_e<E, 15>(x[7], x[15]);

    const c64 js4c = mul_j<FWD>(s4c), js6e = mul_j<FWD>(s6e);
    const c64 js5d = mul_j<FWD>(s5d), js7f = mul_j<FWD>(s7f);

    const c64 a08p1a4c = cadd_e<E, 16>(a08, a4c), s08mjs4c = csub_e<E, 17>(s08, js4c);
    const c64 a08m1a4c = csub_e<E, 18>(a08, a4c), s08pjs4c = cadd_e<E, 19>(s08, js4c);
    const c64 a2ap1a6e = cadd_e<E, 20>(a2a, a6e), s2amjs6e = csub_e<E, 21>(s2a, js6e);
    const c64 a2am1a6e = csub_e<E, 22>(a2a, a6e), s2apjs6e = cadd_e<E, 23>(s2a, js6e);
    const c64 a19p1a5d = cadd_e<E, 24>(a19, a5d), s19mjs5d = csub_e<E, 25>(s19, js5d);
    const c64 a19m1a5d = csub_e<E, 26>(a19, a5d), s19pjs5d = cadd_e<E, 27>(s19, js5d);
    const c64 a3bp1a7f = cadd_e<E, 28>(a3b, a7f), s3bmjs7f = csub_e<E, 29>(s3b, js7f);
    const c64 a3bm1a7f = csub_e<E, 30>(a3b, a7f), s3bpjs7f = cadd_e<E, 31>(s3b, js7f);

    const c64 w8_s2amjs6e = mul_exp_neg_pi_over_8<FWD, E, 64>(s2amjs6e);
    const c64 j_a2am1a6e = mul_j<FWD>(a2am1a6e);
    const c64 v8_s2apjs6e = mul_exp_pi_over_8<FWD, E, 65>(s2apjs6e);

    const c64 e0 = cadd_e<E, 32>(a08p1a4c, a2ap1a6e);
    const c64 e1 = cadd_e<E, 33>(s08mjs4c, w8_s2amjs6e);
    const c64 e2 = csub_e<E, 34>(a08m1a4c, j_a2am1a6e);
    const c64 e3 = csub_e<E, 35>(s08pjs4c, v8_s2apjs6e);
    const c64 e4 = csub_e<E, 36>(a08p1a4c, a2ap1a6e);
    const c64 e5 = csub_e<E, 37>(s08mjs4c, w8_s2amjs6e);
    const c64 e6 = cadd_e<E, 38>(a08m1a4c, j_a2am1a6e);
    const c64 e7 = cadd_e<E, 39>(s08pjs4c, v8_s2apjs6e);

    const c64 w8_s3bmjs7f = mul_exp_neg_pi_over_8<FWD, E, 66>(s3bmjs7f);
    const c64 j_a3bm1a7f = mul_j<FWD>(a3bm1a7f);
    const c64 v8_s3bpjs7f = mul_exp_pi_over_8<FWD, E, 67>(s3bpjs7f);

    const c64 f0 = cadd_e<E, 40>(a19p1a5d, a3bp1a7f);
    const c64 f1 = cadd_e<E, 41>(s19mjs5d, w8_s3bmjs7f);
    const c64 f2 = csub_e<E, 42>(a19m1a5d, j_a3bm1a7f);
    const c64 f3 = csub_e<E, 43>(s19pjs5d, v8_s3bpjs7f);
    const c64 f4 = csub_e<E, 44>(a19p1a5d, a3bp1a7f);
    const c64 f5 = csub_e<E, 45>(s19mjs5d, w8_s3bmjs7f);
    const c64 f6 = cadd_e<E, 46>(a19m1a5d, j_a3bm1a7f);
    const c64 f7 = cadd_e<E, 47>(s19pjs5d, v8_s3bpjs7f);

    const c64 h1 = mul_exp_pi_over_16<FWD>(f1);
    const c64 w8 = mul_exp_neg_pi_over_8<FWD, E, 68>(f2);
    const c64 h3 = mul_exp_17pi_over_16<FWD>(f3);
    const c64 j4 = mul_j<FWD>(f4);
    const c64 hd = mul_exp_17pi_over_16<!FWD>(f5);
    const c64 v8 = mul_exp_pi_over_8<FWD, E, 69>(f6);
    const c64 hf = mul_exp_pi_over_16<!FWD>(f7);

    x[0] = cadd_e<E, 48>(e0, f0);
    x[1] = cadd_e<E, 49>(e1, h1);
    x[2] = cadd_e<E, 50>(e2, w8);
    x[3] = cadd_e<E, 51>(e3, h3);
    x[4] = csub_e<E, 52>(e4, j4);
    x[5] = csub_e<E, 53>(e5, hd);
    x[6] = csub_e<E, 54>(e6, v8);
    x[7] = csub_e<E, 55>(e7, hf);
    x[8] = csub_e<E, 56>(e0, f0);
    x[9] = csub_e<E, 57>(e1, h1);
    x[10] = csub_e<E, 58>(e2, w8);
    x[11] = csub_e<E, 59>(e3, h3);
    x[12] = cadd_e<E, 60>(e4, j4);
    x[13] = cadd_e<E, 61>(e5, hd);
    x[14] = cadd_e<E, 62>(e6, v8);
    x[15] = cadd_e<E, 63>(e7, hf);
  }
};

// Half of a radix-R core: the outputs k with k % 2 == H, by the same
// operations on the same operands as Core<R>.  The even outputs depend only on
// the sums x_k + x_{k+R/2} and the odd outputs only on the differences, so no
// operation is repeated.  Two threads then share one butterfly, which doubles
// the threads a pass can use.  y[j] = output 2j + H.
template <int R, bool FWD, int H>
struct CoreHalf;

template <bool FWD, int H>
struct CoreHalf<2, FWD, H> {
  __device__ __forceinline__ static void run(const c64* x, c64* y) { y[0] = H == 0 ? cadd(x[0], x[1]) : csub(x[0], x[1]); }
};

template <bool FWD>
struct CoreHalf<4, FWD, 0> {
  __device__ __forceinline__ static void run(const c64* x, c64* y) {
    const c64 apc = cadd(x[0], x[2]);
    const c64 bpd = cadd(x[1], x[3]);
    y[0] = cadd(apc, bpd);
    y[1] = csub(apc, bpd);
  }
};

template <bool FWD>
struct CoreHalf<4, FWD, 1> {
  __device__ __forceinline__ static void run(const c64* x, c64* y) {
    const c64 amc = csub(x[0], x[2]);
    const c64 jbmd = mul_j<FWD>(csub(x[1], x[3]));
    y[0] = csub(amc, jbmd);
    y[1] = cadd(amc, jbmd);
  }
};

// Radix 8: the even outputs use the sums x_k + x_{k+4}, the odd outputs the
// differences (src/dif8.rs:311-352, as Core<8>).
template <bool FWD>
struct CoreHalf<8, FWD, 0> {
  __device__ __forceinline__ static void run(const c64* x, c64* y) {
    const c64 a04 = cadd(x[0], x[4]);
    const c64 a26 = cadd(x[2], x[6]);
    const c64 a15 = cadd(x[1], x[5]);
    const c64 a37 = cadd(x[3], x[7]);
    const c64 a04_p1_a26 = cadd(a04, a26);
    const c64 a04_m1_a26 = csub(a04, a26);
    const c64 a15_p1_a37 = cadd(a15, a37);
    const c64 j_a15_m1_a37 = mul_j<FWD>(csub(a15, a37));
    y[0] = cadd(a04_p1_a26, a15_p1_a37);
    y[1] = csub(a04_m1_a26, j_a15_m1_a37);
    y[2] = csub(a04_p1_a26, a15_p1_a37);
    y[3] = cadd(a04_m1_a26, j_a15_m1_a37);
  }
};

template <bool FWD>
struct CoreHalf<8, FWD, 1> {
  __device__ __forceinline__ static void run(const c64* x, c64* y) {
    const c64 s04 = csub(x[0], x[4]);
    const c64 js26 = mul_j<FWD>(csub(x[2], x[6]));
    const c64 s15 = csub(x[1], x[5]);
    const c64 js37 = mul_j<FWD>(csub(x[3], x[7]));
    const c64 s04_mj_s26 = csub(s04, js26);
    const c64 s04_pj_s26 = cadd(s04, js26);
    const c64 w8_s15_mj_s37 = mul_exp_neg_pi_over_8<FWD>(csub(s15, js37));
    const c64 v8_s15_pj_s37 = mul_exp_pi_over_8<FWD>(cadd(s15, js37));
    y[0] = cadd(s04_mj_s26, w8_s15_mj_s37);
    y[1] = csub(s04_pj_s26, v8_s15_pj_s37);
    y[2] = csub(s04_mj_s26, w8_s15_mj_s37);
    y[3] = cadd(s04_pj_s26, v8_s15_pj_s37);
  }
};

// Radix 16 (src/dif16.rs:650-779, as Core<16>): the even outputs use the sums
// x_k + x_{k+8}, the odd outputs the differences.
template <bool FWD>
struct CoreHalf<16, FWD, 0> {
  __device__ __forceinline__ static void run(const c64* x, c64* y) {
    const c64 a08 = cadd(x[0], x[8]), a4c = cadd(x[4], x[12]);
    const c64 a2a = cadd(x[2], x[10]), a6e = cadd(x[6], x[14]);
    const c64 a19 = cadd(x[1], x[9]), a5d = cadd(x[5], x[13]);
    const c64 a3b = cadd(x[3], x[11]), a7f = cadd(x[7], x[15]);
    const c64 a08p1a4c = cadd(a08, a4c), a08m1a4c = csub(a08, a4c);
    const c64 a2ap1a6e = cadd(a2a, a6e), a2am1a6e = csub(a2a, a6e);
    const c64 a19p1a5d = cadd(a19, a5d), a19m1a5d = csub(a19, a5d);
    const c64 a3bp1a7f = cadd(a3b, a7f), a3bm1a7f = csub(a3b, a7f);
    const c64 j_a2am1a6e = mul_j<FWD>(a2am1a6e);
    const c64 e0 = cadd(a08p1a4c, a2ap1a6e);
    const c64 e2 = csub(a08m1a4c, j_a2am1a6e);
    const c64 e4 = csub(a08p1a4c, a2ap1a6e);
    const c64 e6 = cadd(a08m1a4c, j_a2am1a6e);
    const c64 j_a3bm1a7f = mul_j<FWD>(a3bm1a7f);
    const c64 f0 = cadd(a19p1a5d, a3bp1a7f);
    const c64 f2 = csub(a19m1a5d, j_a3bm1a7f);
    const c64 f4 = csub(a19p1a5d, a3bp1a7f);
    const c64 f6 = cadd(a19m1a5d, j_a3bm1a7f);
    const c64 w8 = mul_exp_neg_pi_over_8<FWD>(f2);
    const c64 j4 = mul_j<FWD>(f4);
    const c64 v8 = mul_exp_pi_over_8<FWD>(f6);
    y[0] = cadd(e0, f0);
    y[1] = cadd(e2, w8);
    y[2] = csub(e4, j4);
    y[3] = csub(e6, v8);
    y[4] = csub(e0, f0);
    y[5] = csub(e2, w8);
    y[6] = cadd(e4, j4);
    y[7] = cadd(e6, v8);
  }
};

template <bool FWD>
struct CoreHalf<16, FWD, 1> {
  __device__ __forceinline__ static void run(const c64* x, c64* y) {
    const c64 s08 = csub(x[0], x[8]), s4c = csub(x[4], x[12]);
    const c64 s2a = csub(x[2], x[10]), s6e = csub(x[6], x[14]);
    const c64 s19 = csub(x[1], x[9]), s5d = csub(x[5], x[13]);
    const c64 s3b = csub(x[3], x[11]), s7f = csub(x[7], x[15]);
    const c64 js4c = mul_j<FWD>(s4c), js6e = mul_j<FWD>(s6e);
    const c64 js5d = mul_j<FWD>(s5d), js7f = mul_j<FWD>(s7f);
    const c64 s08mjs4c = csub(s08, js4c), s08pjs4c = cadd(s08, js4c);
    const c64 s2amjs6e = csub(s2a, js6e), s2apjs6e = cadd(s2a, js6e);
    const c64 s19mjs5d = csub(s19, js5d), s19pjs5d = cadd(s19, js5d);
    const c64 s3bmjs7f = csub(s3b, js7f), s3bpjs7f = cadd(s3b, js7f);
    const c64 w8_s2amjs6e = mul_exp_neg_pi_over_8<FWD>(s2amjs6e);
    const c64 v8_s2apjs6e = mul_exp_pi_over_8<FWD>(s2apjs6e);
    const c64 e1 = cadd(s08mjs4c, w8_s2amjs6e);
    const c64 e3 = csub(s08pjs4c, v8_s2apjs6e);
    const c64 e5 = csub(s08mjs4c, w8_s2amjs6e);
    const c64 e7 = cadd(s08pjs4c, v8_s2apjs6e);
    const c64 w8_s3bmjs7f = mul_exp_neg_pi_over_8<FWD>(s3bmjs7f);
    const c64 v8_s3bpjs7f = mul_exp_pi_over_8<FWD>(s3bpjs7f);
    const c64 f1 = cadd(s19mjs5d, w8_s3bmjs7f);
    const c64 f3 = csub(s19pjs5d, v8_s3bpjs7f);
    const c64 f5 = csub(s19mjs5d, w8_s3bmjs7f);
    const c64 f7 = cadd(s19pjs5d, v8_s3bpjs7f);
    const c64 h1 = mul_exp_pi_over_16<FWD>(f1);
    const c64 h3 = mul_exp_17pi_over_16<FWD>(f3);
    const c64 hd = mul_exp_17pi_over_16<!FWD>(f5);
    const c64 hf = mul_exp_pi_over_16<!FWD>(f7);
    y[0] = cadd(e1, h1);
    y[1] = cadd(e3, h3);
    y[2] = csub(e5, hd);
    y[3] = csub(e7, hf);
    y[4] = csub(e1, h1);
    y[5] = csub(e3, h3);
    y[6] = cadd(e5, hd);
    y[7] = cadd(e7, hf);
  }
};

// ----------------------------------------------------------------------------
// Exact integer <-> double conversions on the integer pipe.  On GB300 the
// I2F.F64/F2I.F64 conversions issue on the (narrow) FP64 pipe, so the product
// kernels convert with integer instructions instead; both functions are exact
// IEEE round-to-nearest-even / round-half-up definitions, not approximations.

// (double)(int64_t)v, round to nearest even.
__device__ __forceinline__ double i64_to_f64_rne(int64_t v) {
  if (v == 0) return 0.0;
  const uint64_t sign = (uint64_t)v & 0x8000000000000000ull;
  uint64_t u = sign ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
  const int lz = __clzll((long long)u);
  u <<= lz;                      // leading one at bit 63
  uint64_t m = u >> 11;          // 53 significant bits
  const uint64_t rem = u & 0x7ff;
  uint64_t e = (uint64_t)(1086 - lz);  // biased exponent of 2^(63-lz)
  if (rem > 0x400 || (rem == 0x400 && (m & 1))) {
    m += 1;
    if (m == (1ull << 53)) {
      m >>= 1;
      e += 1;
    }
  }
  return __longlong_as_double((long long)(sign | (e << 52) | (m & 0xfffffffffffffull)));
}

// floor(x + 1/2) mod 2^64 for any finite double (0 for inf/nan/subnormal).
__device__ __forceinline__ uint64_t round_half_up_mod64(double x) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const bool neg = (bits >> 63) != 0;
  const int bexp = (int)((bits >> 52) & 0x7ff);
  if (bexp == 0x7ff || bexp == 0) return 0;
  const uint64_t m = (bits & 0xfffffffffffffull) | (1ull << 52);
  const int e = bexp - 1075;
  if (e >= 0) {
    const uint64_t mag = e >= 64 ? 0 : (m << e);
    return neg ? (uint64_t)0 - mag : mag;
  }
  const int k = -e;
  if (k > 54) return 0;
  const uint64_t half = 1ull << (k - 1);
  if (!neg) return (m + half) >> k;
  return (uint64_t)0 - ((m + half - 1) >> k);
}

}  // namespace cfft
