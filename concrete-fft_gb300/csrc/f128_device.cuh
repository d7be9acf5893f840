// f128_device.cuh -- double-double arithmetic of the reference's fft128 module.
//
// Error-free transformations (TwoSum, TwoDiff, QuickTwoSum, FMA TwoProd) and
// the "estimate" add/sub used by the FFT butterflies, each restated from
// src/fft128/f128_ops.rs with explicit IEEE intrinsics; the library is built
// with --fmad=false so nvcc cannot fuse or reorder any step.
#pragma once
#include <cstdint>

#include "cfft_device.cuh"

namespace cfft {

struct f128 {
  double hi, lo;
};

// src/fft128/f128_ops.rs:3-40
__device__ __forceinline__ void quick_two_sum(double a, double b, double& s, double& e) {
  s = __dadd_rn(a, b);
  e = __dsub_rn(b, __dsub_rn(s, a));
}
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}
__device__ __forceinline__ void two_diff(double a, double b, double& s, double& e) {
  s = __dsub_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dsub_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dadd_rn(b, bb));
}

// src/fft128/f128_ops.rs:314-320
__device__ __forceinline__ f128 add_est(f128 a, f128 b) {
  double s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __dadd_rn(e, __dadd_rn(a.lo, b.lo));
  f128 r;
  quick_two_sum(s, e, r.hi, r.lo);
  return r;
}
// src/fft128/f128_ops.rs:360-367
__device__ __forceinline__ f128 sub_est(f128 a, f128 b) {
  double s, e;
  two_diff(a.hi, b.hi, s, e);
  e = __dadd_rn(e, a.lo);
  e = __dsub_rn(e, b.lo);
  f128 r;
  quick_two_sum(s, e, r.hi, r.lo);
  return r;
}
// src/fft128/f128_ops.rs:395-400 (TwoProd by FMA, src/fft128/f128_ops.rs:37-40)
__device__ __forceinline__ f128 mul(f128 a, f128 b) {
  const double p = __dmul_rn(a.hi, b.hi);
  double e = __fma_rn(a.hi, b.hi, -p);
  e = __dadd_rn(e, __dadd_rn(__dmul_rn(a.hi, b.lo), __dmul_rn(a.lo, b.hi)));
  f128 r;
  quick_two_sum(p, e, r.hi, r.lo);
  return r;
}

// src/fft128/mod.rs:310-346 (Scalar backend: add/sub are the estimate variants)
__device__ __forceinline__ void cplx_mul(f128 ar, f128 ai, f128 br, f128 bi, f128& orr, f128& oi) {
  const f128 rr = mul(ar, br), ri = mul(ar, bi), ir = mul(ai, br), ii = mul(ai, bi);
  orr = sub_est(rr, ii);
  oi = add_est(ir, ri);
}
__device__ __forceinline__ void cplx_mul_conj(f128 ar, f128 ai, f128 br, f128 bi, f128& orr, f128& oi) {
  const f128 rr = mul(ar, br), ri = mul(ar, bi), ir = mul(ai, br), ii = mul(ai, bi);
  orr = add_est(rr, ii);
  oi = sub_est(ir, ri);
}

// Split-array views: four f64 arrays (re0, re1, im0, im1).
struct F128Arrays {
  double* re0;
  double* re1;
  double* im0;
  double* im1;
};
struct F128Tw {
  const double* __restrict__ re0;
  const double* __restrict__ re1;
  const double* __restrict__ im0;
  const double* __restrict__ im1;
};

// Forward radix-2 butterfly of src/fft128/mod.rs:378-397 on element pair (j, j + t).
__device__ __forceinline__ void f128_fwd_bfly(F128Arrays d, long j, long t, const F128Tw& tw, long widx) {
  const f128 wr{__ldg(tw.re0 + widx), __ldg(tw.re1 + widx)};
  const f128 wi{__ldg(tw.im0 + widx), __ldg(tw.im1 + widx)};
  const f128 z0r{d.re0[j], d.re1[j]}, z0i{d.im0[j], d.im1[j]};
  const f128 z1r{d.re0[j + t], d.re1[j + t]}, z1i{d.im0[j + t], d.im1[j + t]};
  f128 zr, zi;
  cplx_mul(z1r, z1i, wr, wi, zr, zi);
  const f128 ar = add_est(z0r, zr), ai = add_est(z0i, zi);
  const f128 sr = sub_est(z0r, zr), si = sub_est(z0i, zi);
  d.re0[j] = ar.hi;
  d.re1[j] = ar.lo;
  d.im0[j] = ai.hi;
  d.im1[j] = ai.lo;
  d.re0[j + t] = sr.hi;
  d.re1[j + t] = sr.lo;
  d.im0[j + t] = si.hi;
  d.im1[j + t] = si.lo;
}

// Inverse radix-2 butterfly of src/fft128/mod.rs:1131-1150.
__device__ __forceinline__ void f128_inv_bfly(F128Arrays d, long j, long t, const F128Tw& tw, long widx) {
  const f128 wr{__ldg(tw.re0 + widx), __ldg(tw.re1 + widx)};
  const f128 wi{__ldg(tw.im0 + widx), __ldg(tw.im1 + widx)};
  const f128 z0r{d.re0[j], d.re1[j]}, z0i{d.im0[j], d.im1[j]};
  const f128 z1r{d.re0[j + t], d.re1[j + t]}, z1i{d.im0[j + t], d.im1[j + t]};
  const f128 dr = sub_est(z0r, z1r), di = sub_est(z0i, z1i);
  const f128 ar = add_est(z0r, z1r), ai = add_est(z0i, z1i);
  f128 mr, mi;
  cplx_mul_conj(dr, di, wr, wi, mr, mi);
  d.re0[j] = ar.hi;
  d.re1[j] = ar.lo;
  d.im0[j] = ai.hi;
  d.im1[j] = ai.lo;
  d.re0[j + t] = mr.hi;
  d.re1[j + t] = mr.lo;
  d.im0[j + t] = mi.hi;
  d.im1[j + t] = mi.lo;
}

// One radix-2 stage of double-double butterflies with two warps per 32
// butterflies: warp 2k computes the real parts of both outputs of butterflies
// 32k .. 32k+31, warp 2k+1 their imaginary parts.  The real and imaginary
// parts of a butterfly share no operation (cplx_mul, cplx_mul_conj), so each
// half does exactly the operations of its outputs and the results are the
// one-thread butterfly's bits; the inverse's conjugate product needs the other
// half's difference, which passes through xs (4 doubles per butterfly of an
// iteration).  A barrier separates every read of an iteration's elements from
// the stores.  Warp-uniform halves keep each warp on one instruction stream.
// map(b, qa, qb, widx) gives butterfly b's elements and twiddle index; nb
// butterflies; every thread of the CTA calls it.
template <bool FWD, class Map>
__device__ __forceinline__ void f128_half_stage(F128Arrays s, double* xs, int nb, Map map, const F128Tw& tw,
                                                int tid, int nth) {
  const int h = (tid >> 5) & 1;
  const int bi = ((tid >> 6) << 5) + (tid & 31);
  const int step = nth >> 1;
  double* d0 = h ? s.im0 : s.re0;
  double* d1 = h ? s.im1 : s.re1;
  for (int b0 = 0; b0 < nb; b0 += step) {
    const int b = b0 + bi;
    const bool act = b < nb;
    int qa = 0, qb = 0;
    f128 u{0, 0}, v{0, 0}, dd{0, 0}, wr{0, 0}, wi{0, 0};
    if (act) {
      long widx;
      map(b, qa, qb, widx);
      wr = f128{__ldg(tw.re0 + widx), __ldg(tw.re1 + widx)};
      wi = f128{__ldg(tw.im0 + widx), __ldg(tw.im1 + widx)};
      const f128 z0{d0[qa], d1[qa]};
      if (FWD) {
        const f128 z1r{s.re0[qb], s.re1[qb]}, z1i{s.im0[qb], s.im1[qb]};
        // real: mul(z1r, wr) - mul(z1i, wi); imaginary: mul(z1i, wr) + mul(z1r, wi)
        const f128 z = h ? add_est(mul(z1i, wr), mul(z1r, wi)) : sub_est(mul(z1r, wr), mul(z1i, wi));
        u = add_est(z0, z);
        v = sub_est(z0, z);
      } else {
        const f128 z1{d0[qb], d1[qb]};
        dd = sub_est(z0, z1);  // dr (h = 0) or di (h = 1)
        u = add_est(z0, z1);
        double* x = xs + (((b - b0) << 1) + h) * 2;
        x[0] = dd.hi;
        x[1] = dd.lo;
      }
    }
    __syncthreads();  // every read of this iteration's elements is done
    if (act) {
      if (!FWD) {
        const double* x = xs + (((b - b0) << 1) + (h ^ 1)) * 2;
        const f128 od{x[0], x[1]};
        // real: mul(dr, wr) + mul(di, wi); imaginary: mul(di, wr) - mul(dr, wi)
        v = h ? sub_est(mul(dd, wr), mul(od, wi)) : add_est(mul(dd, wr), mul(od, wi));
      }
      d0[qa] = u.hi;
      d1[qa] = u.lo;
      d0[qb] = v.hi;
      d1[qb] = v.lo;
    }
    __syncthreads();  // the stores are done before the next reads
  }
}

// Stages of a transform of 2^log2n points restricted to one sub-block of
// 2^log2c points (sub-block index sb), all in shared memory.  Forward runs
// t = 2^(log2c-1) .. 1 (src/fft128/mod.rs:363-401), inverse t = 1 .. 2^(log2c-1)
// (src/fft128/mod.rs:1117-1154); twiddle index m + i uses the global block i.
template <bool FWD>
__device__ __forceinline__ void f128_stages_smem(F128Arrays s, int log2n, int log2c, long sb, const F128Tw& tw,
                                                 int tid, int nth) {
  const int half = 1 << (log2c - 1);  // butterflies per sub-block per stage
  for (int st = 0; st < log2c; ++st) {
    const int log2t = FWD ? (log2c - 1 - st) : st;
    const long t = 1L << log2t;
    const long m = 1L << (log2n - 1 - log2t);  // blocks of 2t in the whole transform
    for (int b = tid; b < half; b += nth) {
      const long i_local = b >> log2t;
      const long jj = b & (t - 1);
      const long j = (i_local << (log2t + 1)) + jj;
      const long i_global = (sb << (log2c - 1 - log2t)) + i_local;
      if (FWD) f128_fwd_bfly(s, j, t, tw, m + i_global);
      else f128_inv_bfly(s, j, t, tw, m + i_global);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- integers
// (double)(__int128)v, round to nearest even, on the integer pipe.
__device__ __forceinline__ double i128_to_f64_rne(uint64_t lo, uint64_t hi) {
  const bool neg = (hi >> 63) != 0;
  if (neg) {  // magnitude of the two's complement value
    lo = ~lo;
    hi = ~hi;
    lo += 1;
    if (lo == 0) hi += 1;
  }
  if (hi == 0 && lo == 0) return 0.0;
  int lz;
  uint64_t top, rest;  // top: normalised leading 64 bits, rest: sticky source
  if (hi != 0) {
    lz = __clzll((long long)hi);
    top = lz == 0 ? hi : ((hi << lz) | (lo >> (64 - lz)));
    rest = lz == 0 ? lo : (lo << lz);
  } else {
    const int l2 = __clzll((long long)lo);
    lz = 64 + l2;
    top = lo << l2;
    rest = 0;
  }
  uint64_t m = top >> 11;
  const uint64_t r = top & 0x7ff;
  uint64_t e = (uint64_t)(1023 + 127 - lz);
  const bool sticky = rest != 0;
  if (r > 0x400 || (r == 0x400 && (sticky || (m & 1)))) {
    m += 1;
    if (m == (1ull << 53)) {
      m >>= 1;
      e += 1;
    }
  }
  return __longlong_as_double((long long)((neg ? 0x8000000000000000ull : 0ull) | (e << 52) | (m & 0xfffffffffffffull)));
}

// trunc(x) as an integer mod 2^128 (lo, hi words), and x - trunc(x).
__device__ __forceinline__ void trunc_mod128(double x, uint64_t& lo, uint64_t& hi, double& frac) {
  const double t = trunc(x);
  frac = __dsub_rn(x, t);
  const uint64_t bits = (uint64_t)__double_as_longlong(t);
  const bool neg = (bits >> 63) != 0;
  const int bexp = (int)((bits >> 52) & 0x7ff);
  lo = hi = 0;
  if (bexp == 0x7ff || bexp == 0) return;
  const uint64_t m = (bits & 0xfffffffffffffull) | (1ull << 52);
  const int e = bexp - 1075;
  if (e >= 128) return;
  if (e >= 64) {
    hi = m << (e - 64);
  } else if (e > 11) {
    lo = m << e;
    hi = m >> (64 - e);
  } else if (e >= 0) {
    lo = m << e;
  } else {
    lo = (-e) >= 64 ? 0 : (m >> (-e));
  }
  if (neg) {
    lo = ~lo;
    hi = ~hi;
    lo += 1;
    if (lo == 0) hi += 1;
  }
}

// floor(hi + lo + 1/2) mod 2^128 for a double-double, exact.
__device__ __forceinline__ void round_half_up_mod128(double xhi, double xlo, uint64_t& rlo, uint64_t& rhi) {
  uint64_t hl, hh, ll, lh;
  double fh, fl;
  trunc_mod128(xhi, hl, hh, fh);
  trunc_mod128(xlo, ll, lh, fl);
  double s, e;
  two_sum(fh, fl, s, e);
  const int f = -2 + (int)(s > -1.5 || (s == -1.5 && e >= 0.0)) + (int)(s > -0.5 || (s == -0.5 && e >= 0.0)) +
                (int)(s > 0.5 || (s == 0.5 && e >= 0.0)) + (int)(s > 1.5 || (s == 1.5 && e >= 0.0));
  uint64_t lo = hl + ll;
  uint64_t hi = hh + lh + (lo < hl ? 1 : 0);
  const uint64_t flo = (uint64_t)(int64_t)f;
  const uint64_t fhi = f < 0 ? ~0ull : 0ull;
  const uint64_t lo2 = lo + flo;
  hi = hi + fhi + (lo2 < lo ? 1 : 0);
  rlo = lo2;
  rhi = hi;
}

}  // namespace cfft
