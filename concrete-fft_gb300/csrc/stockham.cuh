// stockham.cuh -- the reference's transform structure, executed by one CTA.
//
// A CTA owns `nchunks` independent transforms of 2^log2n points stored back to
// back in shared memory and runs the reference's passes over all of them at
// once: every pass is a loop of radix-R butterflies over the CTA's threads,
// ping-ponging between two shared buffers, with one barrier per pass.  The
// unordered outer passes (radix 2/4/8 over the whole transform, src/
// unordered.rs:222-293) run in place before (forward) or after (inverse) the
// ordered base transforms.
#pragma once
#include "cfft_device.cuh"

namespace cfft {

template <int R>
struct Log2;
template <>
struct Log2<2> {
  static constexpr int v = 1;
};
template <>
struct Log2<4> {
  static constexpr int v = 2;
};
template <>
struct Log2<8> {
  static constexpr int v = 3;
};
template <>
struct Log2<16> {
  static constexpr int v = 4;
};

// Buffers are reached through an accessor (FlatBuf: a plain pointer into
// shared or global memory) and passes are separated by a barrier functor
// (CtaSync), so the pass code does not fix where a buffer lives or which
// threads share it.
struct FlatBuf {
  double2* p;
  __device__ __forceinline__ double2* at(int i) const { return p + i; }
};
struct CtaSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// One generic Stockham pass of radix R at stride s = 2^log2s
// (src/dif4.rs:118-168 for DIF, src/dit4.rs:94-140 for DIT, same for radix 2/8/16).
// DIF: in[k] = src[k*n/R + p*s + q], dst[R*s*p + k*s + q] = w_k * core(in)_k.
// DIT: in[k] = w_k * src[R*s*p + k*s + q], dst[k*n/R + p*s + q] = core(in)_k.
// w is the second half of the init_wt table: w_k = w[R*s*p + k].
// twlog: the pass runs on one residue class mod 2^twlog of a transform 2^twlog
// times larger, compacted (see split.cuh); its twiddles are those of the full
// transform's stride s * 2^twlog.  0 for a whole transform.
//
// Half butterflies (HALF, compiled into the split kernels only): when the CTA
// has at least twice as many threads as the pass has butterflies (a multiple
// of 32), a DIF pass gives each
// butterfly two threads, the first `total` threads computing its even outputs
// and the next `total` its odd ones (CoreHalf: the same operations, none
// repeated), so whole warps take one half.  Twiddles multiply the outputs
// after the core, so each half twiddles its own.
template <int R, bool FWD, bool DIT, int E, bool HALF = false, class B>
__device__ __forceinline__ void stockham_pass(int log2n, int log2s, int nchunks, B src, B dst,
                                              const double2* __restrict__ w, int tid, int nth, int twlog = 0) {
  constexpr int LR = Log2<R>::v;
  const int lper = log2n - LR;  // log2(n / R): butterflies per chunk
  const int total = nchunks << lper;
  const int smask = (1 << log2s) - 1;
  if constexpr (HALF && !DIT && E == 0) {
    if (nth >= 2 * total && (total & 31) == 0) {
      if (tid < 2 * total) {
        const int h = tid >= total ? 1 : 0;
        const int b = tid - h * total;
        const int base = (b >> lper) << log2n;
        const int bb = b & ((1 << lper) - 1);
        const int p = bb >> log2s;
        const int q = bb & smask;
        const double2* tw = w + (p << (log2s + twlog + LR));
        c64 v[R];
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = ld(src.at(base + (k << lper) + (p << log2s) + q));
        const int o = base + (p << (log2s + LR)) + q;
        c64 y[R / 2];
        if (h == 0) {
          CoreHalf<R, FWD, 0>::run(v, y);
          st(dst.at(o), y[0]);
#pragma unroll
          for (int j = 1; j < R / 2; ++j) st(dst.at(o + ((2 * j) << log2s)), cmul(ldg(tw + 2 * j), y[j]));
        } else {
          CoreHalf<R, FWD, 1>::run(v, y);
#pragma unroll
          for (int j = 0; j < R / 2; ++j) st(dst.at(o + ((2 * j + 1) << log2s)), cmul(ldg(tw + 2 * j + 1), y[j]));
        }
      }
      return;
    }
  }
  for (int b = tid; b < total; b += nth) {
    const int base = (b >> lper) << log2n;
    const int bb = b & ((1 << lper) - 1);
    const int p = bb >> log2s;
    const int q = bb & smask;
    const double2* tw = w + (p << (log2s + twlog + LR));
    c64 v[R];
    if (!DIT) {
#pragma unroll
      for (int k = 0; k < R; ++k) v[k] = ld(src.at(base + (k << lper) + (p << log2s) + q));
      Core<R, FWD, E>::run(v);
      const int o = base + (p << (log2s + LR)) + q;
      st(dst.at(o), v[0]);
#pragma unroll
      for (int k = 1; k < R; ++k) st(dst.at(o + (k << log2s)), cmul(ldg(tw + k), v[k]));
    } else {
      const int i0 = base + (p << (log2s + LR)) + q;
      v[0] = ld(src.at(i0));
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = cmul(ldg(tw + k), ld(src.at(i0 + (k << log2s))));
      Core<R, FWD, E>::run(v);
#pragma unroll
      for (int k = 0; k < R; ++k) st(dst.at(base + (k << lper) + (p << log2s) + q), v[k]);
    }
  }
}

// End butterfly of size M at stride n/M, in place (src/dif4.rs:195-244 and twins).
// It splits into half butterflies as stockham_pass does; being in
// place, every half loads its inputs before a CTA barrier and stores after it
// (every thread of the CTA calls this function).
template <int M, bool FWD, int E, bool HALF = false, class B>
__device__ __forceinline__ void end_pass(int log2n, int nchunks, B x, int tid, int nth) {
  constexpr int LM = Log2<M>::v;
  const int log2s = log2n - LM;
  const int total = nchunks << log2s;
  const int smask = (1 << log2s) - 1;
  if constexpr (HALF && E == 0) {
    if (nth >= 2 * total && (total & 31) == 0) {
      const bool act = tid < 2 * total;
      const int h = tid >= total ? 1 : 0;
      const int g = tid - h * total;
      const int base = act ? ((g >> log2s) << log2n) + (g & smask) : 0;
      c64 v[M];
      if (act) {
#pragma unroll
        for (int k = 0; k < M; ++k) v[k] = ld(x.at(base + (k << log2s)));
      }
      __syncthreads();
      if (act) {
        c64 y[M / 2];
        if (h == 0) CoreHalf<M, FWD, 0>::run(v, y);
        else CoreHalf<M, FWD, 1>::run(v, y);
#pragma unroll
        for (int j = 0; j < M / 2; ++j) st(x.at(base + ((2 * j + h) << log2s)), y[j]);
      }
      return;
    }
  }
  for (int g = tid; g < total; g += nth) {
    const int base = ((g >> log2s) << log2n) + (g & smask);
    c64 v[M];
#pragma unroll
    for (int k = 0; k < M; ++k) v[k] = ld(x.at(base + (k << log2s)));
    Core<M, FWD, E>::run(v);
#pragma unroll
    for (int k = 0; k < M; ++k) st(x.at(base + (k << log2s)), v[k]);
  }
}

template <int R, bool FWD, int E, bool HALF = false, class B>
__device__ __forceinline__ void end_dispatch(int lm, int log2n, int nchunks, B x, int tid, int nth) {
  if (lm == 1) end_pass<2, FWD, E, HALF>(log2n, nchunks, x, tid, nth);
  if constexpr (R >= 4) {
    if (lm == 2) end_pass<4, FWD, E, HALF>(log2n, nchunks, x, tid, nth);
  }
  if constexpr (R >= 8) {
    if (lm == 3) end_pass<8, FWD, E, HALF>(log2n, nchunks, x, tid, nth);
  }
  if constexpr (R >= 16) {
    if (lm == 4) end_pass<16, FWD, E, HALF>(log2n, nchunks, x, tid, nth);
  }
}

// The ordered transform of src/dif{R}.rs / src/dit{R}.rs (recursion e.g.
// src/dif4.rs:285-303): DIF runs radix-R passes at s = 1, R, R^2, ... while the
// remaining size exceeds R, then the end butterfly of the remaining size; DIT
// runs the end butterfly first at the largest stride, then the passes in
// reverse.  Returns the buffer (x or y) that holds the result.
template <int R, bool FWD, bool DIT, int E, class B = FlatBuf, class S = CtaSync>
__device__ B stockham_t(int log2n, int nchunks, B x, B y, const double2* __restrict__ w, int tid, int nth) {
  constexpr int LR = Log2<R>::v;
  const S sync{};
  if (log2n == 0) return x;
  int lm = log2n, npass = 0;
  while (lm > LR) {
    lm -= LR;
    ++npass;
  }
  B cur = x;
  B oth = y;
  if (!DIT) {
    for (int i = 0; i < npass; ++i) {
      stockham_pass<R, FWD, false, E>(log2n, i * LR, nchunks, cur, oth, w, tid, nth);
      sync();
      const B t = cur;
      cur = oth;
      oth = t;
    }
    end_dispatch<R, FWD, E>(lm, log2n, nchunks, cur, tid, nth);
    sync();
  } else {
    end_dispatch<R, FWD, E>(lm, log2n, nchunks, cur, tid, nth);
    sync();
    for (int i = npass - 1; i >= 0; --i) {
      stockham_pass<R, FWD, true, E>(log2n, i * LR, nchunks, cur, oth, w, tid, nth);
      sync();
      const B t = cur;
      cur = oth;
      oth = t;
    }
  }
  return cur;
}

template <int R, bool FWD, bool DIT, int E>
__device__ double2* stockham_smem(int log2n, int nchunks, double2* x, double2* y, const double2* __restrict__ w,
                                  int tid, int nth) {
  return stockham_t<R, FWD, DIT, E>(log2n, nchunks, FlatBuf{x}, FlatBuf{y}, w, tid, nth).p;
}

// ---------------------------------------------------------------------------
// Unordered outer passes (src/unordered.rs:222-293).  A level of size
// nl = 2^log2nl splits each chunk into r slices of m = nl/r points.  Forward:
// butterfly inputs z[k*m + i], outputs (twiddled after the core) stored to
// slot bitrev(k); inverse: inputs read from slot bitrev(k), twiddled before the
// core, outputs to z[k*m + i].  Level twiddles: w_k = wl[(r-1)*i + k-1].
template <int R>
__device__ __forceinline__ int slot(int k) {
  if constexpr (R == 2) return k;
  if constexpr (R == 4) return ((k & 1) << 1) | (k >> 1);
  return ((k & 1) << 2) | (k & 2) | (k >> 2);
}

template <int R, bool FWD, int E, class B>
__device__ __forceinline__ void outer_group_t(B z, int zc, int lm, int i, const double2* __restrict__ wl) {
  c64 v[R];
  const double2* tw = wl + (R - 1) * i - 1;  // tw[k] = w_k, k >= 1
  if (FWD) {
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = ld(z.at(zc + (k << lm) + i));
    Core<R, true, E>::run(v);
#pragma unroll
    for (int k = 1; k < R; ++k) v[k] = cmul(ldg(tw + k), v[k]);
#pragma unroll
    for (int k = 0; k < R; ++k) st(z.at(zc + (slot<R>(k) << lm) + i), v[k]);
  } else {
    v[0] = ld(z.at(zc + i));
#pragma unroll
    for (int k = 1; k < R; ++k) v[k] = cmul(ldg(tw + k), ld(z.at(zc + (slot<R>(k) << lm) + i)));
    Core<R, false, E>::run(v);
#pragma unroll
    for (int k = 0; k < R; ++k) st(z.at(zc + (k << lm) + i), v[k]);
  }
}

template <int R, bool FWD, int E>
__device__ __forceinline__ void outer_group(double2* zc, int lm, int i, const double2* __restrict__ wl) {
  outer_group_t<R, FWD, E>(FlatBuf{zc}, 0, lm, i, wl);
}

// One level over `nchunks` chunks of 2^log2nl points stored back to back.
template <bool FWD, int E, class B = FlatBuf>
__device__ __forceinline__ void outer_level_t(int log2r, int log2nl, int nchunks, B z, const double2* __restrict__ wl,
                                              int tid, int nth) {
  const int lm = log2nl - log2r;
  const int total = nchunks << lm;
  for (int g = tid; g < total; g += nth) {
    const int zc = (g >> lm) << log2nl;
    const int i = g & ((1 << lm) - 1);
    if (log2r == 1) outer_group_t<2, FWD, E>(z, zc, lm, i, wl);
    else if (log2r == 2) outer_group_t<4, FWD, E>(z, zc, lm, i, wl);
    else outer_group_t<8, FWD, E>(z, zc, lm, i, wl);
  }
}

template <bool FWD, int E>
__device__ __forceinline__ void outer_level(int log2r, int log2nl, int nchunks, double2* z,
                                            const double2* __restrict__ wl, int tid, int nth) {
  outer_level_t<FWD, E>(log2r, log2nl, nchunks, FlatBuf{z}, wl, tid, nth);
}

// Device copy of the level structure (see LevelDesc in cfft_internal.h).
struct DevLevels {
  int nlevels;
  int log2n[9];
  int log2r[8];
  int w_off[9];
  int winv_off[8];
};

template <int ALGO>
struct AlgoInfo {
  static constexpr int R = 2 << (ALGO / 2);
  static constexpr bool DIT = (ALGO & 1) != 0;
};

// Unordered transform of `nchunks` (sub)transforms of size n_{d0} held in x:
// fwd_depth (src/unordered.rs:392-439) or inv_depth (:442-489) from level d0,
// with the ordered base algorithm ALGO.  w: the plan's forward table
// (forward) or inverse table (inverse).
template <bool FWD, int E, int ALGO, class B = FlatBuf, class S = CtaSync>
__device__ B unordered_t(const DevLevels& L, int d0, int nchunks, B x, B y, const double2* __restrict__ w, int tid,
                         int nth) {
  constexpr int R = AlgoInfo<ALGO>::R;
  constexpr bool DIT = AlgoInfo<ALGO>::DIT;
  const S sync{};
  const int log2base = L.log2n[L.nlevels];
  const int log2sub = L.log2n[d0];
  const int nbase = nchunks << (log2sub - log2base);
  if (FWD) {
    for (int l = d0; l < L.nlevels; ++l) {
      outer_level_t<true, E>(L.log2r[l], L.log2n[l], nchunks << (log2sub - L.log2n[l]), x, w + L.w_off[l], tid, nth);
      sync();
    }
    return stockham_t<R, true, DIT, E, B, S>(log2base, nbase, x, y, w + L.w_off[L.nlevels] + (1 << log2base), tid,
                                             nth);
  } else {
    B r = stockham_t<R, false, DIT, E, B, S>(log2base, nbase, x, y, w + (1 << log2base), tid, nth);
    for (int l = L.nlevels - 1; l >= d0; --l) {
      outer_level_t<false, E>(L.log2r[l], L.log2n[l], nchunks << (log2sub - L.log2n[l]), r, w + L.winv_off[l], tid,
                              nth);
      sync();
    }
    return r;
  }
}

// Unordered transform of `nchunks` (sub)transforms of size n_{d0} held in x
// (shared memory of one CTA): fwd_depth (src/unordered.rs:392-439) or
// inv_depth (:442-489) from level d0, with the ordered base algorithm ALGO.
// w: the plan's forward table (forward) or inverse table (inverse).
template <bool FWD, int E, int ALGO>
__device__ double2* unordered_smem(const DevLevels& L, int d0, int nchunks, double2* x, double2* y,
                                   const double2* __restrict__ w, int tid, int nth) {
  return unordered_t<FWD, E, ALGO>(L, d0, nchunks, FlatBuf{x}, FlatBuf{y}, w, tid, nth).p;
}

// Integer-add levels (eighths of the butterfly additions on the integer pipe)
// that have kernel instantiations.  E = 0 exists for every algorithm; E = 4
// only for the radix-4 algorithms (Dif4, Dit4).  Measured on GB300 the
// integer-pipe add issues at half the FP64 add rate and raises register
// pressure, so E = 0 is the default and the tuner's usual choice.
constexpr int kEmuLevels[] = {0, 4};
inline int emu_level_for(int algo, int e) {
  if (algo != 2 && algo != 3) return 0;
  int best = 0;
  for (int v : kEmuLevels)
    if (v <= e) best = v;
  return best;
}

}  // namespace cfft
