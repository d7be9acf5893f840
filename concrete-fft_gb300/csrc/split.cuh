// split.cuh -- one c64 transform spread over S = 2^LS CTAs, with at most one
// exchange between them.
//
// A Stockham pass at stride s >= S only combines elements whose indices agree
// mod S: its inputs k*n/R + p*s + q and outputs R*s*p + k*s + q are all
// congruent to q.  So after the first DIF pass (s = 1) the residue classes mod
// S are independent problems of n/S points, which keep the full transform's
// twiddles (at stride s); before the last DIT pass the same holds in reverse.
// Likewise the unordered outer level 0 of radix r splits a transform into r
// contiguous slices that the later levels and the base treat independently.
//
// The S CTAs of a transform form a thread-block cluster.
//
// "First" kernels: the first step's butterflies are shared out, 1/S per CTA;
// each CTA reads its butterflies' inputs from global memory and stores every
// output into the part that holds its residue class (distributed shared
// memory), so no arithmetic is repeated; then each CTA finishes its part alone
// and stores it.  The transform is updated in place, and the cluster barrier
// after the first step also orders every read of it before any store.  Used
// for DIF-structured transforms (ordered DIF algorithms, the unordered base
// with no outer levels).
//
// The forward unordered transform with levels exchanges once instead: each
// CTA loads its own part, and level 0 takes 1/S of the butterflies per CTA,
// reading inputs from and storing outputs to the parts that hold them
// (distributed shared memory), so no arithmetic is repeated.
//
// "Last" kernels: each CTA loads its part and runs everything but the last
// step alone; the last step reads the other parts through distributed shared
// memory.  Used for DIT-structured transforms and for the inverse unordered
// transform with levels.
//
// Each butterfly does the same operations on the same values as in the
// one-CTA kernels, so results are bit-identical.
#pragma once
#include <cooperative_groups.h>

#include "stockham.cuh"

namespace cfft {

// Passes 1 .. npass-1 and the end butterfly of a DIF transform of 2^log2n
// points, run on one residue class mod 2^LS compacted to 2^(log2n - LS) points.
template <int R, bool FWD>
__device__ __forceinline__ FlatBuf dif_after_first(int log2n, int ls, FlatBuf x, FlatBuf y,
                                                   const double2* __restrict__ wb, int tid, int nth) {
  constexpr int LR = Log2<R>::v;
  int lm = log2n, npass = 0;
  while (lm > LR) {
    lm -= LR;
    ++npass;
  }
  const int log2c = log2n - ls;
  FlatBuf cur = x, oth = y;
  for (int i = 1; i < npass; ++i) {
    stockham_pass<R, FWD, false, 0, true>(log2c, i * LR - ls, 1, cur, oth, wb, tid, nth, ls);
    __syncthreads();
    const FlatBuf t = cur;
    cur = oth;
    oth = t;
  }
  end_dispatch<R, FWD, 0, true>(lm, log2c, 1, cur, tid, nth);
  __syncthreads();
  return cur;
}

// The end butterfly and passes npass-1 .. 1 of a DIT transform, on one
// residue class mod 2^LS (compacted), i.e. everything but the s = 1 pass.
template <int R, bool FWD>
__device__ __forceinline__ FlatBuf dit_before_last(int log2n, int ls, FlatBuf x, FlatBuf y,
                                                   const double2* __restrict__ wb, int tid, int nth) {
  constexpr int LR = Log2<R>::v;
  int lm = log2n, npass = 0;
  while (lm > LR) {
    lm -= LR;
    ++npass;
  }
  const int log2c = log2n - ls;
  FlatBuf cur = x, oth = y;
  end_dispatch<R, FWD, 0>(lm, log2c, 1, cur, tid, nth);
  __syncthreads();
  for (int i = npass - 1; i >= 1; --i) {
    stockham_pass<R, FWD, true, 0>(log2c, i * LR - ls, 1, cur, oth, wb, tid, nth, ls);
    __syncthreads();
    const FlatBuf t = cur;
    cur = oth;
    oth = t;
  }
  return cur;
}

// Forward unordered level 0 of radix R0 for butterflies [i0, i1): inputs from
// the parts `src[j]` (part j holds slices [j*R0/S, (j+1)*R0/S)), each output
// stored into the part that owns its slot (`dst[j]`).
template <int R0, int LS>
__device__ __forceinline__ void level0_scatter(double2* const* src, double2* const* dst, int lm, int i0, int i1,
                                               const double2* __restrict__ wl, int tid, int nth) {
  constexpr int LR0 = Log2<R0>::v;
  constexpr int SL = R0 >> LS;  // slices per part
  for (int i = i0 + tid; i < i1; i += nth) {
    c64 v[R0];
#pragma unroll
    for (int k = 0; k < R0; ++k) v[k] = ld(src[k / SL] + ((k % SL) << lm) + i);
    Core<R0, true, 0>::run(v);
    const double2* tw = wl + (R0 - 1) * i - 1;
#pragma unroll
    for (int k = 0; k < R0; ++k) {
      const c64 o = k == 0 ? v[0] : cmul(ldg(tw + k), v[k]);
      const int sl = slot<R0>(k);
      st(dst[sl >> (LR0 - LS)] + ((sl & (SL - 1)) << lm) + i, o);
    }
  }
}

// Inverse unordered level 0 of radix R0 for butterflies [i0, i1): inputs from
// the cluster's parts (part j holds slots [j*R0/S, (j+1)*R0/S) at `peer[j]`),
// outputs to global g.
template <int R0, int LS>
__device__ __forceinline__ void level0_last(double2* g, int lm, double2* const* peer, int i0, int i1,
                                            const double2* __restrict__ wl, int tid, int nth) {
  constexpr int LR0 = Log2<R0>::v;
  for (int i = i0 + tid; i < i1; i += nth) {
    c64 v[R0];
    const double2* tw = wl + (R0 - 1) * i - 1;
    v[0] = ld(peer[0] + i);
#pragma unroll
    for (int k = 1; k < R0; ++k) {
      const int sl = slot<R0>(k);
      v[k] = cmul(ldg(tw + k), ld(peer[sl >> (LR0 - LS)] + ((sl & ((R0 >> LS) - 1)) << lm) + i));
    }
    Core<R0, false, 0>::run(v);
#pragma unroll
    for (int k = 0; k < R0; ++k) st(g + (k << lm) + i, v[k]);
  }
}

// The first (s = 1) pass of a DIF transform over its cluster, for `per`
// butterflies: butterfly b is p = p0 + b * pstep, load(k, b, p) gives its
// input k (of R), and each output (p*R + k) is stored into the part of its
// residue class mod S (distributed shared memory), compacted.  Every thread
// calls before_store() once, before its first store (warp-uniformly): a
// cluster barrier's wait there overlaps the barrier with the loads.  With
// twice as many threads as butterflies (a multiple of 32), the butterflies are
// split into halves as in stockham_pass.
struct NoWait {
  __device__ void operator()() const {}
};
template <int R, bool FWD, int LS, class Load, class Wait = NoWait>
__device__ __forceinline__ void first_pass_scatter(Load load, int per, int p0, int pstep, double2* const* part,
                                                   const double2* __restrict__ wb, int tid, int nth,
                                                   Wait before_store = Wait{}) {
  constexpr int LR = Log2<R>::v;
  constexpr int S = 1 << LS;
  if (nth >= 2 * per && (per & 31) == 0) {
    if (tid >= 2 * per) {
      before_store();
    } else {
      const int h = tid >= per ? 1 : 0;
      const int b = tid - h * per;
      const int p = p0 + b * pstep;
      c64 v[R];
#pragma unroll
      for (int k = 0; k < R; ++k) v[k] = load(k, b, p);
      const double2* tw = wb + (p << LR);
      c64 y[R / 2];
      before_store();
      if (h == 0) {
        CoreHalf<R, FWD, 0>::run(v, y);
        st(part[0] + ((p << LR) >> LS), y[0]);
#pragma unroll
        for (int j = 1; j < R / 2; ++j)
          st(part[(2 * j) & (S - 1)] + (((p << LR) + 2 * j) >> LS), cmul(ldg(tw + 2 * j), y[j]));
      } else {
        CoreHalf<R, FWD, 1>::run(v, y);
#pragma unroll
        for (int j = 0; j < R / 2; ++j)
          st(part[(2 * j + 1) & (S - 1)] + (((p << LR) + 2 * j + 1) >> LS), cmul(ldg(tw + 2 * j + 1), y[j]));
      }
    }
    return;
  }
  before_store();
  for (int b = tid; b < per; b += nth) {
    const int p = p0 + b * pstep;
    c64 v[R];
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = load(k, b, p);
    Core<R, FWD, 0>::run(v);
    const double2* tw = wb + (p << LR);
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const c64 o = k == 0 ? v[0] : cmul(ldg(tw + k), v[k]);
      st(part[k & (S - 1)] + (((p << LR) + k) >> LS), o);
    }
  }
}

// The first pass of a DIF transform held in global memory: CTA c takes the
// butterflies [c*per, (c+1)*per) in full -- no output is computed twice --
// reading their inputs from g.
template <int R, bool FWD, int LS, class Wait>
__device__ __forceinline__ void dif_first_scatter(const double2* g, int lper, int c, double2* const* part,
                                                  const double2* __restrict__ wb, int tid, int nth,
                                                  Wait before_store) {
  const int per = (1 << lper) >> LS;
  first_pass_scatter<R, FWD, LS>([&](int k, int, int p) { return ld(g + (k << lper) + p); }, per, c * per, 1, part,
                                 wb, tid, nth, before_store);
}

// MODE 0: the plan has no outer levels (ordered plan, or unordered with
// n = base_n); the base algorithm's structure decides (DIF: first, DIT: last).
// MODE 1: unordered with outer levels (forward: first, inverse: last).
// One transform per S consecutive CTAs; w is the plan's forward table
// (forward) or inverse table (inverse).
template <int ALGO, bool FWD, int LS, int MODE>
__global__ void __launch_bounds__(256) c64_split_kernel(double2* data, DevLevels L, const double2* __restrict__ w) {
  constexpr int R = AlgoInfo<ALGO>::R;
  constexpr int LR = Log2<R>::v;
  constexpr int S = 1 << LS;
  constexpr bool LAST = MODE == 0 ? AlgoInfo<ALGO>::DIT : !FWD;
  extern __shared__ double2 smem[];
  grid_dependency_wait();
  const int log2n = L.log2n[0];
  const int log2c = log2n - LS;
  const int c = (int)(blockIdx.x & (S - 1));
  const long t = blockIdx.x >> LS;
  double2* g = data + (t << log2n);
  double2* xs = smem;
  double2* ys = smem + (1 << log2c);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int log2base = L.log2n[L.nlevels];
  const double2* wb = FWD ? w + L.w_off[L.nlevels] + (1 << log2base) : w + (1 << log2base);

  if constexpr (MODE == 0 && !LAST) {
    // DIF: pass 0 (s = 1) over the cluster, 1/S of the butterflies per CTA, each
    // output stored into the part of its residue class; then this class alone.
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    double2* part[S];
#pragma unroll
    for (int j = 0; j < S; ++j) part[j] = cl.map_shared_rank(xs, (unsigned)j);
    // every CTA of the cluster runs before its shared memory is written: the barrier's
    // wait comes after the first pass's loads
    auto token = cl.barrier_arrive();
    dif_first_scatter<R, FWD, LS>(g, log2n - LR, c, part, wb, tid, nth,
                                  [&] { cl.barrier_wait(std::move(token)); });
    cl.sync();  // every part is complete, and every read of the transform in global memory is done
    const FlatBuf r = dif_after_first<R, FWD>(log2n, LS, FlatBuf{xs}, FlatBuf{ys}, wb, tid, nth);
    for (int j = tid; j < (1 << log2c); j += nth) g[(j << LS) + c] = r.p[j];
  } else if constexpr (MODE == 0 && LAST) {
    // DIT: own residue class through every pass but the last, then the s = 1
    // pass over the cluster.
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    for (int j = tid; j < (1 << log2c); j += nth) xs[j] = g[(j << LS) + c];
    __syncthreads();
    const FlatBuf r = dit_before_last<R, FWD>(log2n, LS, FlatBuf{xs}, FlatBuf{ys}, wb, tid, nth);
    double2* peer[S];
#pragma unroll
    for (int j = 0; j < S; ++j) peer[j] = cl.map_shared_rank(r.p, (unsigned)j);
    cl.sync();
    const int lper = log2n - LR;
    const int per = (1 << lper) >> LS;
    for (int p = c * per + tid; p < (c + 1) * per; p += nth) {
      c64 v[R];
      const double2* tw = wb + (p << LR);
      const int lo = p << (LR - LS);
      v[0] = ld(peer[0] + lo);
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = cmul(ldg(tw + k), ld(peer[k & (S - 1)] + lo + (k >> LS)));
      Core<R, FWD, 0>::run(v);
#pragma unroll
      for (int k = 0; k < R; ++k) st(g + (k << lper) + p, v[k]);
    }
    cl.sync();
  } else if constexpr (MODE == 1 && !LAST) {
    // forward unordered: each CTA loads its part; level 0 takes 1/S of the
    // butterflies per CTA, inputs from every part and each output stored into
    // the part that owns its slot (distributed shared memory); then levels 1..
    // and the base on the R0/S slices of this part.
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const double2* gp = g + ((long)c << log2c);
    for (int j = tid; j < (1 << log2c); j += nth) ys[j] = gp[j];
    double2* peer_y[S];
    double2* peer_x[S];
#pragma unroll
    for (int j = 0; j < S; ++j) {
      peer_y[j] = cl.map_shared_rank(ys, (unsigned)j);
      peer_x[j] = cl.map_shared_rank(xs, (unsigned)j);
    }
    cl.sync();
    const int lr0 = L.log2r[0];
    const int lm = log2n - lr0;
    const double2* wl = w + L.w_off[0];
    const int per = (1 << lm) >> LS;
    if (lr0 == 1) {
      if constexpr (LS <= 1) level0_scatter<2, LS>(peer_y, peer_x, lm, c * per, (c + 1) * per, wl, tid, nth);
    } else if (lr0 == 2) {
      if constexpr (LS <= 2) level0_scatter<4, LS>(peer_y, peer_x, lm, c * per, (c + 1) * per, wl, tid, nth);
    } else {
      level0_scatter<8, LS>(peer_y, peer_x, lm, c * per, (c + 1) * per, wl, tid, nth);
    }
    cl.sync();  // every part's xs is complete, and every peer is done reading this CTA's ys
    const FlatBuf r = unordered_t<true, 0, ALGO>(L, 1, 1 << (lr0 - LS), FlatBuf{xs}, FlatBuf{ys}, w, tid, nth);
    double2* gw = g + ((long)c << log2c);
    for (int j = tid; j < (1 << log2c); j += nth) gw[j] = r.p[j];
  } else {
    // inverse unordered: this part's slices through the base and levels
    // nlevels-1 .. 1, then level 0 over the cluster.
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const double2* gp = g + ((long)c << log2c);
    for (int j = tid; j < (1 << log2c); j += nth) xs[j] = gp[j];
    __syncthreads();
    const int lr0 = L.log2r[0];
    const int lm = log2n - lr0;
    const FlatBuf r = unordered_t<false, 0, ALGO>(L, 1, 1 << (lr0 - LS), FlatBuf{xs}, FlatBuf{ys}, w, tid, nth);
    double2* peer[S];
#pragma unroll
    for (int j = 0; j < S; ++j) peer[j] = cl.map_shared_rank(r.p, (unsigned)j);
    cl.sync();
    const double2* wl = w + L.winv_off[0];
    const int per = (1 << lm) >> LS;
    if (lr0 == 1) {
      if constexpr (LS <= 1) level0_last<2, LS>(g, lm, peer, c * per, (c + 1) * per, wl, tid, nth);
    } else if (lr0 == 2) {
      if constexpr (LS <= 2) level0_last<4, LS>(g, lm, peer, c * per, (c + 1) * per, wl, tid, nth);
    } else {
      level0_last<8, LS>(g, lm, peer, c * per, (c + 1) * per, wl, tid, nth);
    }
    cl.sync();
  }
}

// An unordered transform with exactly one outer level, of radix R0 = 2^LS0 <= 4,
// over a DIF base of m points, on a cluster of S = R0 x S1 CTAs (S1 = 2^LS1
// classes of the base, S <= 8): CTA c = s0 * S1 + c1 holds class c1 (mod S1)
// of slice s0, i.e. the slice's points j * S1 + c1 after the base's first pass.
// Forward: CTA c takes 1/S of level 0's butterflies from global memory and
// stores output k (slice slot(k), point i) into the staging buffer of the CTA
// of that slice that computes the base's first-pass butterfly i mod (m/R);
// after a cluster barrier the CTAs of a slice share out its first pass, each
// output into the part of its class; after a second barrier the rest is local.
// Inverse: each CTA loads its class, whose inverse first-pass butterflies
// (p = c1 + b*S1) read only that class, stores each output into the part of its
// class, finishes the base inverse locally, and after a barrier takes 1/S of
// level 0's butterflies, reading point i of every slice from the CTA that
// holds its class.  The same operations on the same values as the one-CTA
// kernel, in place.
template <int ALGO, bool FWD, int LS0, int LS1>
__global__ void __launch_bounds__(256) c64_split2_kernel(double2* data, DevLevels L, const double2* __restrict__ w) {
  constexpr int R = AlgoInfo<ALGO>::R;
  constexpr int LR = Log2<R>::v;
  constexpr int R0 = 1 << LS0;
  constexpr int S1 = 1 << LS1;
  constexpr int LS = LS0 + LS1;
  constexpr int S = 1 << LS;
  static_assert(!AlgoInfo<ALGO>::DIT, "DIF base algorithms only");
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ double2 smem[];
  grid_dependency_wait();
  const int log2n = L.log2n[0];
  const int log2m = L.log2n[1];
  const int m = 1 << log2m;
  const int log2c = log2m - LS1;
  const int c = (int)(blockIdx.x & (S - 1));
  const long t = blockIdx.x >> LS;
  const int s0 = c >> LS1, c1 = c & (S1 - 1);
  double2* g = data + (t << log2n);
  double2* xs = smem;
  double2* ys = smem + (1 << log2c);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lq = log2m - LR;
  const int lpp = lq - LS1;
  const int pp = 1 << lpp;
  const int cnt = m >> LS;  // level-0 butterflies per CTA
  const int i0 = c * cnt;
  double2* part[S1];
  if constexpr (FWD) {
    const double2* wl = w + L.w_off[0];
    const double2* wb = w + L.w_off[1] + m;
#pragma unroll
    for (int j = 0; j < S1; ++j) part[j] = cl.map_shared_rank(xs, (unsigned)((s0 << LS1) + j));
    auto token = cl.barrier_arrive();  // every CTA runs before a peer's memory is written
    c64 v0[R0];
    if (tid < cnt) {
#pragma unroll
      for (int k = 0; k < R0; ++k) v0[k] = ld(g + (k << log2m) + i0 + tid);
    }
    cl.barrier_wait(std::move(token));
    for (int b = tid; b < cnt; b += nth) {
      const int i = i0 + b;
      c64 v[R0];
#pragma unroll
      for (int k = 0; k < R0; ++k) v[k] = b == tid ? v0[k] : ld(g + (k << log2m) + i);
      Core<R0, true, 0>::run(v);
      const double2* twl = wl + (R0 - 1) * i - 1;
      const int p = i & ((1 << lq) - 1);
      const int dst = ((i >> lq) << lpp) + (p & (pp - 1));
      const int cls = p >> lpp;
#pragma unroll
      for (int k = 0; k < R0; ++k) {
        const c64 o = k == 0 ? v[0] : cmul(ldg(twl + k), v[k]);
        st(cl.map_shared_rank(ys, (unsigned)((slot<R0>(k) << LS1) + cls)) + dst, o);
      }
    }
    cl.sync();  // every staging buffer is complete; every read of the transform is done
    first_pass_scatter<R, true, LS1>([&](int k, int b, int) { return ld(ys + (k << lpp) + b); }, pp, c1 * pp, 1,
                                     part, wb, tid, nth);
    cl.sync();  // every part is complete
    const FlatBuf r = dif_after_first<R, true>(log2m, LS1, FlatBuf{xs}, FlatBuf{ys}, wb, tid, nth);
    double2* gs = g + ((long)s0 << log2m) + c1;
    for (int j = tid; j < (1 << log2c); j += nth) gs[j << LS1] = r.p[j];
  } else {
    const double2* wl = w + L.winv_off[0];
    const double2* wb = w + m;
#pragma unroll
    for (int j = 0; j < S1; ++j) part[j] = cl.map_shared_rank(ys, (unsigned)((s0 << LS1) + j));
    auto token = cl.barrier_arrive();
    const double2* gs = g + ((long)s0 << log2m) + c1;
    for (int j = tid; j < (1 << log2c); j += nth) xs[j] = gs[j << LS1];
    __syncthreads();
    cl.barrier_wait(std::move(token));
    first_pass_scatter<R, false, LS1>([&](int k, int b, int) { return ld(xs + (k << lpp) + b); }, pp, c1, S1, part,
                                      wb, tid, nth);
    cl.sync();  // every part is complete; every read of the transform is done
    const FlatBuf sv = dif_after_first<R, false>(log2m, LS1, FlatBuf{ys}, FlatBuf{xs}, wb, tid, nth);
    cl.sync();  // every slice is complete
    for (int b = tid; b < cnt; b += nth) {
      const int i = i0 + b;
      const int cls = i & (S1 - 1);
      const int at = i >> LS1;
      const double2* twl = wl + (R0 - 1) * i - 1;
      c64 v[R0];
      v[0] = ld(cl.map_shared_rank(sv.p, (unsigned)cls) + at);
#pragma unroll
      for (int k = 1; k < R0; ++k)
        v[k] = cmul(ldg(twl + k), ld(cl.map_shared_rank(sv.p, (unsigned)((slot<R0>(k) << LS1) + cls)) + at));
      Core<R0, false, 0>::run(v);
#pragma unroll
      for (int k = 0; k < R0; ++k) st(g + (k << log2m) + i, v[k]);
    }
    cl.sync();  // no CTA exits while a peer reads its shared memory
  }
}

// Kernel pointer for (ALGO, direction, LS, MODE); nullptr where S = 2^LS
// exceeds the radix that is split.
template <int A, int LS>
const void* split_ptr_ls(bool fwd, int mode) {
  if (mode == 0) {
    if constexpr (LS <= Log2<AlgoInfo<A>::R>::v)
      return fwd ? (const void*)c64_split_kernel<A, true, LS, 0> : (const void*)c64_split_kernel<A, false, LS, 0>;
    else
      return nullptr;
  }
  return fwd ? (const void*)c64_split_kernel<A, true, LS, 1> : (const void*)c64_split_kernel<A, false, LS, 1>;
}
// Mode 2 (R0 = 2), 3 (R0 = 4) and 4 (R0 = 8): c64_split2_kernel with S1 = 2^ls / R0,
// for DIF bases with S1 <= R and R0 * S1 <= 8, or 16 (4 x 4 and 8 x 2).
template <int A, int LS0>
const void* split2_ptr(bool fwd, int ls) {
  if constexpr (AlgoInfo<A>::DIT) {
    return nullptr;
  } else {
    constexpr int LRA = Log2<AlgoInfo<A>::R>::v;
    const int ls1 = ls - LS0;
    if constexpr (LS0 == 3 && LRA < 2) {
      return nullptr;
    } else {
      if (ls1 == 1)
        return fwd ? (const void*)c64_split2_kernel<A, true, LS0, 1> : (const void*)c64_split2_kernel<A, false, LS0, 1>;
    }
    if constexpr (LS0 <= 2 && LRA >= 2) {
      if (ls1 == 2)
        return fwd ? (const void*)c64_split2_kernel<A, true, LS0, 2> : (const void*)c64_split2_kernel<A, false, LS0, 2>;
    }
    return nullptr;
  }
}
template <int A>
const void* split_ptr(bool fwd, int ls, int mode) {
  if (mode == 2) return split2_ptr<A, 1>(fwd, ls);
  if (mode == 3) return split2_ptr<A, 2>(fwd, ls);
  if (mode == 4) return split2_ptr<A, 3>(fwd, ls);
  switch (ls) {
    case 1: return split_ptr_ls<A, 1>(fwd, mode);
    case 2: return split_ptr_ls<A, 2>(fwd, mode);
    case 3: return split_ptr_ls<A, 3>(fwd, mode);
    default: return nullptr;
  }
}

}  // namespace cfft
