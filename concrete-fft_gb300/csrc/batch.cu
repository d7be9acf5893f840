// batch.cu -- mixed-size c64 transforms in one persistent launch.
//
// A batch is a list of transforms of different power-of-two sizes and kinds
// (ordered n <= 1024, unordered n <= 65536) living anywhere in one device
// buffer.  At creation the host groups the items by (kind, size, direction)
// into work units of `tpc` same-size transforms, orders the units longest
// first, and picks each size class's schedule (base algorithm, base size,
// transforms per unit) by timing candidates on the device.  A run is a single
// persistent kernel: every CTA takes the next unit from a device counter
// (atomicAdd, no waiting on other CTAs), transforms it -- in shared memory up
// to 2048 points, with the unordered top levels in global memory above that --
// and takes the next, until the queue is empty.  Runs on a user stream are
// replayed from a CUDA graph captured on the first run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/cfft.h"
#include "cfft_internal.h"
#include "runtime.h"
#include "stockham.cuh"

using namespace cfft;

namespace cfft {

constexpr int kBatchSmemLog2 = 11;  // 2048 points x 2 buffers x 16 B = 64 KiB per CTA
constexpr int kBatchThreads = 256;

struct SizeClass {
  DevLevels L;
  const double2* w;
  const double2* winv;
  int algo;  // 2 (Dif4) or 4 (Dif8): the base algorithms compiled into the persistent kernel
  int d0;    // first level handled in shared memory
  int log2n;
};

struct Unit {
  int cls;
  int first;  // index into the sorted item-offset array
  int count;  // transforms in this unit (<= tpc of the class)
  int dir;    // 1 forward, 2 inverse, 3 forward then inverse
};

template <int ALGO>
__device__ void run_unit(double2* __restrict__ data, const SizeClass& C, const uint64_t* __restrict__ offs,
                         const Unit& U, double2* x, double2* y, int tid, int nth) {
  const int log2n = C.log2n;
  const int log2sub = C.L.log2n[C.d0];
  const bool fwd = U.dir & 1, inv = (U.dir & 2) != 0;
  if (C.d0 == 0) {
    // whole transforms in shared memory, U.count of them back to back
    const int n = 1 << log2n;
    for (int t = 0; t < U.count; ++t) {
      const double2* g = data + offs[U.first + t];
      for (int i = tid; i < n; i += nth) x[(t << log2n) + i] = g[i];
    }
    __syncthreads();
    double2* r = x;
    if (fwd) r = unordered_smem<true, 0, ALGO>(C.L, 0, U.count, x, y, C.w, tid, nth);
    if (inv) r = unordered_smem<false, 0, ALGO>(C.L, 0, U.count, r, r == x ? y : x, C.winv, tid, nth);
    for (int t = 0; t < U.count; ++t) {
      double2* g = data + offs[U.first + t];
      for (int i = tid; i < n; i += nth) g[i] = r[(t << log2n) + i];
    }
    __syncthreads();
    return;
  }
  // one large transform: top levels in global memory, sub-transforms in shared memory
  double2* g = data + offs[U.first];
  if (fwd) {
    for (int l = 0; l < C.d0; ++l) {
      outer_level<true, 0>(C.L.log2r[l], C.L.log2n[l], 1 << (log2n - C.L.log2n[l]), g, C.w + C.L.w_off[l], tid, nth);
      __syncthreads();
    }
  }
  const int nsub = 1 << (log2n - log2sub), m = 1 << log2sub;
  for (int c = 0; c < nsub; ++c) {
    double2* gc = g + ((long)c << log2sub);
    for (int i = tid; i < m; i += nth) x[i] = gc[i];
    __syncthreads();
    double2* r = x;
    if (fwd) r = unordered_smem<true, 0, ALGO>(C.L, C.d0, 1, x, y, C.w, tid, nth);
    if (inv) r = unordered_smem<false, 0, ALGO>(C.L, C.d0, 1, r, r == x ? y : x, C.winv, tid, nth);
    for (int i = tid; i < m; i += nth) gc[i] = r[i];
    __syncthreads();
  }
  if (inv) {
    for (int l = C.d0 - 1; l >= 0; --l) {
      outer_level<false, 0>(C.L.log2r[l], C.L.log2n[l], 1 << (log2n - C.L.log2n[l]), g, C.winv + C.L.winv_off[l], tid,
                            nth);
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(kBatchThreads, 2) batch_kernel(double2* __restrict__ data,
                                                             const SizeClass* __restrict__ classes,
                                                             const uint64_t* __restrict__ offs,
                                                             const Unit* __restrict__ units, int nunits,
                                                             unsigned int* __restrict__ head) {
  extern __shared__ double2 smem[];
  __shared__ int s_unit;
  double2* x = smem;
  double2* y = smem + (1 << kBatchSmemLog2);
  const int tid = threadIdx.x, nth = blockDim.x;
  for (;;) {
    if (tid == 0) s_unit = (int)atomicAdd(head, 1u);
    __syncthreads();
    const int u = s_unit;
    __syncthreads();
    if (u >= nunits) break;
    const Unit U = units[u];
    const SizeClass C = classes[U.cls];
    if (C.algo == 2) run_unit<2>(data, C, offs, U, x, y, tid, nth);
    else run_unit<4>(data, C, offs, U, x, y, tid, nth);
  }
}

}  // namespace cfft

// ============================================================ host side
namespace {

struct ClassKey {
  int kind, log2n, dir;
  bool operator<(const ClassKey& o) const { return std::tie(kind, log2n, dir) < std::tie(o.kind, o.log2n, o.dir); }
};

struct ClassHost {
  ClassKey key;
  int algo = 2, base_log2 = 10, tpc = 1;
  double2 *w = nullptr, *winv = nullptr;
  std::vector<uint64_t> items;  // offsets (points)
};

void free_tables(ClassHost& c) {
  if (c.w) cudaFree(c.w);
  if (c.winv) cudaFree(c.winv);
  c.w = c.winv = nullptr;
}

cfft_status build_tables(ClassHost& c) {
  free_tables(c);
  const size_t n = size_t(1) << c.key.log2n, base = size_t(1) << c.base_log2;
  std::vector<c64h> w(n + base), wi(n + base);
  unordered_twiddles(n, base, algo_radix(c.algo), w.data(), wi.data());
  cfft_status st = upload((const double2*)w.data(), n + base, &c.w);
  if (st == CFFT_OK) st = upload((const double2*)wi.data(), n + base, &c.winv);
  return st;
}

SizeClass device_class(const ClassHost& c) {
  const size_t n = size_t(1) << c.key.log2n, base = size_t(1) << c.base_log2;
  const LevelDesc lv = make_levels(n, base);
  SizeClass d;
  std::memset(&d, 0, sizeof(d));
  d.L.nlevels = lv.nlevels;
  for (int i = 0; i <= kMaxLevels; ++i) {
    d.L.log2n[i] = lv.log2n[i];
    d.L.w_off[i] = lv.w_off[i];
  }
  for (int i = 0; i < kMaxLevels; ++i) {
    d.L.log2r[i] = lv.log2r[i];
    d.L.winv_off[i] = lv.winv_off[i];
  }
  d.w = c.w;
  d.winv = c.winv;
  d.algo = c.algo;
  d.log2n = c.key.log2n;
  d.d0 = 0;
  while (lv.log2n[d.d0] > kBatchSmemLog2) ++d.d0;
  return d;
}

// Relative cost of one unit (FP64 work ~ n log n), for longest-first ordering.
double unit_cost(int log2n, int count, int dir) {
  return (double)count * (double)(1L << log2n) * log2n * ((dir == 3) ? 2 : 1);
}

cfft_status batch_attr() {
  return ensure_smem((const void*)batch_kernel, 2 * (1 << kBatchSmemLog2) * sizeof(double2));
}

}  // namespace

struct cfft_batch {
  std::vector<ClassHost> classes;
  std::vector<Unit> units;
  SizeClass* d_classes = nullptr;
  uint64_t* d_offs = nullptr;
  Unit* d_units = nullptr;
  unsigned int* d_head = nullptr;
  int grid = 0;
  size_t total_points = 0;
  // graph cache: one captured launch per (stream, data pointer)
  std::mutex mu;
  cudaStream_t g_stream = nullptr;
  double* g_data = nullptr;
  cudaGraphExec_t g_exec = nullptr;
  // pipelined host runs: the items split into data-contiguous chunks, each
  // with its own units and work counter (built on first use)
  struct Chunk {
    uint64_t lo = 0, hi = 0;  // point range [lo, hi) covered by the chunk's items
    uint64_t* d_offs = nullptr;
    Unit* d_units = nullptr;
    int nunits = 0;
  };
  std::vector<cfft_batch_item> items;
  std::vector<Chunk> chunks;
  unsigned int* d_heads = nullptr;
  cudaStream_t pstream[3] = {};
  cudaEvent_t pevent[4] = {};
};

namespace {

cfft_status launch_batch(cfft_batch* b, double2* data, cudaStream_t s) {
  CFFT_CUDA_TRY(cudaMemsetAsync(b->d_head, 0, sizeof(unsigned int), s));
  const size_t smem = 2 * (1 << kBatchSmemLog2) * sizeof(double2);
  batch_kernel<<<b->grid, kBatchThreads, smem, s>>>(data, b->d_classes, b->d_offs, b->d_units, (int)b->units.size(),
                                                     b->d_head);
  CFFT_CHECK_LAUNCH();
  return CFFT_OK;
}

void free_batch_device(cfft_batch* b) {
  if (b->d_classes) cudaFree(b->d_classes);
  if (b->d_offs) cudaFree(b->d_offs);
  if (b->d_units) cudaFree(b->d_units);
  b->d_classes = nullptr;
  b->d_offs = nullptr;
  b->d_units = nullptr;
}

// Builds units and uploads class descriptors, offsets and units.
cfft_status finalize(cfft_batch* b) {
  free_batch_device(b);
  b->units.clear();
  std::vector<uint64_t> offs;
  std::vector<SizeClass> dcls;
  std::vector<std::pair<double, Unit>> u;
  for (size_t ci = 0; ci < b->classes.size(); ++ci) {
    ClassHost& c = b->classes[ci];
    dcls.push_back(device_class(c));
    const int first = (int)offs.size();
    offs.insert(offs.end(), c.items.begin(), c.items.end());
    const int tpc = dcls.back().d0 == 0 ? c.tpc : 1;
    for (size_t k = 0; k < c.items.size(); k += (size_t)tpc) {
      Unit un{(int)ci, first + (int)k, (int)std::min<size_t>(tpc, c.items.size() - k), c.key.dir};
      u.push_back({unit_cost(c.key.log2n, un.count, un.dir), un});
    }
  }
  std::stable_sort(u.begin(), u.end(), [](const auto& a, const auto& bb) { return a.first > bb.first; });
  for (auto& p : u) b->units.push_back(p.second);
  cfft_status st = upload(dcls.data(), dcls.size(), &b->d_classes);
  if (st == CFFT_OK) st = upload(offs.data(), offs.size(), &b->d_offs);
  if (st == CFFT_OK) st = upload(b->units.data(), b->units.size(), &b->d_units);
  return st;
}

// FP64 instructions (DADD/DMUL/DFMA) of one unordered transform of 2^log2n points
// with the given base: the outer levels' radix-r butterflies plus r - 1 twiddle
// products each, the base's radix-R passes likewise, and its end butterfly.
double fp64_ops_per_point(int log2n, int base_log2, int algo) {
  auto core = [](int r) { return r == 2 ? 4.0 : r == 4 ? 16.0 : r == 8 ? 56.0 : 168.0; };
  const LevelDesc lv = make_levels(size_t(1) << log2n, size_t(1) << base_log2);
  double ops = 0;
  for (int l = 0; l < lv.nlevels; ++l) {
    const int r = 1 << lv.log2r[l];
    ops += (core(r) + 4.0 * (r - 1)) / r;
  }
  const int lr = ilog2((size_t)algo_radix(algo));
  int rem = base_log2;
  while (rem > lr) {
    rem -= lr;
    ops += (core(1 << lr) + 4.0 * ((1 << lr) - 1)) / (1 << lr);
  }
  if (rem > 0) ops += core(1 << rem) / (1 << rem);
  return ops;
}

// Times candidate schedules of one size class on a synthetic homogeneous batch.
// The class runs at the FP64 roof, so among candidates timed within 3% of the
// fastest (short timings are that noisy) the one with the fewest FP64
// instructions per point wins, and the time decides between equal counts.
cfft_status tune_class(cfft_batch* b, size_t ci, double seconds) {
  ClassHost& c = b->classes[ci];
  const int log2n = c.key.log2n;
  std::vector<std::tuple<int, int, int>> cands;  // (algo, base_log2, tpc)
  std::vector<int> bases;
  if (c.key.kind == 0) bases.push_back(log2n);  // ordered: the base is the transform
  else
    for (int bl : {9, 10})
      if (bl <= log2n) bases.push_back(bl);
  if (bases.empty()) bases.push_back(log2n);
  for (int bl : bases)
    for (int algo : {2, 4})
      for (int tpc : {1, 2, 4, 8}) {
        if (log2n > kBatchSmemLog2 && tpc > 1) continue;
        if (log2n <= kBatchSmemLog2 && (tpc << log2n) > (1 << kBatchSmemLog2)) continue;
        cands.emplace_back(algo, bl, tpc);
      }
  const size_t n = size_t(1) << log2n;
  const size_t count = std::max<size_t>(b->grid * 2, (size_t(1) << 21) >> log2n);  // >= 2 units per CTA
  double2* buf = nullptr;
  CFFT_CUDA_TRY(cudaMalloc(&buf, count * n * sizeof(double2)));
  CFFT_CUDA_TRY(cudaMemset(buf, 0, count * n * sizeof(double2)));
  cfft_batch tb;
  tb.grid = b->grid;
  CFFT_CUDA_TRY(cudaMalloc(&tb.d_head, sizeof(unsigned int)));
  cudaStream_t s;
  CFFT_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  std::vector<double> times;
  cfft_status st = CFFT_OK;
  for (auto cand : cands) {
    ClassHost t;
    t.key = c.key;
    std::tie(t.algo, t.base_log2, t.tpc) = cand;
    for (size_t i = 0; i < count; ++i) t.items.push_back(i * n);
    st = build_tables(t);
    if (st != CFFT_OK) break;
    tb.classes.clear();
    tb.classes.push_back(t);
    st = finalize(&tb);
    if (st != CFFT_OK) break;
    launch_batch(&tb, buf, s);
    int reps = 1;
    double per = 0;
    for (;;) {
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps; ++r) launch_batch(&tb, buf, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      per = ms / reps;
      if (ms * 1e-3 >= std::max(seconds, 5e-4) || reps >= 64) break;
      reps *= 2;
    }
    free_tables(tb.classes[0]);
    times.push_back(per);
  }
  free_batch_device(&tb);
  cudaFree(tb.d_head);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(buf);
  if (st != CFFT_OK) return st;
  const double fastest = *std::min_element(times.begin(), times.end());
  size_t pick = 0;
  double pick_ops = 1e30;
  for (size_t i = 0; i < cands.size(); ++i) {
    if (times[i] > 1.03 * fastest) continue;
    const double ops = fp64_ops_per_point(log2n, std::get<1>(cands[i]), std::get<0>(cands[i]));
    if (ops < pick_ops - 1e-9 || (ops < pick_ops + 1e-9 && times[i] < times[pick])) {
      pick = i;
      pick_ops = ops;
    }
  }
  std::tie(c.algo, c.base_log2, c.tpc) = cands[pick];
  return CFFT_OK;
}

void destroy_batch(cfft_batch* b) {
  if (!b) return;
  if (b->g_exec) cudaGraphExecDestroy(b->g_exec);
  for (auto& c : b->chunks) {
    if (c.d_offs) cudaFree(c.d_offs);
    if (c.d_units) cudaFree(c.d_units);
  }
  if (b->d_heads) cudaFree(b->d_heads);
  for (cudaStream_t st : b->pstream)
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t ev : b->pevent)
    if (ev) cudaEventDestroy(ev);
  for (auto& c : b->classes) free_tables(c);
  free_batch_device(b);
  if (b->d_head) cudaFree(b->d_head);
  delete b;
}

// Splits the items, in offset order, into about kChunks groups of equal
// points; each group gets the units of its items (same classes and
// schedules as the whole batch, longest first) and its own work counter.
constexpr int kChunks = 16;
cfft_status build_chunks(cfft_batch* b) {
  std::map<ClassKey, int> cls;
  for (size_t ci = 0; ci < b->classes.size(); ++ci) cls[b->classes[ci].key] = (int)ci;
  std::vector<size_t> order(b->items.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t x, size_t y) { return b->items[x].offset < b->items[y].offset; });
  const size_t target = std::max<size_t>(1, b->total_points / kChunks);
  size_t i = 0;
  while (i < order.size()) {
    size_t j = i, pts = 0;
    while (j < order.size() && (pts < target || j == i)) pts += size_t(1) << b->items[order[j++]].log2n;
    cfft_batch::Chunk ch;
    ch.lo = b->items[order[i]].offset;
    ch.hi = b->items[order[j - 1]].offset + (uint64_t(1) << b->items[order[j - 1]].log2n);
    // per class, this chunk's items in offset order
    std::vector<std::vector<uint64_t>> per(b->classes.size());
    for (size_t k = i; k < j; ++k) {
      const cfft_batch_item& it = b->items[order[k]];
      per[cls[ClassKey{(int)it.kind, (int)it.log2n, (int)it.direction}]].push_back(it.offset);
    }
    std::vector<uint64_t> offs;
    std::vector<std::pair<double, Unit>> u;
    for (size_t ci = 0; ci < per.size(); ++ci) {
      if (per[ci].empty()) continue;
      const ClassHost& c = b->classes[ci];
      const int first = (int)offs.size();
      offs.insert(offs.end(), per[ci].begin(), per[ci].end());
      const int tpc = device_class(c).d0 == 0 ? c.tpc : 1;
      for (size_t k = 0; k < per[ci].size(); k += (size_t)tpc) {
        Unit un{(int)ci, first + (int)k, (int)std::min<size_t>(tpc, per[ci].size() - k), c.key.dir};
        u.push_back({unit_cost(c.key.log2n, un.count, un.dir), un});
      }
    }
    std::stable_sort(u.begin(), u.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
    std::vector<Unit> units;
    for (auto& pu : u) units.push_back(pu.second);
    ch.nunits = (int)units.size();
    b->chunks.push_back(ch);
    cfft_status st = upload(offs.data(), offs.size(), &b->chunks.back().d_offs);
    if (st == CFFT_OK) st = upload(units.data(), units.size(), &b->chunks.back().d_units);
    if (st != CFFT_OK) return st;
    i = j;
  }
  CFFT_CUDA_TRY(cudaMalloc(&b->d_heads, b->chunks.size() * sizeof(unsigned int)));
  for (cudaStream_t& st : b->pstream) CFFT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  for (cudaEvent_t& ev : b->pevent) CFFT_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  return CFFT_OK;
}

}  // namespace

extern "C" {

cfft_status cfft_batch_create(const cfft_batch_item* items, size_t count, double tune_seconds, cfft_batch** out) {
  if (!out || (!items && count)) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  std::map<ClassKey, std::vector<uint64_t>> groups;
  size_t total = 0;
  for (size_t i = 0; i < count; ++i) {
    const cfft_batch_item& it = items[i];
    if (it.kind > 1) return fail(CFFT_ERR_INVALID_ARGUMENT, "item kind must be 0 (ordered) or 1 (unordered)");
    if (it.direction < 1 || it.direction > 3) return fail(CFFT_ERR_INVALID_ARGUMENT, "item direction must be 1..3");
    if (it.log2n > 16 || (it.kind == 0 && it.log2n > 10))
      return fail(CFFT_ERR_INVALID_SIZE, "item size out of range (ordered <= 2^10, unordered <= 2^16)");
    if (it.log2n < 1) return fail(CFFT_ERR_INVALID_SIZE, "item size must be at least 2");
    groups[ClassKey{(int)it.kind, (int)it.log2n, (int)it.direction}].push_back(it.offset);
    total += size_t(1) << it.log2n;
  }
  cfft_status st = batch_attr();
  if (st != CFFT_OK) return st;
  auto* b = new cfft_batch();
  b->total_points = total;
  b->items.assign(items, items + count);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, kBatchThreads,
                                                2 * (1 << kBatchSmemLog2) * sizeof(double2));
  b->grid = sm_count() * std::max(per_sm, 1);
  st = cudaMalloc(&b->d_head, sizeof(unsigned int)) == cudaSuccess ? CFFT_OK : CFFT_ERR_OUT_OF_MEMORY;
  for (auto& g : groups) {
    if (st != CFFT_OK) break;
    ClassHost c;
    c.key = g.first;
    c.items = std::move(g.second);
    // default schedule: Dif4 over a base of 1024 (or the whole ordered/small transform)
    c.algo = 2;
    c.base_log2 = c.key.kind == 0 ? c.key.log2n : std::min(c.key.log2n, 10);
    c.tpc = c.key.log2n <= kBatchSmemLog2 ? std::max(1, (1 << kBatchSmemLog2) >> c.key.log2n) : 1;
    c.tpc = std::min(c.tpc, 8);
    b->classes.push_back(std::move(c));
  }
  if (st == CFFT_OK && tune_seconds > 0)
    for (size_t ci = 0; ci < b->classes.size() && st == CFFT_OK; ++ci) st = tune_class(b, ci, tune_seconds);
  for (size_t ci = 0; ci < b->classes.size() && st == CFFT_OK; ++ci) st = build_tables(b->classes[ci]);
  if (st == CFFT_OK) st = finalize(b);
  if (st != CFFT_OK) {
    destroy_batch(b);
    return st;
  }
  *out = b;
  return CFFT_OK;
}

void cfft_batch_destroy(cfft_batch* batch) { destroy_batch(batch); }

size_t cfft_batch_units(const cfft_batch* batch) { return batch ? batch->units.size() : 0; }

cfft_status cfft_batch_schedule(const cfft_batch* batch, uint32_t kind, uint32_t log2n, uint32_t direction,
                                cfft_algo* base_algo, size_t* base_n, uint32_t* per_unit) {
  if (!batch) return fail(CFFT_ERR_INVALID_ARGUMENT, "null batch");
  for (const auto& c : batch->classes)
    if (c.key.kind == (int)kind && c.key.log2n == (int)log2n && c.key.dir == (int)direction) {
      if (base_algo) *base_algo = (cfft_algo)c.algo;
      if (base_n) *base_n = size_t(1) << c.base_log2;
      if (per_unit) *per_unit = (uint32_t)c.tpc;
      return CFFT_OK;
    }
  return fail(CFFT_ERR_INVALID_ARGUMENT, "no such size class in the batch");
}

cfft_status cfft_batch_run(cfft_batch* b, double* data, void* stream) {
  if (!b || !data) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (b->units.empty()) return CFFT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (s == nullptr) return launch_batch(b, (double2*)data, s);  // the legacy stream cannot be captured
  std::lock_guard<std::mutex> lk(b->mu);
  if (!b->g_exec || b->g_stream != s || b->g_data != data) {
    if (b->g_exec) {
      cudaGraphExecDestroy(b->g_exec);
      b->g_exec = nullptr;
    }
    cudaGraph_t graph;
    CFFT_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cfft_status st = launch_batch(b, (double2*)data, s);
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (st != CFFT_OK) return st;
    if (e != cudaSuccess) return fail(CFFT_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->g_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(CFFT_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    b->g_stream = s;
    b->g_data = data;
  }
  CFFT_CUDA_TRY(cudaGraphLaunch(b->g_exec, s));
  return CFFT_OK;
}

cfft_status cfft_batch_run_host(cfft_batch* b, double* host, double* dev, void* stream) {
  if (!b || !host || !dev) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (b->units.empty()) return CFFT_OK;
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->chunks.empty()) {
    cfft_status st = build_chunks(b);
    if (st != CFFT_OK) return st;
  }
  cudaStream_t s = (cudaStream_t)stream;
  CFFT_CUDA_TRY(cudaEventRecord(b->pevent[3], s));
  for (cudaStream_t ps : b->pstream) CFFT_CUDA_TRY(cudaStreamWaitEvent(ps, b->pevent[3], 0));
  const size_t smem = 2 * (1 << kBatchSmemLog2) * sizeof(double2);
  for (size_t k = 0; k < b->chunks.size(); ++k) {
    const cfft_batch::Chunk& c = b->chunks[k];
    cudaStream_t ps = b->pstream[k % 3];
    const size_t bytes = (size_t)(c.hi - c.lo) * sizeof(double2);
    double* hp = host + 2 * c.lo;
    double* dp = dev + 2 * c.lo;
    CFFT_CUDA_TRY(cudaMemcpyAsync(dp, hp, bytes, cudaMemcpyHostToDevice, ps));
    CFFT_CUDA_TRY(cudaMemsetAsync(b->d_heads + k, 0, sizeof(unsigned int), ps));
    batch_kernel<<<b->grid, kBatchThreads, smem, ps>>>((double2*)dev, b->d_classes, c.d_offs, c.d_units, c.nunits,
                                                        b->d_heads + k);
    CFFT_CHECK_LAUNCH();
    CFFT_CUDA_TRY(cudaMemcpyAsync(hp, dp, bytes, cudaMemcpyDeviceToHost, ps));
  }
  for (int i = 0; i < 3; ++i) {
    CFFT_CUDA_TRY(cudaEventRecord(b->pevent[i], b->pstream[i]));
    CFFT_CUDA_TRY(cudaStreamWaitEvent(s, b->pevent[i], 0));
  }
  return CFFT_OK;
}

}  // extern "C"
