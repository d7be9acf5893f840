// product_engine.cu -- negacyclic u64 products of mixed sizes in one launch.
//
// The serving path: requests carry products of different N (1024..16384 in the
// serving workload), each against its own device-resident Fourier operand.
// An engine holds one product plan per N.  A run is one persistent kernel over
// a device array of items: every CTA takes the next item from a counter and
// runs the whole product pipeline for it (fold, twist, unordered forward,
// pointwise, inverse, untwist, round).  Products with N/2 <= 2048 stay in
// shared memory; larger ones keep their complex data in a per-CTA slice of a
// caller-provided workspace, run their top unordered levels there, and stream
// the <= 2048-point sub-transforms through shared memory, where the pointwise
// product and the sub-transform inverse happen in the same residency.
// Results are bit-identical to cfft_u64_product / the unfused pipeline.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cfft.h"
#include "cfft_internal.h"
#include "runtime.h"
#include "stockham.cuh"

using namespace cfft;

namespace cfft {

constexpr int kEngSmemLog2 = 11;  // 2 x 2048 points x 16 B = 64 KiB per CTA
constexpr int kEngThreads = 256;
constexpr int kEngMaxLog2N = 17;

struct EngClass {
  DevLevels L;
  const double2* w;
  const double2* winv;
  const double2* tw;
  const double2* itw;
  int algo;   // 2 (Dif4) or 4 (Dif8)
  int d0;     // first level in shared memory
  int log2n;  // log2(N/2); 0 when the size is not configured
};

template <int ALGO>
__device__ void engine_product(const EngClass& C, const cfft_product_item& it, double2* x, double2* y,
                               double2* __restrict__ ws, int tid, int nth) {
  const int log2n = C.log2n, n = 1 << log2n;
  const uint64_t* a = it.a;
  const double2* bh = (const double2*)it.bhat;
  uint64_t* out = it.out;
  if (C.d0 == 0) {
    for (int j = tid; j < n; j += nth) {
      const c64 v{i64_to_f64_rne((int64_t)__ldcs(a + j)), i64_to_f64_rne((int64_t)__ldcs(a + j + n))};
      st(x + j, cmul(ldg(C.tw + j), v));
    }
    __syncthreads();
    double2* r = unordered_smem<true, 0, ALGO>(C.L, 0, 1, x, y, C.w, tid, nth);
    for (int k = tid; k < n; k += nth) st(r + k, cmul(ldg(bh + k), ld(r + k)));
    __syncthreads();
    double2* s = unordered_smem<false, 0, ALGO>(C.L, 0, 1, r, r == x ? y : x, C.winv, tid, nth);
    for (int j = tid; j < n; j += nth) {
      const c64 t = cmul(ldg(C.itw + j), ld(s + j));
      __stcs(out + j, round_half_up_mod64(t.re));
      __stcs(out + j + n, round_half_up_mod64(t.im));
    }
    __syncthreads();
    return;
  }
  for (int j = tid; j < n; j += nth) {
    const c64 v{i64_to_f64_rne((int64_t)__ldcs(a + j)), i64_to_f64_rne((int64_t)__ldcs(a + j + n))};
    st(ws + j, cmul(ldg(C.tw + j), v));
  }
  __syncthreads();
  for (int l = 0; l < C.d0; ++l) {
    outer_level<true, 0>(C.L.log2r[l], C.L.log2n[l], 1 << (log2n - C.L.log2n[l]), ws, C.w + C.L.w_off[l], tid, nth);
    __syncthreads();
  }
  const int log2sub = C.L.log2n[C.d0], m = 1 << log2sub;
  for (int c = 0; c < (1 << (log2n - log2sub)); ++c) {
    double2* gc = ws + ((long)c << log2sub);
    for (int i = tid; i < m; i += nth) x[i] = gc[i];
    __syncthreads();
    double2* r = unordered_smem<true, 0, ALGO>(C.L, C.d0, 1, x, y, C.w, tid, nth);
    const double2* bc = bh + ((long)c << log2sub);
    for (int k = tid; k < m; k += nth) st(r + k, cmul(ldg(bc + k), ld(r + k)));
    __syncthreads();
    double2* s = unordered_smem<false, 0, ALGO>(C.L, C.d0, 1, r, r == x ? y : x, C.winv, tid, nth);
    for (int i = tid; i < m; i += nth) gc[i] = s[i];
    __syncthreads();
  }
  for (int l = C.d0 - 1; l >= 0; --l) {
    outer_level<false, 0>(C.L.log2r[l], C.L.log2n[l], 1 << (log2n - C.L.log2n[l]), ws, C.winv + C.L.winv_off[l], tid,
                          nth);
    __syncthreads();
  }
  for (int j = tid; j < n; j += nth) {
    const c64 t = cmul(ldg(C.itw + j), ld(ws + j));
    __stcs(out + j, round_half_up_mod64(t.re));
    __stcs(out + j + n, round_half_up_mod64(t.im));
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kEngThreads, 2) product_engine_kernel(const EngClass* __restrict__ classes,
                                                                       const cfft_product_item* __restrict__ items,
                                                                       int count, unsigned int* __restrict__ head,
                                                                       double2* __restrict__ workspace,
                                                                       long ws_points) {
  extern __shared__ double2 smem[];
  __shared__ int s_item;
  double2* x = smem;
  double2* y = smem + (1 << kEngSmemLog2);
  double2* ws = workspace ? workspace + (long)blockIdx.x * ws_points : nullptr;
  const int tid = threadIdx.x, nth = blockDim.x;
  for (;;) {
    if (tid == 0) s_item = (int)atomicAdd(head, 1u);
    __syncthreads();
    const int i = s_item;
    __syncthreads();
    if (i >= count) break;
    const cfft_product_item it = items[i];
    const EngClass C = classes[it.log2N];
    if (C.algo == 2) engine_product<2>(C, it, x, y, ws, tid, nth);
    else engine_product<4>(C, it, x, y, ws, tid, nth);
  }
}

}  // namespace cfft

struct cfft_product_engine {
  cfft_u64_product_plan* plans[kEngMaxLog2N + 1] = {};
  EngClass* d_classes = nullptr;
  int grid = 0;
  int max_log2n = 0;  // largest configured N/2
  int ws_log2n = 0;   // largest N/2 that needs the workspace (0: none)
};

extern "C" {

cfft_status cfft_product_engine_create(const uint32_t* log2N, size_t count, cfft_product_engine** out) {
  if (!out || (!log2N && count)) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  auto* e = new cfft_product_engine();
  std::vector<EngClass> cls(kEngMaxLog2N + 1);
  std::memset(cls.data(), 0, cls.size() * sizeof(EngClass));
  cfft_status st = CFFT_OK;
  for (size_t i = 0; i < count && st == CFFT_OK; ++i) {
    const uint32_t lN = log2N[i];
    if (lN < 6 || lN > (uint32_t)kEngMaxLog2N) {
      st = fail(CFFT_ERR_INVALID_SIZE, "engine sizes must be 2^6..2^17");
      break;
    }
    if (e->plans[lN]) continue;
    const int log2n = (int)lN - 1;
    const int base_log2 = std::min(log2n, 10);
    // FP64 instruction count decides on this part: Dif4 for even base exponents, Dif8 for odd ones
    const int algo = (base_log2 % 2 == 0) ? 2 : 4;
    st = cfft_u64_product_plan_create(size_t(1) << lN, (cfft_algo)algo, size_t(1) << base_log2, &e->plans[lN]);
    if (st != CFFT_OK) break;
    const size_t n = size_t(1) << log2n, base = size_t(1) << base_log2;
    const LevelDesc lv = make_levels(n, base);
    EngClass& c = cls[lN];
    c.L.nlevels = lv.nlevels;
    for (int k = 0; k <= kMaxLevels; ++k) {
      c.L.log2n[k] = lv.log2n[k];
      c.L.w_off[k] = lv.w_off[k];
    }
    for (int k = 0; k < kMaxLevels; ++k) {
      c.L.log2r[k] = lv.log2r[k];
      c.L.winv_off[k] = lv.winv_off[k];
    }
    cfft_algo a;
    size_t bn;
    cfft_u64_product_algo(e->plans[lN], &a, &bn);
    c.algo = (int)a;
    c.log2n = log2n;
    c.d0 = 0;
    while (lv.log2n[c.d0] > kEngSmemLog2) ++c.d0;
    c.w = nullptr;
    e->max_log2n = std::max(e->max_log2n, log2n);
    if (c.d0 > 0) e->ws_log2n = std::max(e->ws_log2n, log2n);
  }
  // device table pointers come from the plans' own tables
  if (st == CFFT_OK) {
    for (int lN = 0; lN <= kEngMaxLog2N; ++lN) {
      if (!e->plans[lN]) continue;
      const cfft_u64_product_plan* p = e->plans[lN];
      const void *w, *wi, *tw, *itw;
      u64_product_tables(p, &w, &wi, &tw, &itw);
      cls[lN].w = (const double2*)w;
      cls[lN].winv = (const double2*)wi;
      cls[lN].tw = (const double2*)tw;
      cls[lN].itw = (const double2*)itw;
    }
    st = upload(cls.data(), cls.size(), &e->d_classes);
  }
  if (st == CFFT_OK) {
    const size_t smem = 2 * (1 << kEngSmemLog2) * sizeof(double2);
    e->grid = sm_count() * max_blocks_per_sm((const void*)product_engine_kernel, kEngThreads, smem);
  }
  if (st != CFFT_OK) {
    cfft_product_engine_destroy(e);
    return st;
  }
  *out = e;
  return CFFT_OK;
}

void cfft_product_engine_destroy(cfft_product_engine* e) {
  if (!e) return;
  for (auto* p : e->plans)
    if (p) cfft_u64_product_plan_destroy(p);
  if (e->d_classes) cudaFree(e->d_classes);
  delete e;
}

size_t cfft_product_engine_workspace_bytes(const cfft_product_engine* e) {
  if (!e || e->ws_log2n == 0) return 0;
  return (size_t)e->grid * (size_t(1) << e->ws_log2n) * sizeof(double2);
}

const cfft_u64_product_plan* cfft_product_engine_plan(const cfft_product_engine* e, uint32_t log2N) {
  if (!e || log2N > (uint32_t)kEngMaxLog2N) return nullptr;
  return e->plans[log2N];
}

cfft_status cfft_product_engine_run(const cfft_product_engine* e, const cfft_product_item* items, size_t count,
                                    unsigned int* counter, double* workspace, void* stream) {
  if (!e || !items || !counter) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (count == 0) return CFFT_OK;
  if (count > 0x7fffffff) return fail(CFFT_ERR_INVALID_SIZE, "too many items");
  if (e->ws_log2n && !workspace)
    return fail(CFFT_ERR_INVALID_ARGUMENT, "this engine's sizes need a workspace (cfft_product_engine_workspace_bytes)");
  cudaStream_t s = (cudaStream_t)stream;
  CFFT_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s));
  const size_t smem = 2 * (1 << kEngSmemLog2) * sizeof(double2);
  const int grid = (int)std::min<size_t>((size_t)e->grid, count);
  long ws_points = e->ws_log2n ? (1L << e->ws_log2n) : 0;
  double2* ws = (double2*)workspace;
  int cnt = (int)count;
  const EngClass* cls = e->d_classes;
  void* args[] = {(void*)&cls, (void*)&items, &cnt, &counter, &ws, &ws_points};
  return launch_kernel((const void*)product_engine_kernel, grid, kEngThreads, args, smem, s);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Product-engine run without allocation.
//
// For callers that must not allocate device memory on their call path: code
// running inside a host framework that has reserved the whole device memory
// budget for its own allocator (a cudaMalloc there fails or fragments that
// pool), and latency-critical loops, where cudaMalloc/cudaFree would
// synchronise the device.  This entry point takes the queue counter and the
// large-N workspace from the static device array below instead of caller
// buffers, and calls no allocating routine.
//
// Limits and sharing: the array holds 256 bytes of counter and 24 MiB of
// workspace, and every GPU that loads this library keeps it until the process
// exits.  Under CUDA's lazy module loading the 24 MiB is committed when this
// file's kernels are first loaded on a device, which happens at
// cfft_product_engine_create.  Engines with a size above N = 16384 (128 KiB of
// workspace per CTA) are rejected with CFFT_ERR_INVALID_SIZE, on every device.
// The launch is capped at 24 MiB / per-CTA workspace CTAs (192 at N = 16384,
// 384 at N = 8192); that cap holds for the whole launch, including the items
// of an engine's smaller sizes, which then run on fewer CTAs than
// cfft_product_engine_run would give them.  All calls share the array: calls
// whose executions overlap on the GPU (different streams, or several threads)
// race on it and must be serialised by the caller.  The counter is cleared by
// every call; the workspace needs no clearing (each product writes before it
// reads).  The looked-up device address is kept per device ordinal for the
// life of the process; it does not survive cudaDeviceReset.
constexpr int kStaticMaxLog2N = 14;
constexpr size_t kStaticCounterBytes = 256;
constexpr size_t kStaticWorkspaceBytes = size_t(24) << 20;
static __device__ __align__(256) unsigned char g_engine_scratch[kStaticCounterBytes + kStaticWorkspaceBytes];

namespace {
std::mutex g_static_mu;
void* g_static_ptr[64] = {};  // address of g_engine_scratch on each device

// Set-up, once per device, with that device current: the host-side symbol is
// only a stand-in, so the device address comes from cudaGetSymbolAddress.
// The first call on a device does this; make that first call before any
// stream capture on the device.
cfft_status static_scratch(void** out) {
  int dev = 0;
  CFFT_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(CFFT_ERR_NO_DEVICE, "device ordinal out of range for the static scratch");
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_engine_scratch);
    if (e != cudaSuccess || p == nullptr)
      return fail(CFFT_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return CFFT_OK;
}
}  // namespace

extern "C" cfft_status cfft_product_engine_run_static(const cfft_product_engine* e, const cfft_product_item* items,
                                                      size_t count, void* stream) {
  if (!e || !items) return fail(CFFT_ERR_INVALID_ARGUMENT, "null argument");
  if (count == 0) return CFFT_OK;
  if (count > 0x7fffffff) return fail(CFFT_ERR_INVALID_SIZE, "too many items");
  int grid = (int)std::min<size_t>((size_t)e->grid, count);
  long ws_points = 0;
  if (e->ws_log2n) {
    if (e->ws_log2n + 1 > kStaticMaxLog2N)
      return fail(CFFT_ERR_INVALID_SIZE,
                  "cfft_product_engine_run_static: N = 2^" + std::to_string(e->ws_log2n + 1) +
                      " is above the largest size (N = 16384) whose workspace the 24 MiB static scratch holds; "
                      "use cfft_product_engine_run with a caller workspace");
    ws_points = 1L << e->ws_log2n;
    const size_t per_cta = (size_t)ws_points * sizeof(double2);
    const size_t fit = kStaticWorkspaceBytes / per_cta;  // >= 192 for N <= 16384
    grid = (int)std::min<size_t>((size_t)grid, fit);
  }
  void* base = nullptr;
  cfft_status st = static_scratch(&base);
  if (st != CFFT_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int* counter = (unsigned int*)base;
  double2* ws = e->ws_log2n ? (double2*)((unsigned char*)base + kStaticCounterBytes) : nullptr;
  CFFT_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s));
  const size_t smem = 2 * (1 << kEngSmemLog2) * sizeof(double2);
  int cnt = (int)count;
  const EngClass* cls = e->d_classes;
  void* args[] = {(void*)&cls, (void*)&items, &cnt, &counter, &ws, &ws_points};
  return launch_kernel((const void*)product_engine_kernel, grid, kEngThreads, args, smem, s);
}
