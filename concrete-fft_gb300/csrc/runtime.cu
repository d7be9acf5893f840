// runtime.cu -- library-wide state: errors, device checks, staging buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "cfft_internal.h"
#include "runtime.h"

namespace cfft {
std::string get_error();

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 152;
  if (cached[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = v > 0 ? v : 1;
  }
  return cached[dev];
}

namespace {
struct Staging {
  void* ptr = nullptr;
  size_t cap = 0;
  cudaStream_t stream = nullptr;
  int device = -1;
  ~Staging() {
    // Buffers are released at thread exit only when the context is still alive.
    if (ptr) cudaFree(ptr);
    if (stream) cudaStreamDestroy(stream);
  }
};
thread_local Staging t_staging;
}  // namespace

// Device buffer + private stream reused by the *_host entry points of the
// calling thread (grown on demand, never shrunk).
cfft_status host_staging(size_t bytes, void** dev_ptr, cudaStream_t* stream) {
  int dev = 0;
  CFFT_CUDA_TRY(cudaGetDevice(&dev));
  Staging& s = t_staging;
  if (s.device != dev) {
    s.ptr = nullptr;
    s.cap = 0;
    s.stream = nullptr;
    s.device = dev;
  }
  if (!s.stream) CFFT_CUDA_TRY(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
  if (bytes > s.cap) {
    if (s.ptr) {
      CFFT_CUDA_TRY(cudaStreamSynchronize(s.stream));
      CFFT_CUDA_TRY(cudaFree(s.ptr));
      s.ptr = nullptr;
      s.cap = 0;
    }
    CFFT_CUDA_TRY(cudaMalloc(&s.ptr, bytes));
    s.cap = bytes;
  }
  *dev_ptr = s.ptr;
  *stream = s.stream;
  return CFFT_OK;
}

namespace {
struct Bounce {
  void* host = nullptr;
  size_t cap = 0;
  ~Bounce() {
    if (host) cudaFreeHost(host);
  }
};
thread_local Bounce t_bounce;
}  // namespace

// Page-locked, device-mapped host buffer of the calling thread for the *_host
// entry points on pageable memory (grown on demand up to kHostBounceMax, never
// shrunk).  A pageable cudaMemcpy costs ~10 us of fixed driver time each way;
// a CPU memcpy into this buffer costs about a microsecond for a small transform.
cfft_status host_bounce(size_t bytes, void** host_ptr, void** dev_ptr) {
  if (bytes > kHostBounceMax) return fail(CFFT_ERR_INVALID_SIZE, "host bounce buffer request too large");
  Bounce& b = t_bounce;
  if (bytes > b.cap) {
    if (b.host) CFFT_CUDA_TRY(cudaFreeHost(b.host));
    b.host = nullptr;
    b.cap = 0;
    const size_t cap = std::max<size_t>(bytes, 64 << 10);
    CFFT_CUDA_TRY(cudaHostAlloc(&b.host, cap, cudaHostAllocMapped | cudaHostAllocPortable));
    b.cap = cap;
  }
  CFFT_CUDA_TRY(cudaHostGetDevicePointer(dev_ptr, b.host, 0));
  *host_ptr = b.host;
  return CFFT_OK;
}

namespace {
std::mutex g_attr_mu;
struct AttrEntry {
  const void* fn;
  int dev;
  size_t smem;
};
std::vector<AttrEntry> g_attrs;
cfft_status ensure_smem_attr(const void* fn, size_t smem) {
  if (smem <= 48 * 1024) return CFFT_OK;
  int dev = 0;
  CFFT_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_attr_mu);
  for (const auto& e : g_attrs)
    if (e.fn == fn && e.dev == dev && e.smem >= smem) return CFFT_OK;
  CFFT_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  g_attrs.push_back({fn, dev, smem});
  return CFFT_OK;
}
}  // namespace

cfft_status launch_kernel(const void* fn, int grid, int block, void** args, size_t smem, cudaStream_t stream,
                          bool pdl) {
  if (!fn) return fail(CFFT_ERR_INVALID_ARGUMENT, "no kernel instantiated for this configuration");
  cfft_status st = ensure_smem_attr(fn, smem);
  if (st != CFFT_OK) return st;
  if (!pdl) {
    CFFT_CUDA_TRY(cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, stream));
    return CFFT_OK;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CFFT_CUDA_TRY(cudaLaunchKernelExC(&cfg, fn, args));
  return CFFT_OK;
}

// Cluster scheduling policy of every cluster launch (cfft_diag_set_cluster_policy):
// load balancing by default (N = 16384 products on 8-CTA clusters: 661 vs 649 k/s
// with the driver's default; the split transforms are unchanged).
static std::atomic<int> g_cluster_policy{(int)cudaClusterSchedulingPolicyLoadBalancing};

int cluster_count_query(const void* fn, int block, int cluster, size_t smem);

cfft_status allow_cluster16(const void* fn) {
  static std::mutex mu;
  static std::vector<std::pair<const void*, int>> done;
  int dev = 0;
  CFFT_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  for (const auto& e : done)
    if (e.first == fn && e.second == dev) return CFFT_OK;
  CFFT_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  done.emplace_back(fn, dev);
  return CFFT_OK;
}

int cluster_count(const void* fn, int block, int cluster, size_t smem) {
  // answers are kept per device, kernel and shape: the query costs microseconds and
  // the launchers ask before every small-batch launch
  struct Key {
    const void* fn;
    int dev, block, cluster;
    size_t smem;
  };
  static std::mutex mu;
  static std::vector<std::pair<Key, int>> known;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    for (const auto& e : known)
      if (e.first.fn == fn && e.first.dev == dev && e.first.block == block && e.first.cluster == cluster &&
          e.first.smem == smem)
        return e.second;
  }
  const int count = cluster_count_query(fn, block, cluster, smem);
  std::lock_guard<std::mutex> lk(mu);
  known.push_back({Key{fn, dev, block, cluster, smem}, count});
  return count;
}

bool cluster_fits(const void* fn, int block, int cluster, size_t smem) {
  return cluster_count(fn, block, cluster, smem) >= 1;
}

int spread_clusters(const void* fn, int block, int cluster) {
  // the padded size per device and kernel (the attribute queries are driver calls)
  static std::mutex mu;
  static std::vector<std::pair<std::pair<const void*, int>, size_t>> padded;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  size_t smem = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    for (const auto& e : padded)
      if (e.first.first == fn && e.first.second == dev) smem = e.second;
  }
  if (smem == 0) {
    int max_block = 0;
    cudaFuncAttributes fa{};
    if (cudaDeviceGetAttribute(&max_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, fn) != cudaSuccess || (size_t)max_block <= fa.sharedSizeBytes) {
      cudaGetLastError();
      return 0;
    }
    smem = (size_t)max_block - fa.sharedSizeBytes;
    std::lock_guard<std::mutex> lk(mu);
    padded.push_back({{fn, dev}, smem});
  }
  return cluster_count(fn, block, cluster, smem);
}

int cluster_count_query(const void* fn, int block, int cluster, size_t smem) {
  if (ensure_smem_attr(fn, smem) != CFFT_OK) return 0;
  if (cluster > 8 && allow_cluster16(fn) != CFFT_OK) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cluster);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return clusters;
}

cfft_status launch_kernel_cluster(const void* fn, int grid, int block, int cluster, void** args, size_t smem,
                                  cudaStream_t stream, bool pdl) {
  if (!fn) return fail(CFFT_ERR_INVALID_ARGUMENT, "no kernel instantiated for this configuration");
  if (cluster < 1 || cluster > 16 || grid % cluster != 0) return fail(CFFT_ERR_INVALID_ARGUMENT, "bad cluster shape");
  if (cluster > 8) {
    cfft_status a = allow_cluster16(fn);
    if (a != CFFT_OK) return a;
  }
  cfft_status st = ensure_smem_attr(fn, smem);
  if (st != CFFT_OK) return st;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[3];
  unsigned na = 0;
  attr[na].id = cudaLaunchAttributeClusterDimension;
  attr[na].val.clusterDim.x = (unsigned)cluster;
  attr[na].val.clusterDim.y = 1;
  attr[na].val.clusterDim.z = 1;
  ++na;
  if (pdl) {
    attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[na].val.programmaticStreamSerializationAllowed = 1;
    ++na;
  }
  const int policy = g_cluster_policy.load(std::memory_order_relaxed);
  if (policy) {
    attr[na].id = cudaLaunchAttributeClusterSchedulingPolicyPreference;
    attr[na].val.clusterSchedulingPolicyPreference = (cudaClusterSchedulingPolicy)policy;
    ++na;
  }
  cfg.attrs = attr;
  cfg.numAttrs = na;
  CFFT_CUDA_TRY(cudaLaunchKernelExC(&cfg, fn, args));
  return CFFT_OK;
}

cfft_status ensure_smem(const void* fn, size_t smem) { return ensure_smem_attr(fn, smem); }

int max_blocks_per_sm(const void* fn, int block, size_t smem) {
  if (ensure_smem_attr(fn, smem) != CFFT_OK) return 1;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, smem);
  return per_sm > 0 ? per_sm : 1;
}

// Even spreading of a grid that fits in one wave.  The block scheduler fills
// an SM up to its occupancy before the next, so a grid of 1024 CTAs that fits
// 28 to an SM ran with some SMs holding 8 CTAs and others none (ordered n =
// 1024, batch 256 on 4-CTA clusters: SM active cycles min 0, max 1.07 x the
// mean).  Padding the dynamic shared memory so that ceil(grid / SMs) CTAs fit
// an SM, and no more, makes the scheduler use every SM; the kernel's time is
// then that of the busiest SM at the even share.  Only when the padded shape
// still holds the whole grid at once (with clusters: cudaOccupancyMaxActiveClusters).
static std::atomic<int> g_spread{1};

namespace {
struct SpreadKey {
  const void* fn;
  int grid, block, cluster, dev;
  size_t smem;
  bool operator==(const SpreadKey& o) const {
    return fn == o.fn && grid == o.grid && block == o.block && cluster == o.cluster && dev == o.dev &&
           smem == o.smem;
  }
};
struct SpreadKeyHash {
  size_t operator()(const SpreadKey& k) const {
    size_t h = std::hash<const void*>()(k.fn);
    for (size_t v : {(size_t)k.grid, (size_t)k.block, (size_t)k.cluster, (size_t)k.dev, k.smem})
      h = h * 0x9e3779b97f4a7c15ull + v;
    return h;
  }
};
std::mutex g_spread_mu;
// launch shapes seen so far (one entry per kernel, grid, block, cluster, device and
// shared-memory size); cleared when it reaches 65536 entries
std::unordered_map<SpreadKey, size_t, SpreadKeyHash> g_spread_cache;

size_t compute_spread(const void* fn, int grid, int block, int cluster, size_t smem, int dev) {
  const int nsm = sm_count();
  const int occ = max_blocks_per_sm(fn, block, smem);
  if (occ <= 1 || (long)grid > (long)occ * nsm) return smem;  // several waves: the scheduler balances them
  const int need = (grid + nsm - 1) / nsm;
  if (need >= occ) return smem;
  int per_sm = 0, reserved = 0, max_block = 0;
  cudaFuncAttributes fa{};
  if (cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&max_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, fn) != cudaSuccess)
    return smem;
  const long per_block = (long)per_sm / need - reserved - (long)fa.sharedSizeBytes;
  if (per_block <= (long)smem) return smem;
  size_t padded = std::min<size_t>((size_t)per_block & ~(size_t)127, (size_t)max_block - fa.sharedSizeBytes);
  if (padded <= smem || max_blocks_per_sm(fn, block, padded) != need) return smem;
  if (cluster > 1) {  // every cluster of the grid must still be resident at once
    if (cluster > 8 && allow_cluster16(fn) != CFFT_OK) return smem;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = padded;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess || (long)clusters * cluster < grid) {
      cudaGetLastError();
      return smem;
    }
  }
  return padded;
}
}  // namespace

size_t spread_smem(const void* fn, int grid, int block, int cluster, size_t smem) {
  if (!fn || !g_spread.load(std::memory_order_relaxed) || grid <= 0) return smem;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return smem;
  const SpreadKey key{fn, grid, block, cluster, dev, smem};
  {
    std::lock_guard<std::mutex> lk(g_spread_mu);
    const auto it = g_spread_cache.find(key);
    if (it != g_spread_cache.end()) return it->second;
  }
  const size_t v = compute_spread(fn, grid, block, cluster, smem, dev);
  std::lock_guard<std::mutex> lk(g_spread_mu);
  if (g_spread_cache.size() >= 65536) g_spread_cache.clear();
  g_spread_cache.emplace(key, v);
  return v;
}

namespace {
constexpr int kMaxSlots = 8;
struct Pipeline {
  void* ptr[kMaxSlots] = {};
  size_t cap = 0;
  cudaStream_t stream[kMaxSlots] = {};
  int device = -1;
};
thread_local Pipeline t_pipe;
}  // namespace

cfft_status host_pipeline(int nslots, size_t bytes, PipeSlot* slots) {
  if (nslots < 1 || nslots > kMaxSlots) return fail(CFFT_ERR_INVALID_ARGUMENT, "bad pipeline depth");
  int dev = 0;
  CFFT_CUDA_TRY(cudaGetDevice(&dev));
  Pipeline& p = t_pipe;
  if (p.device != dev) {
    p = Pipeline();
    p.device = dev;
  }
  for (int i = 0; i < kMaxSlots; ++i)
    if (!p.stream[i]) CFFT_CUDA_TRY(cudaStreamCreateWithFlags(&p.stream[i], cudaStreamNonBlocking));
  if (bytes > p.cap) {
    for (int i = 0; i < kMaxSlots; ++i) {
      CFFT_CUDA_TRY(cudaStreamSynchronize(p.stream[i]));
      if (p.ptr[i]) CFFT_CUDA_TRY(cudaFree(p.ptr[i]));
      p.ptr[i] = nullptr;
    }
    p.cap = 0;
    for (int i = 0; i < kMaxSlots; ++i) CFFT_CUDA_TRY(cudaMalloc(&p.ptr[i], bytes));
    p.cap = bytes;
  }
  for (int i = 0; i < nslots; ++i) slots[i] = PipeSlot{p.ptr[i], p.stream[i]};
  return CFFT_OK;
}

namespace {
std::atomic<int> g_hc_chunks{24}, g_hc_slots{4}, g_hc_first{0}, g_hc_last{0};
}

HostChunks host_chunks() {
  return HostChunks{g_hc_chunks.load(std::memory_order_relaxed), g_hc_slots.load(std::memory_order_relaxed),
                    g_hc_first.load(std::memory_order_relaxed), g_hc_last.load(std::memory_order_relaxed)};
}

void bind_device_context() {
  // a thread's first runtime call does not always make the device's primary
  // context current, and pointer queries then miss page-locked host memory;
  // cudaSetDevice makes it current (a no-op once it is)
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaSetDevice(dev);
}

void* mapped_host_range(const void* p, size_t bytes) {
  if (!p || bytes == 0) return nullptr;
  bind_device_context();
  cudaPointerAttributes first{}, last{};
  const char* end = (const char*)p + bytes - 1;
  if (cudaPointerGetAttributes(&first, p) != cudaSuccess || cudaPointerGetAttributes(&last, end) != cudaSuccess) {
    cudaGetLastError();  // pageable memory on older drivers reports an error: clear it
    return nullptr;
  }
  if (first.type != cudaMemoryTypeHost || last.type != cudaMemoryTypeHost) return nullptr;
  if (!first.devicePointer || !last.devicePointer) return nullptr;
  if ((const char*)last.devicePointer - (const char*)first.devicePointer != (long)(bytes - 1)) return nullptr;
  return first.devicePointer;
}

}  // namespace cfft

extern "C" {

const char* cfft_last_error(void) {
  thread_local std::string copy;
  copy = cfft::get_error();
  return copy.c_str();
}

const char* cfft_version(void) { return "concrete-fft-gb300 0.1.0 (sm_103a, FP64 bit-exact)"; }

cfft_status cfft_device_check(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return cfft::fail(CFFT_ERR_NO_DEVICE, "no CUDA device");
  }
  int dev = 0, major = 0, minor = 0;
  CFFT_CUDA_TRY(cudaGetDevice(&dev));
  CFFT_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  CFFT_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  if (major != 10 || minor != 3)
    return cfft::fail(CFFT_ERR_NO_DEVICE, "this build targets sm_103a (GB300); found compute capability " +
                                              std::to_string(major) + "." + std::to_string(minor));
  return CFFT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- diagnostics
#include "../../include/cfft_diag.h"

namespace {
constexpr int kPeakIters = 2048;
// OP 0: DFMA chains, 1: DADD, 2: DMUL, 3: the product kernel's mix.  Eight
// independent chains per thread, 64 warps per SM; every chain stays near 1.
template <int OP>
__global__ void fp64_peak_kernel(double* out, double seed) {
  double a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed + 1e-3 * (threadIdx.x & 7) + 1e-4 * i;
  for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (OP == 0) a[i] = __fma_rn(a[i], 0.999999, 1e-6);
      if (OP == 1) a[i] = __dadd_rn(a[i], (it & 1) ? 1e-9 : -1e-9);
      if (OP == 2) a[i] = __dmul_rn(a[i], (it & 1) ? 1.000001 : 0.999999);
      if (OP == 3) {  // 2 DADD : 1 DFMA : 1 DMUL, the product kernel's 40960 : 18432 : 18432
        if (i < 4) a[i] = __dadd_rn(a[i], (it & 1) ? 1e-9 : -1e-9);
        else if (i < 6) a[i] = __fma_rn(a[i], 0.999999, 1e-6);
        else a[i] = __dmul_rn(a[i], (it & 1) ? 1.000001 : 0.999999);
      }
    }
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cfft_status time_fp64(const void* fn, double* ops_per_second) {
  const int blocks = cfft::sm_count() * 8, threads = 256;  // 64 warps per SM
  double* d = nullptr;
  CFFT_CUDA_TRY(cudaMalloc(&d, (size_t)blocks * threads * sizeof(double)));
  cudaEvent_t e0, e1;
  CFFT_CUDA_TRY(cudaEventCreate(&e0));
  CFFT_CUDA_TRY(cudaEventCreate(&e1));
  double seed = 1.0;
  void* args[] = {&d, &seed};
  CFFT_CUDA_TRY(cudaLaunchKernel(fn, dim3(blocks), dim3(threads), args, 0, 0));
  CFFT_CUDA_TRY(cudaEventRecord(e0));
  const int reps = 5;
  for (int r = 0; r < reps; ++r) CFFT_CUDA_TRY(cudaLaunchKernel(fn, dim3(blocks), dim3(threads), args, 0, 0));
  CFFT_CUDA_TRY(cudaEventRecord(e1));
  CFFT_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  CFFT_CHECK_LAUNCH();
  *ops_per_second = (double)reps * blocks * threads * kPeakIters * 8 / (ms * 1e-3);
  return CFFT_OK;
}
}  // namespace

extern "C" cfft_status cfft_diag_fp64_rates(double* rates4) {
  if (!rates4) return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  const void* fns[4] = {(const void*)fp64_peak_kernel<0>, (const void*)fp64_peak_kernel<1>,
                        (const void*)fp64_peak_kernel<2>, (const void*)fp64_peak_kernel<3>};
  for (int k = 0; k < 4; ++k) {
    cfft_status st = time_fp64(fns[k], rates4 + k);
    if (st != CFFT_OK) return st;
  }
  return CFFT_OK;
}

extern "C" cfft_status cfft_diag_fp64_peak(double* ops_per_second) {
  if (!ops_per_second) return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  double r[4];
  cfft_status st = cfft_diag_fp64_rates(r);
  if (st != CFFT_OK) return st;
  *ops_per_second = std::max(std::max(r[0], r[1]), std::max(r[2], r[3]));
  return CFFT_OK;
}

#include "int_fp64.cuh"

namespace {
__device__ __forceinline__ uint64_t mix64(uint64_t z) {  // splitmix64 finaliser
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ void make_pair(uint64_t i, uint64_t seed, double& x, double& y) {
  const uint64_t r0 = mix64(seed ^ (i * 4 + 0)), r1 = mix64(seed ^ (i * 4 + 1)), r2 = mix64(seed ^ (i * 4 + 2));
  const int mode = (int)(i & 3);
  uint64_t bx, by;
  if (mode == 0) {  // raw bit patterns: every exponent, zeros, subnormals, inf, nan
    bx = r0;
    by = r1;
  } else if (mode == 1) {  // normal operands with exponent gaps 0..70
    const uint64_t ex = 200 + (r2 & 1023);
    const uint64_t gap = (r2 >> 10) % 71;
    bx = (r0 & 0x800fffffffffffffull) | (ex << 52);
    by = (r1 & 0x800fffffffffffffull) | ((ex - gap) << 52);
  } else if (mode == 2) {  // near cancellation: y ~ -x with low bits perturbed
    const uint64_t ex = 100 + (r2 & 1023);
    bx = (r0 & 0x000fffffffffffffull) | (ex << 52);
    const int k = (int)((r2 >> 12) % 54);
    by = (bx ^ (r1 & ((1ull << k) - 1))) | 0x8000000000000000ull;
    if ((r2 >> 20) & 1) by += ((r2 >> 21) & 3) << 52;  // also exponent off by 0..3
    if ((r2 >> 23) & 1) bx ^= 0x8000000000000000ull, by ^= 0x8000000000000000ull;
  } else {  // rounding ties and near ties: y's bits straddle x's last place
    const uint64_t ex = 300 + (r2 & 511);
    const uint64_t gap = 52 + ((r2 >> 9) % 4);
    bx = (r0 & 0x800fffffffffffffull) | (ex << 52);
    uint64_t my = (r2 >> 16) & 0x7;  // few significant bits: exact halves are common
    by = (r1 & 0x8000000000000000ull) | ((ex - gap) << 52) | (my << 49);
  }
  x = __longlong_as_double((long long)bx);
  y = __longlong_as_double((long long)by);
}

__global__ void dadd_check_kernel(uint64_t count, uint64_t seed, unsigned long long* bad, unsigned long long* first) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
    double x, y;
    make_pair(i, seed, x, y);
    const double a = cfft::dadd_int(x, y);
    const double b = __dadd_rn(x, y);
    const bool nan_both = (a != a) && (b != b);
    if (!nan_both && __double_as_longlong(a) != __double_as_longlong(b)) {
      if (atomicAdd(bad, 1ull) == 0) {
        first[0] = (unsigned long long)__double_as_longlong(x);
        first[1] = (unsigned long long)__double_as_longlong(y);
      }
    }
  }
}

constexpr int kIntIters = 512;
__global__ void dadd_int_rate_kernel(double* out, double seed) {
  double a[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) a[i] = seed + threadIdx.x * 1e-3 + i;
  const double c = 1.0000000001e-3;
  for (int it = 0; it < kIntIters; ++it) {
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = cfft::dadd_int(a[i], c);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = a[0] + a[1] + a[2] + a[3];
}
}  // namespace

extern "C" cfft_status cfft_diag_dadd_check(uint64_t count, uint64_t seed, uint64_t* mismatches, uint64_t* bad_pair) {
  if (!mismatches) return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  unsigned long long* d = nullptr;
  CFFT_CUDA_TRY(cudaMalloc(&d, 3 * sizeof(unsigned long long)));
  CFFT_CUDA_TRY(cudaMemset(d, 0, 3 * sizeof(unsigned long long)));
  dadd_check_kernel<<<cfft::sm_count() * 8, 256>>>(count, seed, d, d + 1);
  CFFT_CHECK_LAUNCH();
  unsigned long long h[3];
  CFFT_CUDA_TRY(cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost));
  cudaFree(d);
  *mismatches = h[0];
  if (bad_pair) {
    bad_pair[0] = h[1];
    bad_pair[1] = h[2];
  }
  return CFFT_OK;
}

extern "C" cfft_status cfft_diag_dadd_int_rate(double* adds_per_second) {
  if (!adds_per_second) return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  const int blocks = cfft::sm_count() * 4, threads = 256;
  double* d = nullptr;
  CFFT_CUDA_TRY(cudaMalloc(&d, (size_t)blocks * threads * sizeof(double)));
  cudaEvent_t e0, e1;
  CFFT_CUDA_TRY(cudaEventCreate(&e0));
  CFFT_CUDA_TRY(cudaEventCreate(&e1));
  dadd_int_rate_kernel<<<blocks, threads>>>(d, 1.0);
  CFFT_CUDA_TRY(cudaEventRecord(e0));
  const int reps = 5;
  for (int r = 0; r < reps; ++r) dadd_int_rate_kernel<<<blocks, threads>>>(d, 1.0);
  CFFT_CUDA_TRY(cudaEventRecord(e1));
  CFFT_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  CFFT_CHECK_LAUNCH();
  *adds_per_second = (double)reps * blocks * threads * kIntIters * 4 / (ms * 1e-3);
  return CFFT_OK;
}

extern "C" cfft_status cfft_diag_host_mapping(const void* p, size_t bytes, void** device_address) {
  if (!device_address) return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  *device_address = cfft::mapped_host_range(p, bytes);
  return CFFT_OK;
}

extern "C" cfft_status cfft_diag_set_host_chunks(int chunks, int slots, int first, int last) {
  if (chunks < 0 || chunks > 1024 || slots < 0 || slots > 8 || first < 0 || last < 0)
    return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "chunks 0..1024, slots 0..8, first and last >= 0");
  cfft::g_hc_chunks.store(chunks ? chunks : 24, std::memory_order_relaxed);
  cfft::g_hc_slots.store(slots ? slots : 4, std::memory_order_relaxed);
  cfft::g_hc_first.store(first, std::memory_order_relaxed);
  cfft::g_hc_last.store(last, std::memory_order_relaxed);
  return CFFT_OK;
}

extern "C" cfft_status cfft_diag_set_spread(int on) {
  if (on != 0 && on != 1) return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "spread must be 0 or 1");
  cfft::g_spread.store(on, std::memory_order_relaxed);
  return CFFT_OK;
}

extern "C" cfft_status cfft_diag_set_cluster_policy(int policy) {
  if (policy < 0 || policy > 2) return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "policy must be 0, 1 or 2");
  cfft::g_cluster_policy.store(policy, std::memory_order_relaxed);
  return CFFT_OK;
}
