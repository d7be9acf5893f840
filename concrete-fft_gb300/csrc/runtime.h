// runtime.h -- host runtime helpers shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "cfft_internal.h"

#define CFFT_CUDA_TRY(expr)                                                                  \
  do {                                                                                       \
    cudaError_t err__ = (expr);                                                              \
    if (err__ != cudaSuccess) {                                                              \
      ::cfft::set_error(std::string(#expr) + ": " + cudaGetErrorString(err__));              \
      return err__ == cudaErrorMemoryAllocation ? CFFT_ERR_OUT_OF_MEMORY : CFFT_ERR_CUDA;    \
    }                                                                                        \
  } while (0)

#define CFFT_CHECK_LAUNCH()                                                                  \
  do {                                                                                       \
    cudaError_t err__ = cudaGetLastError();                                                  \
    if (err__ != cudaSuccess) {                                                              \
      ::cfft::set_error(std::string("kernel launch: ") + cudaGetErrorString(err__));         \
      return CFFT_ERR_CUDA;                                                                  \
    }                                                                                        \
  } while (0)

namespace cfft {

inline cfft_status fail(cfft_status s, const std::string& msg) {
  set_error(msg);
  return s;
}

// Device-resident copy of a host table.
template <class T>
cfft_status upload(const T* host, size_t count, T** dev) {
  *dev = nullptr;
  if (count == 0) return CFFT_OK;
  CFFT_CUDA_TRY(cudaMalloc((void**)dev, count * sizeof(T)));
  CFFT_CUDA_TRY(cudaMemcpy(*dev, host, count * sizeof(T), cudaMemcpyHostToDevice));
  return CFFT_OK;
}

int sm_count();

// Launch a kernel through its pointer, raising its dynamic shared-memory limit
// the first time it is used with more than 48 KiB.  `pdl`: programmatic stream
// serialization (the kernel may start while the previous one drains; it must
// call grid_dependency_wait() before its first global access).
cfft_status launch_kernel(const void* fn, int grid, int block, void** args, size_t smem, cudaStream_t stream,
                          bool pdl = false);
// Raises a kernel's dynamic shared-memory limit to `smem` on the current
// device, once (thread-safe); a no-op up to 48 KiB.
cfft_status ensure_smem(const void* fn, size_t smem);
// The same with a thread-block cluster of `cluster` CTAs (grid a multiple of it).
cfft_status launch_kernel_cluster(const void* fn, int grid, int block, int cluster, void** args, size_t smem,
                                  cudaStream_t stream, bool pdl = false);
int max_blocks_per_sm(const void* fn, int block, size_t smem);
// Dynamic shared memory for a launch that spreads a one-wave grid evenly over
// the SMs (ceil(grid / SMs) CTAs per SM); `smem` itself when the grid takes
// several waves, already spreads, or the padded shape would not hold it.
size_t spread_smem(const void* fn, int grid, int block, int cluster, size_t smem);
// Clusters of 9-16 CTAs (non-portable sizes) for fn; launch_kernel_cluster calls it.
cfft_status allow_cluster16(const void* fn);
// Clusters of `cluster` CTAs of fn with this shape resident at once
// (cudaOccupancyMaxActiveClusters, kept per device, kernel and shape).
int cluster_count(const void* fn, int block, int cluster, size_t smem);
// Whether one cluster of `cluster` CTAs of fn with this shape can be resident.
bool cluster_fits(const void* fn, int block, int cluster, size_t smem);
// Clusters of `cluster` CTAs of fn resident at once with one CTA per SM (dynamic
// shared memory padded to the per-block limit).  A 16-CTA cluster needs 16 SMs of
// one GPC: a 152-SM GB300 holds 7 such clusters, and 15 of 8 CTAs.
int spread_clusters(const void* fn, int block, int cluster);

// kernel<<<grid, block, smem, stream>>>(args...) as a programmatic dependent
// launch (the kernel calls grid_dependency_wait() before its first global access).
template <typename... Params, typename... Args>
cudaError_t launch_dependent(void (*kernel)(Params...), int grid, int block, size_t smem, cudaStream_t stream,
                             Args... args) {
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
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

// Persistent scratch for the *_host convenience entry points (one per thread).
cfft_status host_staging(size_t bytes, void** dev_ptr, cudaStream_t* stream);
// Page-locked, device-mapped bounce buffer of the calling thread (at most
// kHostBounceMax bytes) for small host calls on pageable memory: host address
// and the address kernels use.
constexpr size_t kHostBounceMax = size_t(4) << 20;
cfft_status host_bounce(size_t bytes, void** host_ptr, void** dev_ptr);

// Copy/compute pipeline of the *_host product entry points: `nslots` device
// buffers of `bytes` each, one stream per slot (per thread, grown on demand).
struct PipeSlot {
  void* dev;
  cudaStream_t stream;
};
cfft_status host_pipeline(int nslots, size_t bytes, PipeSlot* slots);
// The schedule of the host product entry points' pipeline (cfft_diag_set_host_chunks):
// `chunks` equal chunks on `slots` streams, after a first chunk of `first` products and
// before a last one of `last` (0: none).
struct HostChunks {
  int chunks, slots, first, last;
};
HostChunks host_chunks();

// The device address of `bytes` of page-locked host memory starting at p, or
// nullptr when the range is not one page-locked, device-mapped allocation
// (pageable memory, device memory).  Kernels then write results there
// directly: on a Grace host they cross NVLink-C2C as the kernel stores them.
void* mapped_host_range(const void* p, size_t bytes);
// Makes the current device's primary context current on the calling thread.
void bind_device_context();

}  // namespace cfft
