// runtime.cu -- library-wide state: errors, device checks, staging buffers.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

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
__global__ void fp64_peak_kernel(double* out, double seed) {
  double a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed + threadIdx.x + i;
  for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = __fma_rn(a[i], 0.999999, 1e-9);
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += a[i];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" cfft_status cfft_diag_fp64_peak(double* ops_per_second) {
  if (!ops_per_second) return cfft::fail(CFFT_ERR_INVALID_ARGUMENT, "null output pointer");
  const int blocks = cfft::sm_count() * 4, threads = 256;
  double* d = nullptr;
  CFFT_CUDA_TRY(cudaMalloc(&d, (size_t)blocks * threads * sizeof(double)));
  cudaEvent_t e0, e1;
  CFFT_CUDA_TRY(cudaEventCreate(&e0));
  CFFT_CUDA_TRY(cudaEventCreate(&e1));
  fp64_peak_kernel<<<blocks, threads>>>(d, 1.0);
  CFFT_CUDA_TRY(cudaEventRecord(e0));
  const int reps = 5;
  for (int r = 0; r < reps; ++r) fp64_peak_kernel<<<blocks, threads>>>(d, 1.0);
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
