/*
 * cfft_diag.h -- diagnostics of libcfft_gb300.so (no counterpart in the
 * reference crate, which has no device).
 */
#ifndef CFFT_DIAG_H
#define CFFT_DIAG_H
#include "cfft.h"
#ifdef __cplusplus
extern "C" {
#endif

/* Measures the device's FP64 issue rate: eight independent chains per thread
 * on every SM, timed with CUDA events, for DFMA, DADD, DMUL and the product
 * kernel's mix (2 DADD : 1 DFMA : 1 DMUL).  rates4 receives FP64 thread
 * instructions per second for each, in that order.  The FFT kernels of this
 * library are bound by this rate on GB300, where FP64 runs at 1/64 of the
 * FP32 rate. */
cfft_status cfft_diag_fp64_rates(double* rates4);
/* The largest of the four rates of cfft_diag_fp64_rates. */
cfft_status cfft_diag_fp64_peak(double* ops_per_second);

/* Self-check of the integer-pipe double addition used by the FFT kernels:
 * `count` operand pairs from four generators (random bit patterns, random
 * exponent gaps, near-cancellation, constructed rounding ties), each summed by
 * the integer routine and by the native FP64 add.  *mismatches receives the
 * number of pairs whose results differ in any bit (NaN payloads excepted);
 * bad_pair (may be NULL) receives the first differing pair's bit patterns. */
cfft_status cfft_diag_dadd_check(uint64_t count, uint64_t seed, uint64_t* mismatches, uint64_t* bad_pair);

/* Issue rate of the integer-pipe double addition alone (additions per second). */
cfft_status cfft_diag_dadd_int_rate(double* adds_per_second);

/* Whether `bytes` at p are page-locked host memory that kernels can reach
 * directly (the in-place and direct-store host paths use it): *device_address
 * receives the address kernels use, or NULL when the range takes the staged
 * copies (pageable or device memory). */
cfft_status cfft_diag_host_mapping(const void* p, size_t bytes, void** device_address);

/* Cluster scheduling policy requested for every thread-block-cluster launch of
 * the library: 0 the driver's default, 1 spread, 2 load balancing (the
 * library's default).  Process-wide; for measurement. */
cfft_status cfft_diag_set_cluster_policy(int policy);

/* Even spreading of one-wave grids over the SMs (the c64 transform kernels pad
 * their shared memory so that ceil(grid / SMs) CTAs fit an SM): 1 on (the
 * default), 0 off.  Process-wide; for measurement. */
cfft_status cfft_diag_set_spread(int on);

/* Schedule of the u64 product's host entry point (cfft_u64_product_host): the
 * batch is copied in and multiplied in `chunks` equal chunks (default 24, at
 * least two products per SM each) over `slots` streams (default 4, at most 8),
 * after a first chunk of `first` products and before a last one of `last`
 * (0: none, the default).  0 for chunks or slots restores its default.
 * Process-wide; for measurement. */
cfft_status cfft_diag_set_host_chunks(int chunks, int slots, int first, int last);

#ifdef __cplusplus
}
#endif
#endif
