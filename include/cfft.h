/*
 * cfft.h -- C ABI of the GB300 implementation of concrete-fft's FFT hot path.
 *
 * One shared library, libcfft_gb300.so (sm_103a).  Every entry point takes
 * plain pointers, sizes and a CUDA stream passed as `void*` (a cudaStream_t,
 * NULL = the legacy default stream), and returns a cfft_status.  The reference
 * crate (zama-ai/concrete-fft v0.5.1) panics where this ABI returns an error
 * code; cfft_last_error() gives the message.
 *
 * Buffers: a "c64" buffer is interleaved (re, im) f64 pairs, 16 bytes per
 * point, the memory layout of num_complex::Complex64.  Batched calls process
 * `batch` transforms stored back to back.  Functions without a `_host` suffix
 * take DEVICE pointers and are asynchronous on `stream`; `_host` functions take
 * host pointers, copy in and out and return when the result is in host memory
 * (the shape of the reference's slice API, `fwd(&self, buf: &mut [c64], ..)`).
 *
 * Results: the transforms are bit-identical to the reference's output for the
 * same algorithm, size and base size (the GPU executes the reference's exact
 * operation sequence in IEEE FP64, with the reference's twiddle tables).
 *
 * Plans are immutable after creation and may be shared across threads, like
 * the reference's `Plan: Clone + Send + Sync`.  The speed knobs without a
 * reference counterpart (cfft_*_set_int_adds, cfft_*_set_cluster_size) change
 * a plan: call them before sharing it, not while another thread uses it.
 * Results never depend on them.
 */
#ifndef CFFT_H
#define CFFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cfft_status {
  CFFT_OK = 0,
  CFFT_ERR_INVALID_SIZE = -1,      /* not a power of two, or outside the plan's range */
  CFFT_ERR_INVALID_ARGUMENT = -2,  /* null pointer, unknown algorithm, bad base size */
  CFFT_ERR_LENGTH_MISMATCH = -3,   /* buffer length differs from the plan's size */
  CFFT_ERR_CUDA = -4,              /* a CUDA call failed (message in cfft_last_error) */
  CFFT_ERR_OUT_OF_MEMORY = -5,     /* device allocation failed */
  CFFT_ERR_NO_DEVICE = -6,         /* no usable sm_103 device */
  CFFT_ERR_TIMEOUT = -7            /* a bounded device wait expired */
} cfft_status;

/* ordered::FftAlgo (src/ordered.rs:28-45), same discriminant order. */
typedef enum cfft_algo {
  CFFT_DIF2 = 0,
  CFFT_DIT2 = 1,
  CFFT_DIF4 = 2,
  CFFT_DIT4 = 3,
  CFFT_DIF8 = 4,
  CFFT_DIT8 = 5,
  CFFT_DIF16 = 6,
  CFFT_DIT16 = 7
} cfft_algo;

/* Human-readable text of the last error on any thread (never NULL). */
const char* cfft_last_error(void);
/* Library version string. */
const char* cfft_version(void);
/* 0 when a device of compute capability 10.3 is usable, else a cfft_status. */
cfft_status cfft_device_check(void);

/* Persisted Method::Measure results (no counterpart in the reference, whose
 * Measure re-times on every Plan::new).  Every *_create_measure call first
 * looks up (GPU model, plan kind, size) in a process-wide table and times the
 * candidates only on a miss, storing its choice.  save/load write and read
 * the table as text (one tab-separated entry per line). */
cfft_status cfft_tune_save(const char* path);
cfft_status cfft_tune_load(const char* path);
void cfft_tune_clear(void);
size_t cfft_tune_entries(void);

/* ======================================================= ordered::Plan ====
 * Replaces src/ordered.rs:187-373.  Sizes: powers of two, 1 <= n <= 1024
 * (the reference asserts n.trailing_zeros() < 11, src/ordered.rs:244). */
typedef struct cfft_ordered_plan cfft_ordered_plan;

/* Plan::new(n, Method::UserProvided(algo)) -- src/ordered.rs:242-278 */
cfft_status cfft_ordered_plan_create(size_t n, cfft_algo algo, cfft_ordered_plan** out);
/* Plan::new(n, Method::Measure(duration)) -- src/ordered.rs:99-180: times every
 * algorithm on the GPU for about `seconds_per_algo` each and keeps the fastest. */
cfft_status cfft_ordered_plan_create_measure(size_t n, double seconds_per_algo, cfft_ordered_plan** out);
void cfft_ordered_plan_destroy(cfft_ordered_plan* plan);
/* Plan::fft_size -- src/ordered.rs:291 */
size_t cfft_ordered_fft_size(const cfft_ordered_plan* plan);
/* Plan::algo -- src/ordered.rs:305 */
cfft_algo cfft_ordered_algo(const cfft_ordered_plan* plan);
/* Plan::fft_scratch -- src/ordered.rs:320-322: bytes of caller scratch a call
 * needs.  The GPU path keeps its scratch in shared memory: always 0. */
size_t cfft_ordered_scratch_bytes(const cfft_ordered_plan* plan);
/* Plan::fwd / Plan::inv -- src/ordered.rs:342-373, batched, in place, unnormalised. */
cfft_status cfft_ordered_fwd(const cfft_ordered_plan* plan, double* buf, size_t batch, void* stream);
cfft_status cfft_ordered_inv(const cfft_ordered_plan* plan, double* buf, size_t batch, void* stream);
cfft_status cfft_ordered_fwd_host(const cfft_ordered_plan* plan, double* buf, size_t batch);
cfft_status cfft_ordered_inv_host(const cfft_ordered_plan* plan, double* buf, size_t batch);

/* Integer-pipe share of the butterfly additions (no counterpart in the
 * reference).  GB300 issues FP64 at 1/64 of its integer rate; `eighths` (0..8)
 * of every butterfly's additions run as an exact integer-pipe IEEE add
 * instead, alongside the FP64 pipe.  Results are bit-identical for every
 * value; only the speed changes.  Measure-created plans tune it themselves. */
cfft_status cfft_ordered_set_int_adds(cfft_ordered_plan* plan, int eighths);
int cfft_ordered_int_adds(const cfft_ordered_plan* plan);

/* CTAs per transform (no counterpart in the reference): 0 chooses per call
 * (each transform split over 2..8 CTAs of a thread-block cluster when the
 * batch is too small to give every SM work; unordered transforms above 4096
 * points only up to 8192), 1 keeps the one-CTA / global-level path, 2/4/8
 * force that split.  A forced value is capped at what the plan allows (the
 * radix of the step that is split, and 8) and raised to the smallest split
 * whose parts fit shared memory (4096 points, so unordered n <= 32768).  Results
 * are bit-identical for every value. */
cfft_status cfft_ordered_set_cluster_size(cfft_ordered_plan* plan, int ctas);

/* ===================================================== unordered::Plan ====
 * Replaces src/unordered.rs:496-1036.  Any power-of-two n up to 2^28 with a
 * base (internal ordered) size base_n <= 1024, base_n >= 32 unless base_n == n
 * (src/unordered.rs:660-670). */
typedef struct cfft_unordered_plan cfft_unordered_plan;

/* Plan::new(n, Method::UserProvided { base_algo, base_n }) -- src/unordered.rs:659-747 */
cfft_status cfft_unordered_plan_create(size_t n, cfft_algo base_algo, size_t base_n, cfft_unordered_plan** out);
/* Plan::new(n, Method::Measure(duration)) -- src/unordered.rs:540-640: GPU timing
 * of bases 512/1024 (n > 256) or every ordered algorithm (n <= 256). */
cfft_status cfft_unordered_plan_create_measure(size_t n, double seconds_per_algo, cfft_unordered_plan** out);
void cfft_unordered_plan_destroy(cfft_unordered_plan* plan);
/* Plan::fft_size -- src/unordered.rs:770 */
size_t cfft_unordered_fft_size(const cfft_unordered_plan* plan);
/* Plan::algo -- src/unordered.rs:793: (base_algo, base_n) */
void cfft_unordered_algo(const cfft_unordered_plan* plan, cfft_algo* base_algo, size_t* base_n);
/* Plan::fft_scratch -- src/unordered.rs:798-800 (0: scratch is on chip or plan-owned) */
size_t cfft_unordered_scratch_bytes(const cfft_unordered_plan* plan);
/* Plan::fwd -- src/unordered.rs:826-839: standard order in, permuted order out. */
cfft_status cfft_unordered_fwd(const cfft_unordered_plan* plan, double* buf, size_t batch, void* stream);
/* Plan::inv -- src/unordered.rs:927-940: permuted order in, standard order out. */
cfft_status cfft_unordered_inv(const cfft_unordered_plan* plan, double* buf, size_t batch, void* stream);
cfft_status cfft_unordered_fwd_host(const cfft_unordered_plan* plan, double* buf, size_t batch);
cfft_status cfft_unordered_inv_host(const cfft_unordered_plan* plan, double* buf, size_t batch);
/* Plan::fwd_monomial -- src/unordered.rs:844-900: FFT of X^degree, permuted order. */
cfft_status cfft_unordered_fwd_monomial(const cfft_unordered_plan* plan, size_t degree, double* buf, void* stream);
cfft_status cfft_unordered_fwd_monomial_host(const cfft_unordered_plan* plan, size_t degree, double* buf);
/* serialize_fourier_buffer's element order -- src/unordered.rs:951-970:
 * standard[i] = permuted[bit_rev_twice(i)], batch buffers, out of place. */
cfft_status cfft_unordered_to_standard(const cfft_unordered_plan* plan, const double* permuted, double* standard,
                                       size_t batch, void* stream);
/* deserialize_fourier_buffer's element order -- src/unordered.rs:981-1036. */
cfft_status cfft_unordered_from_standard(const cfft_unordered_plan* plan, const double* standard, double* permuted,
                                         size_t batch, void* stream);
cfft_status cfft_unordered_to_standard_host(const cfft_unordered_plan* plan, const double* permuted,
                                            double* standard, size_t batch);
cfft_status cfft_unordered_from_standard_host(const cfft_unordered_plan* plan, const double* standard,
                                              double* permuted, size_t batch);
/* Serialized (standard-order) host data straight into device Fourier buffers in
 * the plan's permuted order, and back: the wire format loads into resident
 * operands (for a u64 product plan, through cfft_u64_product_fft) for any
 * base_n.  With page-locked host memory the permutation kernel reads (writes)
 * it directly and the call is asynchronous on `stream`; pageable memory is
 * staged and the call returns when done. */
cfft_status cfft_unordered_from_standard_h2d(const cfft_unordered_plan* plan, const double* standard_host,
                                             double* permuted, size_t batch, void* stream);
cfft_status cfft_unordered_to_standard_d2h(const cfft_unordered_plan* plan, const double* permuted,
                                           double* standard_host, size_t batch, void* stream);

/* Integer-pipe share of the butterfly additions, as cfft_ordered_set_int_adds. */
cfft_status cfft_unordered_set_int_adds(cfft_unordered_plan* plan, int eighths);
/* CTAs per transform, as cfft_ordered_set_cluster_size. */
cfft_status cfft_unordered_set_cluster_size(cfft_unordered_plan* plan, int ctas);
/* Points per shared-memory block (no counterpart in the reference): the
 * sub-transform one CTA holds after the levels above it ran in global memory
 * (forward; the inverse runs them after).  0 = automatic (the first level of
 * at most 4096 points); otherwise the size of one of the plan's levels (n, its
 * outer-level sizes, base_n) of at most 4096 points.  Automatic blocks shrink
 * for a call whose blocks would cover fewer than half the SMs; a block set
 * here is used for every call.  Resets the launch shape that Method::Measure
 * chose.  Results are bit-identical for every value. */
cfft_status cfft_unordered_set_block_points(cfft_unordered_plan* plan, size_t points);
size_t cfft_unordered_block_points(const cfft_unordered_plan* plan);
int cfft_unordered_int_adds(const cfft_unordered_plan* plan);

/* ======================================================== fft128::Plan ====
 * Replaces src/fft128/mod.rs:1832-1960.  n a power of two, 32 <= n <= 2^24.
 * Split double-double storage: four f64 arrays (re0, re1, im0, im1), each
 * batch * n long; forward output is in bit-reversed order, inverse is
 * unnormalised. */
typedef struct cfft_f128_plan cfft_f128_plan;
cfft_status cfft_f128_plan_create(size_t n, cfft_f128_plan** out);
void cfft_f128_plan_destroy(cfft_f128_plan* plan);
size_t cfft_f128_fft_size(const cfft_f128_plan* plan);
/* Points per shared-memory block (no counterpart in the reference): 0 =
 * automatic (512 for large batches; for small ones 4096 and fewer until the
 * blocks cover half the SMs), else a power of two in
 * [256, 4096]; the stages above the block run in global memory.  The u128
 * product plan's transforms use their fft128 plan's value.  Results are
 * bit-identical for every value.  cfft_f128_block_points returns 0 when
 * automatic. */
cfft_status cfft_f128_set_block_points(cfft_f128_plan* plan, size_t points);
size_t cfft_f128_block_points(const cfft_f128_plan* plan);
cfft_status cfft_f128_fwd(const cfft_f128_plan* plan, double* re0, double* re1, double* im0, double* im1,
                          size_t batch, void* stream);
cfft_status cfft_f128_inv(const cfft_f128_plan* plan, double* re0, double* re1, double* im0, double* im1,
                          size_t batch, void* stream);
cfft_status cfft_f128_fwd_host(const cfft_f128_plan* plan, double* re0, double* re1, double* im0, double* im1,
                               size_t batch);
cfft_status cfft_f128_inv_host(const cfft_f128_plan* plan, double* re0, double* re1, double* im0, double* im1,
                               size_t batch);

/* The crate's #[doc(hidden)] free functions, used by its benchmarks:
 * init_negacyclic_twiddles (src/fft128/mod.rs:1805-1828) fills positions
 * 1..n-1 of four host arrays of n (position 0 is left as it is), and
 * negacyclic_fwd_fft / negacyclic_inv_fft (src/fft128/mod.rs:1041-1104, one
 * entry for the _scalar/_avxfma/_avx512 variants, whose results are equal)
 * transform `batch` sets of n points with explicit twiddle arrays.  Data and
 * twiddles are DEVICE arrays here; n is a power of two in [2, 2^24]. */
cfft_status cfft_f128_init_negacyclic_twiddles(size_t n, double* twid_re0, double* twid_re1, double* twid_im0,
                                               double* twid_im1);
cfft_status cfft_f128_negacyclic_fwd(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                     const double* twid_re0, const double* twid_re1, const double* twid_im0,
                                     const double* twid_im1, void* stream);
cfft_status cfft_f128_negacyclic_inv(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                     const double* twid_re0, const double* twid_re1, const double* twid_im0,
                                     const double* twid_im1, void* stream);
/* The same on HOST arrays, the reference's slice signatures (staged through
 * device memory; returns when the result is back in host memory). */
cfft_status cfft_f128_negacyclic_fwd_host(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                          const double* twid_re0, const double* twid_re1, const double* twid_im0,
                                          const double* twid_im1);
cfft_status cfft_f128_negacyclic_inv_host(size_t n, size_t batch, double* re0, double* re1, double* im0, double* im1,
                                          const double* twid_re0, const double* twid_re1, const double* twid_im0,
                                          const double* twid_im1);
/* f128::sincospi -- src/fft128/f128_ops.rs:534-575, on the host: sin(pi x) and
 * cos(pi x) of the double-double x = x_hi + x_lo as (hi, lo) pairs, bit-identical
 * to the crate.  Inputs above 1 or below -1 (f128's lexicographic order) give
 * CFFT_ERR_INVALID_ARGUMENT where the crate panics. */
cfft_status cfft_f128_sincospi(double x_hi, double x_lo, double* sin_out2, double* cos_out2);

/* ================================================ negacyclic products ====
 * The reference's caller (TFHE-rs) builds polynomial products mod X^N + 1 on
 * unordered::Plan (u64 torus) and fft128::Plan (u128 torus); the crate itself
 * has no product code.  These entry points fuse that whole pipeline into one
 * kernel: fold N coefficients into N/2 complex points, twist, forward FFT,
 * pointwise product with a device-resident Fourier operand, inverse FFT,
 * untwist, exact rounding back to the integer ring.
 *
 * u64: coefficients are read as i64, rounded with floor(x + 1/2) and reduced
 * mod 2^64.  N a power of two, 64 <= N <= 2^29: one CTA per product up to
 * N = 8192, a thread-block cluster of 2..16 CTAs per product up to 16384 (and
 * for small batches, see cfft_u64_product_set_cluster_size), and from 32768
 * the five-launch path on a workspace from the stream-ordered allocator (a
 * forced cluster size keeps clusters up to 65536).  bhat
 * holds N/2 c64 per operand in the plan's permuted order; `bhat_stride` is 0
 * (one operand shared by all products) or N/2 (one operand per product). */
typedef struct cfft_u64_product_plan cfft_u64_product_plan;
cfft_status cfft_u64_product_plan_create(size_t N, cfft_algo base_algo, size_t base_n, cfft_u64_product_plan** out);
cfft_status cfft_u64_product_plan_create_measure(size_t N, double seconds_per_algo, cfft_u64_product_plan** out);
void cfft_u64_product_plan_destroy(cfft_u64_product_plan* plan);
size_t cfft_u64_product_poly_size(const cfft_u64_product_plan* plan);
void cfft_u64_product_algo(const cfft_u64_product_plan* plan, cfft_algo* base_algo, size_t* base_n);
/* Integer-pipe share of the butterfly additions, as cfft_ordered_set_int_adds. */
cfft_status cfft_u64_product_set_int_adds(cfft_u64_product_plan* plan, int eighths);
int cfft_u64_product_int_adds(const cfft_u64_product_plan* plan);
/* CTAs per product (no counterpart in the reference): 0 chooses per call (a
 * cluster when N > 8192, which needs one, or when the batch is too small to
 * give every SM a product; a few products of a plan without an outer level,
 * N/2 = base_n (up to one per SM; radix-2 bases fewer than SMs/2), or with one
 * of radix 2 or 4 over a DIF base (fewer than SMs/2), on a cluster over the
 * base algorithm's residue classes), 1 one CTA (N <= 8192),
 * 2/4/8 force a cluster of that size, capped
 * at what the plan allows (level 0's radix, or the base radix without levels,
 * with at least 64 points per CTA; N > 8192 also needs N/2/S <= 4096).
 * Results are bit-identical for every value. */
cfft_status cfft_u64_product_set_cluster_size(cfft_u64_product_plan* plan, int ctas);
/* b: `count` polynomials of N signed digits -> bhat: count * N/2 c64. */
cfft_status cfft_u64_prepare_operand(const cfft_u64_product_plan* plan, const int64_t* b, double* bhat, size_t count,
                                     void* stream);
/* out[i] = a[i] * B_i mod (X^N + 1), i < count; a, out: count * N u64. */
cfft_status cfft_u64_product(const cfft_u64_product_plan* plan, const uint64_t* a, const double* bhat,
                             size_t bhat_stride, uint64_t* out, size_t count, void* stream);
/* Host buffers for a and out (bhat stays device-resident). */
cfft_status cfft_u64_product_host(const cfft_u64_product_plan* plan, const uint64_t* a, const double* bhat,
                                  size_t bhat_stride, uint64_t* out, size_t count);

/* Products summed in the Fourier domain (the external-product shape; no
 * counterpart in the reference): out[g] = sum_{t < terms} a[g][t] * B[g][t]
 * mod (X^N + 1), every term transformed forward, multiplied and accumulated
 * in term order, then one inverse per group instead of one per term.
 * a: count * terms * N u64; bhat: count * terms * N/2 c64; out: count * N u64.
 * N <= 2^29: one output per CTA up to 8192 (fewer than SMs/2 outputs of a plan
 * on a DIF base without an outer level or with one of radix 2, 4 or 8: one
 * thread-block cluster each), per
 * thread-block cluster up to 16384 (65536 with a forced cluster size), and
 * from 32768 the unfused steps on a stream-ordered workspace of at most 1 GiB
 * (groups in chunks). */
cfft_status cfft_u64_product_sum(const cfft_u64_product_plan* plan, const uint64_t* a, const double* bhat,
                                 size_t terms, uint64_t* out, size_t count, void* stream);

/* The same pipeline unfused, one launch per step (for callers that keep the
 * Fourier-domain data themselves; bit-identical to cfft_u64_product):
 *   cfft_u64_fold_twist -> cfft_unordered_fwd(cfft_u64_product_fft(plan)) ->
 *   cfft_c64_pointwise -> cfft_unordered_inv -> cfft_u64_untwist_round.
 * z holds count * N/2 c64.  Every plan size (N up to 2^29) works here. */
cfft_status cfft_u64_fold_twist(const cfft_u64_product_plan* plan, const uint64_t* a, double* z, size_t count,
                                void* stream);
/* z[p][k] = bhat[p*bhat_stride + k] * z[p][k] (the reference's FMA complex product). */
cfft_status cfft_c64_pointwise(const double* bhat, size_t bhat_stride, double* z, size_t n, size_t count,
                               void* stream);
cfft_status cfft_u64_untwist_round(const cfft_u64_product_plan* plan, const double* z, uint64_t* out, size_t count,
                                   void* stream);
/* The plan's N/2-point unordered transform (owned by the product plan). */
cfft_unordered_plan* cfft_u64_product_fft(const cfft_u64_product_plan* plan);
/* z[p] <- Fourier form of X^degree mod (X^N + 1) times z[p], p < count, in place
 * (z: count * N/2 c64 in the plan's Fourier layout: a prepared operand or a
 * forward-transformed, twisted polynomial).  degree is taken mod 2N, X^N = -1.
 * The monomial's Fourier form is cfft_u64_prepare_operand of its digits, so the
 * result is bit-identical to preparing X^degree and calling cfft_c64_pointwise
 * (the blind-rotation step: rotate a Fourier-domain polynomial by a monomial). */
cfft_status cfft_u64_fourier_mul_monomial(const cfft_u64_product_plan* plan, unsigned long long degree, double* z,
                                          size_t count, void* stream);

/* Mixed-size product engine: one persistent launch over a DEVICE array of
 * items of any configured N (2^6..2^17), each with its own operand, result
 * bit-identical to cfft_u64_product.  Products with N/2 > 2048 keep their
 * complex data in `workspace` (cfft_product_engine_workspace_bytes, device
 * memory, one per concurrently running launch).  `counter` is a device uint
 * the run zeroes and uses as its work queue head (one per concurrently
 * running launch).  Operands for size N are prepared with
 * cfft_u64_prepare_operand(cfft_product_engine_plan(engine, log2N), ...). */
typedef struct cfft_product_item {
  const uint64_t* a;  /* N u64 coefficients (device) */
  const double* bhat; /* N/2 c64 Fourier operand (device, the size's permuted order) */
  uint64_t* out;      /* N u64 result (device) */
  uint32_t log2N;
  uint32_t reserved;  /* must be 0 */
} cfft_product_item;
typedef struct cfft_product_engine cfft_product_engine;
cfft_status cfft_product_engine_create(const uint32_t* log2N, size_t count, cfft_product_engine** out);
void cfft_product_engine_destroy(cfft_product_engine* engine);
size_t cfft_product_engine_workspace_bytes(const cfft_product_engine* engine);
const cfft_u64_product_plan* cfft_product_engine_plan(const cfft_product_engine* engine, uint32_t log2N);
cfft_status cfft_product_engine_run(const cfft_product_engine* engine, const cfft_product_item* items, size_t count,
                                    unsigned int* counter, double* workspace, void* stream);
/* The engine behind a work queue (the submit / poll API; no counterpart in the
 * reference, whose callers run one product per call): callers on any thread
 * submit groups of items and get a ticket; one worker thread per queue gathers
 * everything pending into the next launch on a free slot (the engine over the
 * small products and, beside it, one thread-block cluster per product of
 * N >= 2^cluster_log2N), at most max_inflight launches at once.  Item buffers
 * are device memory or page-locked host memory (results are then stored
 * straight into host memory); pageable host memory is refused.  Buffers must
 * stay valid until the ticket is done.  poll returns 1 when the ticket's
 * products are complete, 0 while they are queued or running, a negative
 * cfft_status if its launch failed; a ticket reported done once reads as done
 * afterwards.  destroy runs everything submitted, then returns; no other call
 * on the queue may run or start meanwhile. */
typedef struct cfft_product_queue_config {
  uint32_t max_inflight;  /* concurrent launches, 1..4 (0: 3) */
  uint32_t cluster_log2N; /* products with N >= 2^cluster_log2N run one per thread-block cluster
                             (> 17: never; 0: automatic, N >= 8192, and every size that has a
                             cluster kernel in a launch of at most 12 products) */
} cfft_product_queue_config;
typedef struct cfft_product_queue cfft_product_queue;
cfft_status cfft_product_queue_create(const cfft_product_engine* engine, const cfft_product_queue_config* config,
                                      cfft_product_queue** out);
void cfft_product_queue_destroy(cfft_product_queue* queue);
cfft_status cfft_product_queue_submit(cfft_product_queue* queue, const cfft_product_item* items, size_t count,
                                      uint64_t* ticket);
int cfft_product_queue_poll(cfft_product_queue* queue, uint64_t ticket);
cfft_status cfft_product_queue_wait(cfft_product_queue* queue, uint64_t ticket);

/* cfft_product_engine_run without any allocation (no counterpart in the
 * reference): for callers that cannot allocate device memory on their call
 * path -- code inside a framework whose own allocator has reserved the device
 * memory budget, or latency-critical loops where cudaMalloc/cudaFree would
 * synchronise the device.  The counter and the workspace come from a static
 * device array (256 B + 24 MiB) instead of caller buffers.  Every GPU that
 * loads the library holds that array until exit; under CUDA's lazy module
 * loading it is committed at the first cfft_product_engine_create on a device,
 * so a caller that hands the device budget to its own allocator creates its
 * engines first (or leaves 24 MiB free).  Limit: engines with a size above
 * N = 16384 are rejected with CFFT_ERR_INVALID_SIZE, on any device.  The
 * launch runs on at most 24 MiB / (N_max / 2 x 16 B) CTAs (192 when the
 * engine's largest N is 16384), and that cap applies to all items of the call,
 * small N included.  The first call on a device looks up the array's device
 * address; make it before any stream capture.  The address is kept for the
 * life of the process and does not survive cudaDeviceReset.  All calls share
 * the array, so calls that overlap on the GPU race: serialise them.  Results
 * are bit-identical to cfft_product_engine_run. */
cfft_status cfft_product_engine_run_static(const cfft_product_engine* engine, const cfft_product_item* items,
                                           size_t count, void* stream);

/* ============================================ serving loop (continuous batching) ====
 * A request is (k+1)*l products of one size N: signed b-bit digit polynomials
 * times device-resident Fourier operands (the TFHE external-product shape);
 * its content is a function of (seed, request id).  cfft_server_run serves a
 * seeded Poisson stream in real time: admission gated by the output ring and
 * by the device's free memory read during the run (mem_reserve_bytes),
 * everything admitted since the last launch batched into one
 * product-engine run, up to max_inflight runs overlapping on the device.  With
 * plain = 1 it serves the same stream one request at a time through the
 * unfused pipeline (one launch per step), the comparator. */
typedef struct cfft_serve_config {
  double rate;          /* mean arrivals per second */
  double duration_s;    /* arrival window */
  uint32_t log2N_min;   /* N uniform over 2^log2N_min .. 2^log2N_max */
  uint32_t log2N_max;
  uint32_t k_max;       /* k uniform in 1..k_max */
  uint32_t l_max;       /* l uniform in 1..l_max; (k+1)*l <= 16 products */
  uint32_t plain;       /* 1: unbatched comparator */
  uint32_t max_inflight; /* concurrent launches, 1..3 */
  uint32_t record_every; /* keep the outputs of every k-th request (0: none) */
  uint32_t cluster_log2N; /* batched mode: products with N >= 2^cluster_log2N run one per
                             thread-block cluster beside the engine launch (> 17: never; 0:
                             automatic, N >= 8192, and every size that has a cluster kernel in
                             a launch of at most 12 products) */
  uint32_t staged_io;    /* batched mode: 0 = the kernels read the item records from and store
                            the results into page-locked host memory; 1 = item records copied
                            in and results copied out per launch */
  uint32_t via_queue;    /* batched mode through the public work queue (cfft_product_queue_*):
                            each request submitted on arrival, its ticket polled */
  uint64_t mem_reserve_bytes; /* batched mode, device memory gate: the output bytes of admitted,
                                 unfinished requests stay within the device's free memory less
                                 this reserve, read with cudaMemGetInfo by a reader thread every
                                 20 ms during the run (a request is always admitted when
                                 nothing is in flight, so the stream makes progress) */
  uint64_t mem_free_override; /* nonzero: stands in for cudaMemGetInfo's free bytes (tests) */
} cfft_serve_config;
typedef struct cfft_serve_stats {
  uint64_t requests, products, launches, deferred_admissions;
  double products_per_s, p50_ms, p99_ms, max_ms, mean_batch, span_s;
  uint64_t memory_deferrals; /* admissions held back by the device memory gate (the others by ring space) */
  uint64_t input_bytes;      /* item records the launches read (32 B per product) */
  uint64_t output_bytes;     /* results delivered to host memory */
  double min_memory_budget_mib; /* smallest device memory budget the gate saw */
} cfft_serve_stats;
typedef struct cfft_server cfft_server;
/* Resident state: digit pools and Fourier operands (operand_bytes in total) for
 * each size, and an output ring of ring_bytes (0: a quarter of free memory,
 * at most 4 GiB), the admission gate. */
cfft_status cfft_server_create(const cfft_product_engine* engine, const uint32_t* log2N, size_t nsizes,
                               uint64_t operand_bytes, uint64_t ring_bytes, uint64_t seed, cfft_server** out);
void cfft_server_destroy(cfft_server* server);
cfft_status cfft_server_run(cfft_server* server, const cfft_serve_config* config, cfft_serve_stats* stats);
/* Checking: outputs kept by the last run, the shape and inputs of request `id`,
 * and the same request computed alone (outside any mix). */
size_t cfft_server_recorded(const cfft_server* server);
cfft_status cfft_server_recorded_ids(const cfft_server* server, uint64_t* ids, size_t cap);
cfft_status cfft_server_recorded_output(const cfft_server* server, uint64_t id, uint64_t* out, size_t words);
cfft_status cfft_server_request_shape(const cfft_server* server, const cfft_serve_config* config, uint64_t id,
                                      uint32_t* log2N, uint32_t* nprod);
cfft_status cfft_server_request_inputs(const cfft_server* server, const cfft_serve_config* config, uint64_t id,
                                       int64_t* digits, double* bhat);
cfft_status cfft_server_run_alone(cfft_server* server, const cfft_serve_config* config, uint64_t id, uint64_t* out,
                                  size_t words);

/* u128: coefficients as little-endian (lo, hi) u64 pairs read as i128,
 * double-double arithmetic around fft128::Plan(N/2), floor(x + 1/2) mod 2^128.
 * 64 <= N <= 2^25: one fused kernel up to N = 8192 (a few products of
 * N = 128..8192: one thread-block cluster each, of 16 CTAs at N = 4096 and
 * 8192 where the device fits one); above, five launches around the plan's
 * transform on a workspace from the stream-ordered allocator (2N f64 per
 * product, freed on the stream).  bhat holds 4 arrays of N/2 f64
 * (re0, re1, im0, im1) per operand; bhat_stride is 0 or 2N (doubles). */
typedef struct cfft_u128_product_plan cfft_u128_product_plan;
cfft_status cfft_u128_product_plan_create(size_t N, cfft_u128_product_plan** out);
void cfft_u128_product_plan_destroy(cfft_u128_product_plan* plan);
size_t cfft_u128_product_poly_size(const cfft_u128_product_plan* plan);
/* The plan's fft128::Plan(N/2) (owned by the product plan; do not destroy it). */
cfft_f128_plan* cfft_u128_product_fft(cfft_u128_product_plan* plan);
cfft_status cfft_u128_prepare_operand(const cfft_u128_product_plan* plan, const int64_t* b, double* bhat4,
                                      size_t count, void* stream);
cfft_status cfft_u128_product(const cfft_u128_product_plan* plan, const uint64_t* a, const double* bhat4,
                              size_t bhat_stride, uint64_t* out, size_t count, void* stream);
/* Host buffers for a and out (bhat4 stays device-resident): the count is split
 * into chunks whose copies in, products and copies out are pipelined over
 * several streams.  Returns when the results are in `out`. */
cfft_status cfft_u128_product_host(const cfft_u128_product_plan* plan, const uint64_t* a, const double* bhat4,
                                   size_t bhat_stride, uint64_t* out, size_t count);

/* ============================================ mixed-size batch (persistent) ====
 * Many c64 transforms of different sizes and kinds in one persistent kernel
 * launch (no counterpart in the reference, whose plans transform one buffer of
 * one size per call).  Items live anywhere in one device buffer; each is the
 * transform the matching ordered::Plan / unordered::Plan would compute, with
 * the schedule below, and its result is bit-identical to that plan's. */
typedef struct cfft_batch_item {
  uint64_t offset;     /* first point of the item in the buffer (c64 units) */
  uint32_t log2n;      /* size 2^log2n: ordered 1..10, unordered 1..16 */
  uint32_t kind;       /* 0: ordered::Plan, 1: unordered::Plan */
  uint32_t direction;  /* 1: fwd, 2: inv, 3: fwd then inv (one shared-memory residency) */
  uint32_t reserved;   /* must be 0 */
} cfft_batch_item;
typedef struct cfft_batch cfft_batch;
/* Groups the items into same-size work units ordered longest first and picks
 * each size class's schedule (base algorithm, base size, transforms per unit).
 * tune_seconds > 0 times the candidates on the device for about that long per
 * candidate (the analogue of Method::Measure); 0 keeps the default schedule. */
cfft_status cfft_batch_create(const cfft_batch_item* items, size_t count, double tune_seconds, cfft_batch** out);
void cfft_batch_destroy(cfft_batch* batch);
size_t cfft_batch_units(const cfft_batch* batch);
/* The schedule chosen for one size class. */
cfft_status cfft_batch_schedule(const cfft_batch* batch, uint32_t kind, uint32_t log2n, uint32_t direction,
                                cfft_algo* base_algo, size_t* base_n, uint32_t* per_unit);
/* One persistent launch over every item, in place on `data`.  On a non-NULL
 * stream the launch is captured into a CUDA graph on first use (per stream and
 * buffer) and replayed afterwards.  Runs of one batch must not overlap. */
cfft_status cfft_batch_run(cfft_batch* batch, double* data, void* stream);
/* The batch from host memory and back (no counterpart in the reference): the
 * items, in offset order, are split into about 16 chunks of equal size; each
 * chunk's points are copied host -> device into `dev` (same layout as `host`),
 * transformed by a persistent launch over the chunk's items, and copied back,
 * the chunks pipelined over three internal streams so that copies overlap
 * transforms.  Ordered after prior work on `stream`; later work on `stream`
 * waits for it.  Only the point ranges of items are copied.  `host` should be
 * pinned (page-locked) memory for the copies to overlap.  Runs of one batch
 * must not overlap on the GPU. */
cfft_status cfft_batch_run_host(cfft_batch* batch, double* host, double* dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CFFT_H */
