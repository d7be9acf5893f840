//! GPU extensions with no counterpart in the reference's API.
//!
//! The reference transforms one host buffer per call; on the GPU, throughput
//! comes from batches on device memory.  These calls take device pointers and a
//! CUDA stream (`cudaStream_t` as an untyped pointer, null = the legacy default
//! stream), are asynchronous on that stream, and return the library's status as
//! a [`GpuError`] instead of panicking.  Device memory is the caller's (allocated
//! with the CUDA runtime or a framework); every pointer must stay valid until the
//! stream has run the call.
//!
//! The negacyclic polynomial products are the pipeline that the reference's
//! caller (TFHE-rs) builds around `unordered::Plan` (u64 torus) and
//! `fft128::Plan` (u128 torus), fused into one kernel: fold, twist, forward FFT,
//! pointwise product with a device-resident Fourier operand, inverse FFT,
//! untwist and exact rounding back to the integer ring.

use alloc::sync::Arc;
use alloc::vec::Vec;
use core::ffi::{c_int, c_void};

use crate::ffi;
use crate::ordered::FftAlgo;
use crate::GpuError;

/// A CUDA stream (`cudaStream_t`), or null for the legacy default stream.
pub type Stream = *mut c_void;

impl crate::ordered::Plan {
    /// Forward FFTs of `batch` transforms stored back to back at the device pointer `buf`.
    ///
    /// # Safety
    ///
    /// `buf` must be device memory holding `batch * fft_size()` c64, valid until the stream
    /// has run the call.
    pub unsafe fn fwd_device(&self, buf: *mut f64, batch: usize, stream: Stream) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_ordered_fwd(self.raw(), buf, batch, stream))
    }

    /// Inverse FFTs of `batch` device transforms (unnormalised).
    ///
    /// # Safety
    ///
    /// As for [`fwd_device`](Self::fwd_device).
    pub unsafe fn inv_device(&self, buf: *mut f64, batch: usize, stream: Stream) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_ordered_inv(self.raw(), buf, batch, stream))
    }
}

impl crate::unordered::Plan {
    /// Forward FFTs of `batch` device transforms; outputs in the plan's permuted order.
    ///
    /// # Safety
    ///
    /// `buf` must be device memory holding `batch * fft_size()` c64, valid until the stream
    /// has run the call.
    pub unsafe fn fwd_device(&self, buf: *mut f64, batch: usize, stream: Stream) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_unordered_fwd(self.raw(), buf, batch, stream))
    }

    /// Inverse FFTs of `batch` device transforms (permuted order in, standard order out).
    ///
    /// # Safety
    ///
    /// As for [`fwd_device`](Self::fwd_device).
    pub unsafe fn inv_device(&self, buf: *mut f64, batch: usize, stream: Stream) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_unordered_inv(self.raw(), buf, batch, stream))
    }

    /// `fwd_monomial` into device memory.
    ///
    /// # Safety
    ///
    /// `buf` must be device memory of `fft_size()` c64, valid until the stream has run the call.
    pub unsafe fn fwd_monomial_device(&self, degree: usize, buf: *mut f64, stream: Stream) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_unordered_fwd_monomial(self.raw(), degree, buf, stream))
    }

    /// Serialized (standard-order) host data straight into device buffers in the plan's
    /// permuted order: the wire format loads into resident Fourier operands in one pass.
    ///
    /// # Safety
    ///
    /// `permuted` must be device memory of `batch * fft_size()` c64; `standard` must hold
    /// as many in host memory.  Both stay valid until the stream has run the call.
    pub unsafe fn from_standard_h2d(
        &self,
        standard: *const f64,
        permuted: *mut f64,
        batch: usize,
        stream: Stream,
    ) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_unordered_from_standard_h2d(self.raw(), standard, permuted, batch, stream))
    }

    /// Device Fourier buffers back to the serialized standard order in host memory.
    ///
    /// # Safety
    ///
    /// As for [`from_standard_h2d`](Self::from_standard_h2d).
    pub unsafe fn to_standard_d2h(
        &self,
        permuted: *const f64,
        standard: *mut f64,
        batch: usize,
        stream: Stream,
    ) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_unordered_to_standard_d2h(self.raw(), permuted, standard, batch, stream))
    }
}

#[cfg(feature = "fft128")]
impl crate::fft128::Plan {
    /// Forward negacyclic FFTs of `batch` transforms in four device arrays.
    ///
    /// # Safety
    ///
    /// Each pointer must be device memory of `batch * fft_size()` f64, valid until the
    /// stream has run the call.
    pub unsafe fn fwd_device(
        &self,
        re0: *mut f64,
        re1: *mut f64,
        im0: *mut f64,
        im1: *mut f64,
        batch: usize,
        stream: Stream,
    ) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_f128_fwd(self.raw(), re0, re1, im0, im1, batch, stream))
    }

    /// Inverse negacyclic FFTs of `batch` device transforms (unnormalised).
    ///
    /// # Safety
    ///
    /// As for [`fwd_device`](Self::fwd_device).
    pub unsafe fn inv_device(
        &self,
        re0: *mut f64,
        re1: *mut f64,
        im0: *mut f64,
        im1: *mut f64,
        batch: usize,
        stream: Stream,
    ) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_f128_inv(self.raw(), re0, re1, im0, im1, batch, stream))
    }
}

struct RawU64(*mut ffi::cfft_u64_product_plan);
// SAFETY: immutable after creation (include/cfft.h) but for the CTAs-per-product
// setting, an int read at each launch that changes speed only (set_cluster_size).
unsafe impl Send for RawU64 {}
unsafe impl Sync for RawU64 {}
impl Drop for RawU64 {
    fn drop(&mut self) {
        // SAFETY: created by cfft_u64_product_plan_create* and destroyed once, here.
        unsafe { ffi::cfft_u64_product_plan_destroy(self.0) }
    }
}

/// Negacyclic products of u64 polynomials of `N` coefficients (mod X^N + 1, mod 2^64),
/// through an N/2-point unordered FFT in FP64.
#[derive(Clone)]
pub struct U64ProductPlan {
    raw: Arc<RawU64>,
    n: usize,
}

impl U64ProductPlan {
    /// A plan with the given base algorithm and base size of its unordered FFT.
    pub fn new(n: usize, base_algo: FftAlgo, base_n: usize) -> Result<Self, GpuError> {
        let mut raw = core::ptr::null_mut();
        // SAFETY: valid out-pointer.
        ffi::status(unsafe { ffi::cfft_u64_product_plan_create(n, base_algo.to_c(), base_n, &mut raw) })?;
        Ok(Self { raw: Arc::new(RawU64(raw)), n })
    }

    /// A plan whose FFT is chosen by timing the candidates on the GPU.
    pub fn measure(n: usize, seconds_per_candidate: f64) -> Result<Self, GpuError> {
        let mut raw = core::ptr::null_mut();
        // SAFETY: valid out-pointer.
        ffi::status(unsafe { ffi::cfft_u64_product_plan_create_measure(n, seconds_per_candidate, &mut raw) })?;
        Ok(Self { raw: Arc::new(RawU64(raw)), n })
    }

    /// The polynomial size N.
    pub fn poly_size(&self) -> usize {
        self.n
    }

    /// The (base algorithm, base size) of the plan's unordered FFT.
    pub fn algo(&self) -> (FftAlgo, usize) {
        let mut a: c_int = 0;
        let mut b = 0usize;
        // SAFETY: live plan, valid out-pointers.
        unsafe { ffi::cfft_u64_product_algo(self.raw.0, &mut a, &mut b) };
        (FftAlgo::from_c(a), b)
    }

    /// CTAs per product: 0 automatic (a thread-block cluster for a few products or a
    /// large N), 1 one CTA, 2/4/8 a cluster of that size, capped at what the plan
    /// allows.  Changes speed only, never results.  The setting belongs to the plan,
    /// so it applies to every clone; set it before the plan is shared across threads.
    pub fn set_cluster_size(&mut self, ctas: i32) -> Result<(), GpuError> {
        // SAFETY: live plan; `&mut self` orders this call after this handle's launches.
        ffi::status(unsafe { ffi::cfft_u64_product_set_cluster_size(self.raw.0, ctas) })
    }

    /// Fourier operands of `count` signed-digit polynomials: `b` holds count * N i64,
    /// `bhat` receives count * N/2 c64 in the plan's permuted order.
    ///
    /// # Safety
    ///
    /// Both are device memory of those sizes, valid until the stream has run the call.
    pub unsafe fn prepare_operand(&self, b: *const i64, bhat: *mut f64, count: usize, stream: Stream) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_u64_prepare_operand(self.raw.0, b, bhat, count, stream))
    }

    /// `out[i] = a[i] * B_i mod (X^N + 1)` for `i < count`; `bhat_stride` is 0 (one
    /// operand for all) or N/2 (one per product).
    ///
    /// # Safety
    ///
    /// `a` and `out` are device memory of count * N u64, `bhat` of the operands; all
    /// valid until the stream has run the call.
    pub unsafe fn product(
        &self,
        a: *const u64,
        bhat: *const f64,
        bhat_stride: usize,
        out: *mut u64,
        count: usize,
        stream: Stream,
    ) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_u64_product(self.raw.0, a, bhat, bhat_stride, out, count, stream))
    }

    /// The same with `a` and `out` in host memory (best page-locked): copies in, the
    /// products and the results out are pipelined; returns when `out` holds them.
    ///
    /// # Safety
    ///
    /// `bhat` is device memory holding the operands.
    pub unsafe fn product_host(
        &self,
        a: &[u64],
        bhat: *const f64,
        bhat_stride: usize,
        out: &mut [u64],
    ) -> Result<(), GpuError> {
        assert_eq!(a.len(), out.len());
        assert_eq!(a.len() % self.n, 0);
        ffi::status(ffi::cfft_u64_product_host(
            self.raw.0,
            a.as_ptr(),
            bhat,
            bhat_stride,
            out.as_mut_ptr(),
            a.len() / self.n,
        ))
    }

    /// `out[g] = sum over t < terms of a[g][t] * B[g][t]`, accumulated in the Fourier
    /// domain with one inverse FFT per output (the external-product shape).
    ///
    /// # Safety
    ///
    /// Device memory: `a` count * terms * N u64, `bhat` count * terms * N/2 c64, `out`
    /// count * N u64, valid until the stream has run the call.
    pub unsafe fn product_sum(
        &self,
        a: *const u64,
        bhat: *const f64,
        terms: usize,
        out: *mut u64,
        count: usize,
        stream: Stream,
    ) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_u64_product_sum(self.raw.0, a, bhat, terms, out, count, stream))
    }

    /// Multiplies `count` Fourier-domain polynomials by X^degree mod (X^N + 1), in place
    /// (the blind-rotation step).
    ///
    /// # Safety
    ///
    /// `z` is device memory of count * N/2 c64, valid until the stream has run the call.
    pub unsafe fn fourier_mul_monomial(&self, degree: u64, z: *mut f64, count: usize, stream: Stream) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_u64_fourier_mul_monomial(self.raw.0, degree, z, count, stream))
    }
}

struct RawU128(*mut ffi::cfft_u128_product_plan);
// SAFETY: immutable after creation (include/cfft.h).
unsafe impl Send for RawU128 {}
unsafe impl Sync for RawU128 {}
impl Drop for RawU128 {
    fn drop(&mut self) {
        // SAFETY: created by cfft_u128_product_plan_create and destroyed once, here.
        unsafe { ffi::cfft_u128_product_plan_destroy(self.0) }
    }
}

/// Negacyclic products of u128 polynomials (coefficients as little-endian (lo, hi) u64
/// pairs) through `fft128::Plan(N/2)` in double-double arithmetic.
#[derive(Clone)]
pub struct U128ProductPlan {
    raw: Arc<RawU128>,
    n: usize,
}

impl U128ProductPlan {
    pub fn new(n: usize) -> Result<Self, GpuError> {
        let mut raw = core::ptr::null_mut();
        // SAFETY: valid out-pointer.
        ffi::status(unsafe { ffi::cfft_u128_product_plan_create(n, &mut raw) })?;
        Ok(Self { raw: Arc::new(RawU128(raw)), n })
    }

    pub fn poly_size(&self) -> usize {
        self.n
    }

    /// Fourier operands (four arrays of N/2 f64 per operand) of `count` digit polynomials.
    ///
    /// # Safety
    ///
    /// Device memory: `b` count * N i64, `bhat4` count * 2N f64.
    pub unsafe fn prepare_operand(&self, b: *const i64, bhat4: *mut f64, count: usize, stream: Stream) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_u128_prepare_operand(self.raw.0, b, bhat4, count, stream))
    }

    /// `out[i] = a[i] * B_i mod (X^N + 1, 2^128)`; `bhat_stride` is 0 or 2N (f64).
    ///
    /// # Safety
    ///
    /// Device memory: `a` and `out` count * 2N u64, `bhat4` the operands.
    pub unsafe fn product(
        &self,
        a: *const u64,
        bhat4: *const f64,
        bhat_stride: usize,
        out: *mut u64,
        count: usize,
        stream: Stream,
    ) -> Result<(), GpuError> {
        ffi::status(ffi::cfft_u128_product(self.raw.0, a, bhat4, bhat_stride, out, count, stream))
    }

    /// The same with `a` and `out` in host memory; returns when `out` holds the results.
    ///
    /// # Safety
    ///
    /// `bhat4` is device memory holding the operands.
    pub unsafe fn product_host(&self, a: &[u64], bhat4: *const f64, bhat_stride: usize, out: &mut [u64]) -> Result<(), GpuError> {
        assert_eq!(a.len(), out.len());
        assert_eq!(a.len() % (2 * self.n), 0);
        ffi::status(ffi::cfft_u128_product_host(
            self.raw.0,
            a.as_ptr(),
            bhat4,
            bhat_stride,
            out.as_mut_ptr(),
            a.len() / (2 * self.n),
        ))
    }
}

/// One product for the [`ProductQueue`]: `a` (N u64) times the Fourier operand `bhat`
/// (N/2 c64 of that size's plan) into `out` (N u64), N = 2^log2n.
pub type ProductItem = ffi::cfft_product_item;

struct RawEngine(*mut ffi::cfft_product_engine);
// SAFETY: immutable after creation (include/cfft.h).
unsafe impl Send for RawEngine {}
unsafe impl Sync for RawEngine {}
impl Drop for RawEngine {
    fn drop(&mut self) {
        // SAFETY: created by cfft_product_engine_create and destroyed once, here.
        unsafe { ffi::cfft_product_engine_destroy(self.0) }
    }
}

/// Products of mixed sizes (N = 2^6..2^17) in one persistent launch.
#[derive(Clone)]
pub struct ProductEngine {
    raw: Arc<RawEngine>,
}

impl ProductEngine {
    pub fn new(log2n: &[u32]) -> Result<Self, GpuError> {
        let mut raw = core::ptr::null_mut();
        // SAFETY: `log2n` is a valid array; valid out-pointer.
        ffi::status(unsafe { ffi::cfft_product_engine_create(log2n.as_ptr(), log2n.len(), &mut raw) })?;
        Ok(Self { raw: Arc::new(RawEngine(raw)) })
    }

    /// Prepares Fourier operands for the engine's size 2^log2n (see
    /// [`U64ProductPlan::prepare_operand`]).
    ///
    /// # Safety
    ///
    /// As for [`U64ProductPlan::prepare_operand`].
    pub unsafe fn prepare_operand(
        &self,
        log2n: u32,
        b: *const i64,
        bhat: *mut f64,
        count: usize,
        stream: Stream,
    ) -> Result<(), GpuError> {
        let plan = ffi::cfft_product_engine_plan(self.raw.0, log2n);
        if plan.is_null() {
            return Err(GpuError { status: -1, message: "size not configured in the engine".into() });
        }
        ffi::status(ffi::cfft_u64_prepare_operand(plan, b, bhat, count, stream))
    }
}

/// Work queue over a [`ProductEngine`]: callers on any thread submit groups of products
/// and get a ticket; one worker thread gathers everything pending into the next launch.
pub struct ProductQueue {
    raw: *mut ffi::cfft_product_queue,
    _engine: ProductEngine,
}

// SAFETY: submit / poll / wait may be called from any thread (include/cfft.h).
unsafe impl Send for ProductQueue {}
unsafe impl Sync for ProductQueue {}

impl ProductQueue {
    /// `max_inflight` concurrent launches (0: 3); products with N >= 2^cluster_log2n run
    /// one per thread-block cluster (0: 13).
    pub fn new(engine: &ProductEngine, max_inflight: u32, cluster_log2n: u32) -> Result<Self, GpuError> {
        let cfg = ffi::cfft_product_queue_config { max_inflight, cluster_log2n };
        let mut raw = core::ptr::null_mut();
        // SAFETY: live engine, valid config and out-pointer.
        ffi::status(unsafe { ffi::cfft_product_queue_create(engine.raw.0, &cfg, &mut raw) })?;
        Ok(Self { raw, _engine: engine.clone() })
    }

    /// Queues the items; returns their ticket at once.
    ///
    /// # Safety
    ///
    /// Every item's buffers (device memory, or page-locked host memory for `out`) must stay
    /// valid until the ticket is done.
    pub unsafe fn submit(&self, items: &[ProductItem]) -> Result<u64, GpuError> {
        let mut ticket = 0u64;
        ffi::status(ffi::cfft_product_queue_submit(self.raw, items.as_ptr(), items.len(), &mut ticket))?;
        Ok(ticket)
    }

    /// True once the ticket's products are complete.
    pub fn poll(&self, ticket: u64) -> Result<bool, GpuError> {
        // SAFETY: live queue.
        let r = unsafe { ffi::cfft_product_queue_poll(self.raw, ticket) };
        if r < 0 {
            ffi::status(r).map(|_| false)
        } else {
            Ok(r == 1)
        }
    }

    /// Blocks until the ticket's products are complete.
    pub fn wait(&self, ticket: u64) -> Result<(), GpuError> {
        // SAFETY: live queue.
        ffi::status(unsafe { ffi::cfft_product_queue_wait(self.raw, ticket) })
    }
}

impl Drop for ProductQueue {
    fn drop(&mut self) {
        // SAFETY: runs what is pending, then releases the queue; no other call runs on it now.
        unsafe { ffi::cfft_product_queue_destroy(self.raw) }
    }
}

/// Saves the persisted `Method::Measure` results (per GPU model, plan kind and size) to
/// a text file, and loads them back, so that plans created with `Measure` skip timing.
#[cfg(feature = "std")]
pub fn tune_save(path: &std::path::Path) -> Result<(), GpuError> {
    let c = std::ffi::CString::new(path.as_os_str().to_string_lossy().as_bytes()).expect("path without NUL");
    // SAFETY: NUL-terminated path.
    ffi::status(unsafe { ffi::cfft_tune_save(c.as_ptr()) })
}

#[cfg(feature = "std")]
pub fn tune_load(path: &std::path::Path) -> Result<(), GpuError> {
    let c = std::ffi::CString::new(path.as_os_str().to_string_lossy().as_bytes()).expect("path without NUL");
    // SAFETY: NUL-terminated path.
    ffi::status(unsafe { ffi::cfft_tune_load(c.as_ptr()) })
}

/// 0 when a usable sm_103 device is present, else the library's error.
pub fn device_check() -> Result<(), GpuError> {
    // SAFETY: no arguments.
    ffi::status(unsafe { ffi::cfft_device_check() })
}

/// The library's version string.
pub fn version() -> Vec<u8> {
    // SAFETY: cfft_version returns a static NUL-terminated string.
    unsafe { core::ffi::CStr::from_ptr(ffi::cfft_version()) }.to_bytes().to_vec()
}
