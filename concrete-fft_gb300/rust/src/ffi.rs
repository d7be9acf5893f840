//! Raw bindings of libcfft_gb300.so: one declaration per entry point of
//! include/cfft.h that this crate calls.  Every function returns a cfft_status
//! (0 = success, negative = error, message in `cfft_last_error`), except the
//! destroy/query functions noted in the header.
//!
//! Enum and status arguments cross the boundary as `c_int`; `size_t` as `usize`;
//! the CUDA stream as an untyped pointer (a `cudaStream_t`, null = the legacy
//! default stream).

#![allow(non_camel_case_types)]

use alloc::string::String;
use core::ffi::{c_char, c_int, c_void};

#[repr(C)]
pub struct cfft_ordered_plan {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct cfft_unordered_plan {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct cfft_f128_plan {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct cfft_u64_product_plan {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct cfft_u128_product_plan {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct cfft_product_engine {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct cfft_product_queue {
    _opaque: [u8; 0],
}

/// `cfft_product_item` of include/cfft.h: one product of the engine / work queue.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cfft_product_item {
    pub a: *const u64,
    pub bhat: *const f64,
    pub out: *mut u64,
    pub log2n: u32,
    pub reserved: u32,
}

/// `cfft_product_queue_config` of include/cfft.h.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cfft_product_queue_config {
    pub max_inflight: u32,
    pub cluster_log2n: u32,
}

pub type Stream = *mut c_void;

extern "C" {
    pub fn cfft_last_error() -> *const c_char;
    pub fn cfft_version() -> *const c_char;
    pub fn cfft_device_check() -> c_int;
    pub fn cfft_tune_save(path: *const c_char) -> c_int;
    pub fn cfft_tune_load(path: *const c_char) -> c_int;

    // ordered::Plan (src/ordered.rs:187-373)
    pub fn cfft_ordered_plan_create(n: usize, algo: c_int, out: *mut *mut cfft_ordered_plan) -> c_int;
    pub fn cfft_ordered_plan_create_measure(n: usize, seconds: f64, out: *mut *mut cfft_ordered_plan) -> c_int;
    pub fn cfft_ordered_plan_destroy(plan: *mut cfft_ordered_plan);
    pub fn cfft_ordered_fft_size(plan: *const cfft_ordered_plan) -> usize;
    pub fn cfft_ordered_algo(plan: *const cfft_ordered_plan) -> c_int;
    pub fn cfft_ordered_fwd(plan: *const cfft_ordered_plan, buf: *mut f64, batch: usize, stream: Stream) -> c_int;
    pub fn cfft_ordered_inv(plan: *const cfft_ordered_plan, buf: *mut f64, batch: usize, stream: Stream) -> c_int;
    pub fn cfft_ordered_fwd_host(plan: *const cfft_ordered_plan, buf: *mut f64, batch: usize) -> c_int;
    pub fn cfft_ordered_inv_host(plan: *const cfft_ordered_plan, buf: *mut f64, batch: usize) -> c_int;

    // unordered::Plan (src/unordered.rs:496-1036)
    pub fn cfft_unordered_plan_create(
        n: usize,
        base_algo: c_int,
        base_n: usize,
        out: *mut *mut cfft_unordered_plan,
    ) -> c_int;
    pub fn cfft_unordered_plan_create_measure(n: usize, seconds: f64, out: *mut *mut cfft_unordered_plan) -> c_int;
    pub fn cfft_unordered_plan_destroy(plan: *mut cfft_unordered_plan);
    pub fn cfft_unordered_fft_size(plan: *const cfft_unordered_plan) -> usize;
    pub fn cfft_unordered_algo(plan: *const cfft_unordered_plan, base_algo: *mut c_int, base_n: *mut usize);
    pub fn cfft_unordered_fwd(plan: *const cfft_unordered_plan, buf: *mut f64, batch: usize, stream: Stream) -> c_int;
    pub fn cfft_unordered_inv(plan: *const cfft_unordered_plan, buf: *mut f64, batch: usize, stream: Stream) -> c_int;
    pub fn cfft_unordered_fwd_host(plan: *const cfft_unordered_plan, buf: *mut f64, batch: usize) -> c_int;
    pub fn cfft_unordered_inv_host(plan: *const cfft_unordered_plan, buf: *mut f64, batch: usize) -> c_int;
    pub fn cfft_unordered_fwd_monomial(
        plan: *const cfft_unordered_plan,
        degree: usize,
        buf: *mut f64,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_unordered_fwd_monomial_host(plan: *const cfft_unordered_plan, degree: usize, buf: *mut f64) -> c_int;
    pub fn cfft_unordered_to_standard_host(
        plan: *const cfft_unordered_plan,
        permuted: *const f64,
        standard: *mut f64,
        batch: usize,
    ) -> c_int;
    pub fn cfft_unordered_from_standard_host(
        plan: *const cfft_unordered_plan,
        standard: *const f64,
        permuted: *mut f64,
        batch: usize,
    ) -> c_int;
    pub fn cfft_unordered_from_standard_h2d(
        plan: *const cfft_unordered_plan,
        standard_host: *const f64,
        permuted: *mut f64,
        batch: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_unordered_to_standard_d2h(
        plan: *const cfft_unordered_plan,
        permuted: *const f64,
        standard_host: *mut f64,
        batch: usize,
        stream: Stream,
    ) -> c_int;

    // fft128 (src/fft128/mod.rs:1041-1960, src/fft128/f128_ops.rs:534-575)
    pub fn cfft_f128_plan_create(n: usize, out: *mut *mut cfft_f128_plan) -> c_int;
    pub fn cfft_f128_plan_destroy(plan: *mut cfft_f128_plan);
    pub fn cfft_f128_fft_size(plan: *const cfft_f128_plan) -> usize;
    pub fn cfft_f128_fwd(
        plan: *const cfft_f128_plan,
        re0: *mut f64,
        re1: *mut f64,
        im0: *mut f64,
        im1: *mut f64,
        batch: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_f128_inv(
        plan: *const cfft_f128_plan,
        re0: *mut f64,
        re1: *mut f64,
        im0: *mut f64,
        im1: *mut f64,
        batch: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_f128_fwd_host(
        plan: *const cfft_f128_plan,
        re0: *mut f64,
        re1: *mut f64,
        im0: *mut f64,
        im1: *mut f64,
        batch: usize,
    ) -> c_int;
    pub fn cfft_f128_inv_host(
        plan: *const cfft_f128_plan,
        re0: *mut f64,
        re1: *mut f64,
        im0: *mut f64,
        im1: *mut f64,
        batch: usize,
    ) -> c_int;
    pub fn cfft_f128_init_negacyclic_twiddles(
        n: usize,
        twid_re0: *mut f64,
        twid_re1: *mut f64,
        twid_im0: *mut f64,
        twid_im1: *mut f64,
    ) -> c_int;
    pub fn cfft_f128_negacyclic_fwd_host(
        n: usize,
        batch: usize,
        re0: *mut f64,
        re1: *mut f64,
        im0: *mut f64,
        im1: *mut f64,
        twid_re0: *const f64,
        twid_re1: *const f64,
        twid_im0: *const f64,
        twid_im1: *const f64,
    ) -> c_int;
    pub fn cfft_f128_negacyclic_inv_host(
        n: usize,
        batch: usize,
        re0: *mut f64,
        re1: *mut f64,
        im0: *mut f64,
        im1: *mut f64,
        twid_re0: *const f64,
        twid_re1: *const f64,
        twid_im0: *const f64,
        twid_im1: *const f64,
    ) -> c_int;
    pub fn cfft_f128_sincospi(x_hi: f64, x_lo: f64, sin_out2: *mut f64, cos_out2: *mut f64) -> c_int;

    // negacyclic products (the caller-side pipeline of TFHE-rs, fused on the GPU)
    pub fn cfft_u64_product_plan_create(
        n: usize,
        base_algo: c_int,
        base_n: usize,
        out: *mut *mut cfft_u64_product_plan,
    ) -> c_int;
    pub fn cfft_u64_product_plan_create_measure(
        n: usize,
        seconds: f64,
        out: *mut *mut cfft_u64_product_plan,
    ) -> c_int;
    pub fn cfft_u64_product_plan_destroy(plan: *mut cfft_u64_product_plan);
    pub fn cfft_u64_product_poly_size(plan: *const cfft_u64_product_plan) -> usize;
    pub fn cfft_u64_product_algo(plan: *const cfft_u64_product_plan, base_algo: *mut c_int, base_n: *mut usize);
    pub fn cfft_u64_product_set_cluster_size(plan: *mut cfft_u64_product_plan, ctas: c_int) -> c_int;
    pub fn cfft_u64_prepare_operand(
        plan: *const cfft_u64_product_plan,
        b: *const i64,
        bhat: *mut f64,
        count: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_u64_product(
        plan: *const cfft_u64_product_plan,
        a: *const u64,
        bhat: *const f64,
        bhat_stride: usize,
        out: *mut u64,
        count: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_u64_product_host(
        plan: *const cfft_u64_product_plan,
        a: *const u64,
        bhat: *const f64,
        bhat_stride: usize,
        out: *mut u64,
        count: usize,
    ) -> c_int;
    pub fn cfft_u64_product_sum(
        plan: *const cfft_u64_product_plan,
        a: *const u64,
        bhat: *const f64,
        terms: usize,
        out: *mut u64,
        count: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_u64_fourier_mul_monomial(
        plan: *const cfft_u64_product_plan,
        degree: u64,
        z: *mut f64,
        count: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_u128_product_plan_create(n: usize, out: *mut *mut cfft_u128_product_plan) -> c_int;
    pub fn cfft_u128_product_plan_destroy(plan: *mut cfft_u128_product_plan);
    pub fn cfft_u128_product_poly_size(plan: *const cfft_u128_product_plan) -> usize;
    pub fn cfft_u128_prepare_operand(
        plan: *const cfft_u128_product_plan,
        b: *const i64,
        bhat4: *mut f64,
        count: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_u128_product(
        plan: *const cfft_u128_product_plan,
        a: *const u64,
        bhat4: *const f64,
        bhat_stride: usize,
        out: *mut u64,
        count: usize,
        stream: Stream,
    ) -> c_int;
    pub fn cfft_u128_product_host(
        plan: *const cfft_u128_product_plan,
        a: *const u64,
        bhat4: *const f64,
        bhat_stride: usize,
        out: *mut u64,
        count: usize,
    ) -> c_int;

    // mixed-size product engine and its work queue
    pub fn cfft_product_engine_create(log2n: *const u32, count: usize, out: *mut *mut cfft_product_engine) -> c_int;
    pub fn cfft_product_engine_destroy(engine: *mut cfft_product_engine);
    pub fn cfft_product_engine_plan(engine: *const cfft_product_engine, log2n: u32) -> *const cfft_u64_product_plan;
    pub fn cfft_product_queue_create(
        engine: *const cfft_product_engine,
        config: *const cfft_product_queue_config,
        out: *mut *mut cfft_product_queue,
    ) -> c_int;
    pub fn cfft_product_queue_destroy(queue: *mut cfft_product_queue);
    pub fn cfft_product_queue_submit(
        queue: *mut cfft_product_queue,
        items: *const cfft_product_item,
        count: usize,
        ticket: *mut u64,
    ) -> c_int;
    pub fn cfft_product_queue_poll(queue: *mut cfft_product_queue, ticket: u64) -> c_int;
    pub fn cfft_product_queue_wait(queue: *mut cfft_product_queue, ticket: u64) -> c_int;
}

/// The message of the library's last error.
pub fn last_error() -> String {
    // SAFETY: cfft_last_error never returns null and points at a NUL-terminated string.
    String::from(unsafe { core::ffi::CStr::from_ptr(cfft_last_error()) }.to_string_lossy())
}

/// Where the reference panics (`assert!` on sizes, base sizes and buffer lengths), the library
/// returns a status: turn it back into the reference's panic.
#[track_caller]
pub fn check(status: c_int) {
    if status != 0 {
        panic!("concrete-fft (GB300, status {status}): {}", last_error());
    }
}

/// A status as a `Result`, for the GPU-only extensions that report errors instead of panicking.
pub fn status(status: c_int) -> Result<(), crate::GpuError> {
    if status == 0 {
        Ok(())
    } else {
        Err(crate::GpuError { status, message: last_error() })
    }
}
