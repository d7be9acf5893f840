//! concrete-fft's API on a GB300 GPU.
//!
//! This crate has the module layout, types and method signatures of concrete-fft
//! v0.5.1 (`ordered`, `unordered`, `fft128`, `c64`), so that a user of the
//! reference (TFHE-rs, for example) switches by patching the dependency.  Every
//! transform runs on the GPU through libcfft_gb300.so (include/cfft.h): the
//! slice methods (`fwd(&self, buf: &mut [c64], stack)` and the like) use the
//! library's host entry points, which copy in, transform and copy out (or, with
//! page-locked buffers, transform in place across the host link); results are
//! bit-identical to the reference's for the same algorithm and size.
//!
//! Where the reference panics (`assert!` on sizes, base sizes and buffer
//! lengths), so does this crate, with the library's message.  There is no CPU
//! fallback: without a usable sm_103 device every call panics.
//!
//! Beyond the reference's API, [`gpu`] exposes what a GPU caller needs for
//! throughput: batched transforms on device buffers and a stream, and the fused
//! negacyclic polynomial products (u64 and u128 torus) with device-resident
//! Fourier operands, the product engine and its work queue.

#![cfg_attr(not(feature = "std"), no_std)]
#![allow(non_camel_case_types)]
#![cfg_attr(docsrs, feature(doc_cfg))]

extern crate alloc;

use alloc::string::String;

mod ffi;

pub mod gpu;
pub mod ordered;
pub mod unordered;

#[cfg(feature = "fft128")]
#[cfg_attr(docsrs, doc(cfg(feature = "fft128")))]
pub mod fft128;

/// 64-bit complex number, as in the reference (`src/lib.rs:84`).
pub type c64 = num_complex::Complex64;

/// An error status of the GPU library, returned by the [`gpu`] extensions (the
/// reference-compatible methods panic instead, as the reference does).
#[derive(Clone, Debug, PartialEq, Eq)]
pub struct GpuError {
    /// The `cfft_status` code (negative).
    pub status: i32,
    /// The library's message for it.
    pub message: String,
}

impl core::fmt::Display for GpuError {
    fn fmt(&self, f: &mut core::fmt::Formatter<'_>) -> core::fmt::Result {
        write!(f, "cfft status {}: {}", self.status, self.message)
    }
}

#[cfg(feature = "std")]
impl std::error::Error for GpuError {}

/// `c64` slices as the interleaved (re, im) f64 buffers of the C ABI.
#[inline]
pub(crate) fn as_f64_mut(buf: &mut [c64]) -> *mut f64 {
    bytemuck::cast_slice_mut::<c64, f64>(buf).as_mut_ptr()
}

#[inline]
pub(crate) fn as_f64(buf: &[c64]) -> *const f64 {
    bytemuck::cast_slice::<c64, f64>(buf).as_ptr()
}
