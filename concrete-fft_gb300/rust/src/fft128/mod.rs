//! 128-bit (double-double) negacyclic FFT (the reference's `src/fft128/mod.rs`).
//!
//! Data are split into four f64 arrays (re0, re1, im0, im1): the high and low
//! words of the real and imaginary parts.  The forward transform leaves its
//! output in bit-reversed order; the inverse takes it back, unnormalised.  The
//! transforms run on the GPU (compensated double-double butterflies); results are
//! bit-identical to the reference's.

pub mod f128_ops;

use alloc::sync::Arc;

use crate::ffi;

/// 128-bit floating point number: the unevaluated sum `self.0 + self.1`.
#[allow(non_camel_case_types)]
#[derive(Copy, Clone, Debug)]
#[repr(C)]
pub struct f128(pub f64, pub f64);

#[track_caller]
fn same_lengths(n: usize, arrays: [usize; 4]) {
    for len in arrays {
        assert_eq!(len, n);
    }
}

/// Fills positions `1..n` of the four twiddle arrays of length `n` with the
/// negacyclic twiddles in bit-reversed order (`src/fft128/mod.rs:1804-1828`);
/// position 0 is left as it is.
#[doc(hidden)]
#[track_caller]
pub fn init_negacyclic_twiddles(
    twid_re0: &mut [f64],
    twid_re1: &mut [f64],
    twid_im0: &mut [f64],
    twid_im1: &mut [f64],
) {
    let n = twid_re0.len();
    same_lengths(n, [twid_re0.len(), twid_re1.len(), twid_im0.len(), twid_im1.len()]);
    if n == 0 {
        return;
    }
    // SAFETY: four host arrays of n f64.
    ffi::check(unsafe {
        ffi::cfft_f128_init_negacyclic_twiddles(
            n,
            twid_re0.as_mut_ptr(),
            twid_re1.as_mut_ptr(),
            twid_im0.as_mut_ptr(),
            twid_im1.as_mut_ptr(),
        )
    });
}

#[track_caller]
fn negacyclic(
    fwd: bool,
    data: [&mut [f64]; 4],
    twid: [&[f64]; 4],
) {
    let n = twid[0].len();
    same_lengths(n, [twid[0].len(), twid[1].len(), twid[2].len(), twid[3].len()]);
    same_lengths(n, [data[0].len(), data[1].len(), data[2].len(), data[3].len()]);
    let [re0, re1, im0, im1] = data;
    // SAFETY: eight host arrays of n f64; the library transforms the four data arrays in place.
    ffi::check(unsafe {
        let f = if fwd { ffi::cfft_f128_negacyclic_fwd_host } else { ffi::cfft_f128_negacyclic_inv_host };
        f(
            n,
            1,
            re0.as_mut_ptr(),
            re1.as_mut_ptr(),
            im0.as_mut_ptr(),
            im1.as_mut_ptr(),
            twid[0].as_ptr(),
            twid[1].as_ptr(),
            twid[2].as_ptr(),
            twid[3].as_ptr(),
        )
    });
}

/// Forward negacyclic FFT with caller-owned twiddles (`src/fft128/mod.rs:1040-1071`).
#[doc(hidden)]
#[track_caller]
#[allow(clippy::too_many_arguments)]
pub fn negacyclic_fwd_fft(
    data_re0: &mut [f64],
    data_re1: &mut [f64],
    data_im0: &mut [f64],
    data_im1: &mut [f64],
    twid_re0: &[f64],
    twid_re1: &[f64],
    twid_im0: &[f64],
    twid_im1: &[f64],
) {
    negacyclic(true, [data_re0, data_re1, data_im0, data_im1], [twid_re0, twid_re1, twid_im0, twid_im1]);
}

/// Inverse negacyclic FFT with caller-owned twiddles, unnormalised
/// (`src/fft128/mod.rs:1072-1103`).
#[doc(hidden)]
#[track_caller]
#[allow(clippy::too_many_arguments)]
pub fn negacyclic_inv_fft(
    data_re0: &mut [f64],
    data_re1: &mut [f64],
    data_im0: &mut [f64],
    data_im1: &mut [f64],
    twid_re0: &[f64],
    twid_re1: &[f64],
    twid_im0: &[f64],
    twid_im1: &[f64],
) {
    negacyclic(false, [data_re0, data_re1, data_im0, data_im1], [twid_re0, twid_re1, twid_im0, twid_im1]);
}

/// The reference's per-instruction-set entry points (`src/fft128/mod.rs:351-1792`)
/// give equal results; here they are all the GPU transform.
#[doc(hidden)]
#[allow(clippy::too_many_arguments)]
pub fn negacyclic_fwd_fft_scalar(
    data_re0: &mut [f64],
    data_re1: &mut [f64],
    data_im0: &mut [f64],
    data_im1: &mut [f64],
    twid_re0: &[f64],
    twid_re1: &[f64],
    twid_im0: &[f64],
    twid_im1: &[f64],
) {
    negacyclic_fwd_fft(data_re0, data_re1, data_im0, data_im1, twid_re0, twid_re1, twid_im0, twid_im1);
}

#[doc(hidden)]
#[allow(clippy::too_many_arguments)]
pub fn negacyclic_inv_fft_scalar(
    data_re0: &mut [f64],
    data_re1: &mut [f64],
    data_im0: &mut [f64],
    data_im1: &mut [f64],
    twid_re0: &[f64],
    twid_re1: &[f64],
    twid_im0: &[f64],
    twid_im1: &[f64],
) {
    negacyclic_inv_fft(data_re0, data_re1, data_im0, data_im1, twid_re0, twid_re1, twid_im0, twid_im1);
}

#[cfg(any(target_arch = "x86", target_arch = "x86_64"))]
#[doc(hidden)]
#[allow(clippy::too_many_arguments)]
pub fn negacyclic_fwd_fft_avxfma(
    simd: pulp::x86::V3,
    data_re0: &mut [f64],
    data_re1: &mut [f64],
    data_im0: &mut [f64],
    data_im1: &mut [f64],
    twid_re0: &[f64],
    twid_re1: &[f64],
    twid_im0: &[f64],
    twid_im1: &[f64],
) {
    let _ = simd;
    negacyclic_fwd_fft(data_re0, data_re1, data_im0, data_im1, twid_re0, twid_re1, twid_im0, twid_im1);
}

#[cfg(any(target_arch = "x86", target_arch = "x86_64"))]
#[doc(hidden)]
#[allow(clippy::too_many_arguments)]
pub fn negacyclic_inv_fft_avxfma(
    simd: pulp::x86::V3,
    data_re0: &mut [f64],
    data_re1: &mut [f64],
    data_im0: &mut [f64],
    data_im1: &mut [f64],
    twid_re0: &[f64],
    twid_re1: &[f64],
    twid_im0: &[f64],
    twid_im1: &[f64],
) {
    let _ = simd;
    negacyclic_inv_fft(data_re0, data_re1, data_im0, data_im1, twid_re0, twid_re1, twid_im0, twid_im1);
}

#[cfg(all(feature = "nightly", any(target_arch = "x86", target_arch = "x86_64")))]
#[doc(hidden)]
#[allow(clippy::too_many_arguments)]
pub fn negacyclic_fwd_fft_avx512(
    simd: pulp::x86::V4,
    data_re0: &mut [f64],
    data_re1: &mut [f64],
    data_im0: &mut [f64],
    data_im1: &mut [f64],
    twid_re0: &[f64],
    twid_re1: &[f64],
    twid_im0: &[f64],
    twid_im1: &[f64],
) {
    let _ = simd;
    negacyclic_fwd_fft(data_re0, data_re1, data_im0, data_im1, twid_re0, twid_re1, twid_im0, twid_im1);
}

#[cfg(all(feature = "nightly", any(target_arch = "x86", target_arch = "x86_64")))]
#[doc(hidden)]
#[allow(clippy::too_many_arguments)]
pub fn negacyclic_inv_fft_avx512(
    simd: pulp::x86::V4,
    data_re0: &mut [f64],
    data_re1: &mut [f64],
    data_im0: &mut [f64],
    data_im1: &mut [f64],
    twid_re0: &[f64],
    twid_re1: &[f64],
    twid_im0: &[f64],
    twid_im1: &[f64],
) {
    let _ = simd;
    negacyclic_inv_fft(data_re0, data_re1, data_im0, data_im1, twid_re0, twid_re1, twid_im0, twid_im1);
}

struct Raw(*mut ffi::cfft_f128_plan);

// SAFETY: the library's plans are immutable after creation and safe to share across
// threads (include/cfft.h).
unsafe impl Send for Raw {}
unsafe impl Sync for Raw {}

impl Drop for Raw {
    fn drop(&mut self) {
        // SAFETY: created by cfft_f128_plan_create and destroyed once, here.
        unsafe { ffi::cfft_f128_plan_destroy(self.0) }
    }
}

/// 128-bit negacyclic FFT plan (`src/fft128/mod.rs:1830-1960`); its twiddles live on
/// the device and are shared by the clones.
#[derive(Clone)]
pub struct Plan {
    raw: Arc<Raw>,
    n: usize,
}

impl core::fmt::Debug for Plan {
    fn fmt(&self, f: &mut core::fmt::Formatter<'_>) -> core::fmt::Result {
        f.debug_struct("Plan").field("fft_size", &self.n).finish()
    }
}

impl Plan {
    /// Returns a new negacyclic FFT plan for the given vector size.
    ///
    /// # Panics
    ///
    /// Panics if `n` is not a power of two, or if it is less than 32.
    #[track_caller]
    pub fn new(n: usize) -> Self {
        assert!(n.is_power_of_two());
        assert!(n >= 32);
        let mut raw = core::ptr::null_mut();
        // SAFETY: `raw` is a valid out-pointer.
        ffi::check(unsafe { ffi::cfft_f128_plan_create(n, &mut raw) });
        Self { raw: Arc::new(Raw(raw)), n }
    }

    /// Returns the vector size of the FFT.
    pub fn fft_size(&self) -> usize {
        self.n
    }

    /// Performs a forward negacyclic FFT in place.
    ///
    /// # Panics
    ///
    /// Panics if any buffer's length is not equal to the FFT size.
    #[track_caller]
    pub fn fwd(&self, buf_re0: &mut [f64], buf_re1: &mut [f64], buf_im0: &mut [f64], buf_im1: &mut [f64]) {
        same_lengths(self.n, [buf_re0.len(), buf_re1.len(), buf_im0.len(), buf_im1.len()]);
        // SAFETY: four host arrays of n f64.
        ffi::check(unsafe {
            ffi::cfft_f128_fwd_host(
                self.raw.0,
                buf_re0.as_mut_ptr(),
                buf_re1.as_mut_ptr(),
                buf_im0.as_mut_ptr(),
                buf_im1.as_mut_ptr(),
                1,
            )
        });
    }

    /// Performs an inverse negacyclic FFT in place, unnormalised.
    ///
    /// # Panics
    ///
    /// Panics if any buffer's length is not equal to the FFT size.
    #[track_caller]
    pub fn inv(&self, buf_re0: &mut [f64], buf_re1: &mut [f64], buf_im0: &mut [f64], buf_im1: &mut [f64]) {
        same_lengths(self.n, [buf_re0.len(), buf_re1.len(), buf_im0.len(), buf_im1.len()]);
        // SAFETY: four host arrays of n f64.
        ffi::check(unsafe {
            ffi::cfft_f128_inv_host(
                self.raw.0,
                buf_re0.as_mut_ptr(),
                buf_re1.as_mut_ptr(),
                buf_im0.as_mut_ptr(),
                buf_im1.as_mut_ptr(),
                1,
            )
        });
    }

    pub(crate) fn raw(&self) -> *const ffi::cfft_f128_plan {
        self.raw.0
    }
}
