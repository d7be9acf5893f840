//! Unordered FFT: standard order in, a plan-specific permuted order out (the
//! reference's `src/unordered.rs`).
//!
//! The forward transform leaves its output in the permuted order of
//! `bit_rev_twice(log2 n, log2 base_n, i)`, which depends only on `(n, base_n)`;
//! the inverse takes that order back to standard order, unnormalised.  The
//! serde helpers convert between the permuted order and the standard order on
//! the GPU (the library's wire-format kernels) and hand the standard-order
//! sequence to the serializer, element for element as the reference does.

use alloc::sync::Arc;
#[cfg(feature = "serde")]
use alloc::vec::Vec;
use core::ffi::c_int;
#[cfg(feature = "std")]
use core::time::Duration;

use dyn_stack::{PodStack, SizeOverflow, StackReq};

use crate::ffi;
use crate::ordered::FftAlgo;
use crate::{as_f64_mut, c64};

/// Method for selecting the unordered FFT plan (`src/unordered.rs:524-537`).
#[derive(Clone, Copy, Debug)]
pub enum Method {
    /// Select the FFT plan by manually providing the underlying algorithm: the
    /// internal ordered plan's size and algorithm.
    UserProvided { base_algo: FftAlgo, base_n: usize },
    /// Select the FFT plan by timing the candidates on the GPU (bases 512 and 1024
    /// with their fastest ordered algorithm, or every ordered algorithm for n <= 256,
    /// as `src/unordered.rs:553-640`), about the given duration each.
    #[cfg(feature = "std")]
    #[cfg_attr(docsrs, doc(cfg(feature = "std")))]
    Measure(Duration),
}

struct Raw(*mut ffi::cfft_unordered_plan);

// SAFETY: the library's plans are immutable after creation and safe to share across
// threads (include/cfft.h).
unsafe impl Send for Raw {}
unsafe impl Sync for Raw {}

impl Drop for Raw {
    fn drop(&mut self) {
        // SAFETY: created by cfft_unordered_plan_create* and destroyed once, here.
        unsafe { ffi::cfft_unordered_plan_destroy(self.0) }
    }
}

/// Unordered FFT plan (`src/unordered.rs:496-1036`).  `Clone + Send + Sync`; the
/// twiddle tables live on the device and are shared by the clones.
#[derive(Clone)]
pub struct Plan {
    raw: Arc<Raw>,
    n: usize,
    base_algo: FftAlgo,
    base_n: usize,
}

impl core::fmt::Debug for Plan {
    fn fmt(&self, f: &mut core::fmt::Formatter<'_>) -> core::fmt::Result {
        f.debug_struct("Plan")
            .field("base_algo", &self.base_algo)
            .field("base_size", &self.base_n)
            .field("fft_size", &self.n)
            .finish()
    }
}

impl Plan {
    /// Returns a new FFT plan for the given vector size, selected by the provided method.
    ///
    /// # Panics
    ///
    /// - Panics if `n` is not a power of two.
    /// - If the method is user-provided, panics if `base_n` is not a power of two, is
    ///   greater than `n` or 1024, or is below 32 while `n` is larger (the reference's
    ///   assertions, `src/unordered.rs:660-670`).
    /// - Panics if no usable GB300 (sm_103) device is present.
    #[track_caller]
    pub fn new(n: usize, method: Method) -> Self {
        let mut raw = core::ptr::null_mut();
        // SAFETY: `raw` is a valid out-pointer; the library validates the sizes.
        ffi::check(unsafe {
            match method {
                Method::UserProvided { base_algo, base_n } => {
                    ffi::cfft_unordered_plan_create(n, base_algo.to_c(), base_n, &mut raw)
                }
                #[cfg(feature = "std")]
                Method::Measure(duration) => {
                    ffi::cfft_unordered_plan_create_measure(n, duration.as_secs_f64(), &mut raw)
                }
            }
        });
        let mut algo: c_int = 0;
        let mut base_n = 0usize;
        // SAFETY: `raw` is a live plan; the out-pointers are valid.
        unsafe { ffi::cfft_unordered_algo(raw, &mut algo, &mut base_n) };
        Self { raw: Arc::new(Raw(raw)), n, base_algo: FftAlgo::from_c(algo), base_n }
    }

    /// Returns the vector size of the FFT.
    pub fn fft_size(&self) -> usize {
        self.n
    }

    /// Returns the algorithm and size of the internal ordered FFT plan.
    pub fn algo(&self) -> (FftAlgo, usize) {
        (self.base_algo, self.base_n)
    }

    /// Returns the size and alignment of the scratch memory needed to perform an FFT:
    /// nothing from the caller (the GPU keeps its scratch on chip or in the plan).
    pub fn fft_scratch(&self) -> Result<StackReq, SizeOverflow> {
        Ok(StackReq::empty())
    }

    /// Performs a forward FFT in place; the output is in the plan's permuted order.
    ///
    /// # Panics
    ///
    /// Panics if the length of `buf` is not equal to the FFT size.
    #[track_caller]
    pub fn fwd(&self, buf: &mut [c64], stack: PodStack) {
        let _ = stack;
        assert_eq!(buf.len(), self.n);
        // SAFETY: `buf` holds exactly one transform.
        ffi::check(unsafe { ffi::cfft_unordered_fwd_host(self.raw.0, as_f64_mut(buf), 1) });
    }

    /// Performs a forward FFT of the monomial `X^degree` into `buf`, in the permuted
    /// order (`src/unordered.rs:844-900`).
    ///
    /// # Panics
    ///
    /// Panics if the length of `buf` is not equal to the FFT size, or if `degree` is
    /// not below it.
    #[track_caller]
    pub fn fwd_monomial(&self, degree: usize, buf: &mut [c64]) {
        assert_eq!(buf.len(), self.n);
        assert!(degree < self.n);
        // SAFETY: `buf` holds exactly one transform.
        ffi::check(unsafe { ffi::cfft_unordered_fwd_monomial_host(self.raw.0, degree, as_f64_mut(buf)) });
    }

    /// Performs an inverse FFT in place: permuted order in, standard order out,
    /// unnormalised.
    ///
    /// # Panics
    ///
    /// Panics if the length of `buf` is not equal to the FFT size.
    #[track_caller]
    pub fn inv(&self, buf: &mut [c64], stack: PodStack) {
        let _ = stack;
        assert_eq!(buf.len(), self.n);
        // SAFETY: `buf` holds exactly one transform.
        ffi::check(unsafe { ffi::cfft_unordered_inv_host(self.raw.0, as_f64_mut(buf), 1) });
    }

    /// Forward FFTs of buffers stored back to back in host memory, in one call.
    #[track_caller]
    pub fn fwd_batch(&self, bufs: &mut [c64]) {
        assert_eq!(bufs.len() % self.n, 0);
        // SAFETY: `bufs` holds a whole number of transforms.
        ffi::check(unsafe { ffi::cfft_unordered_fwd_host(self.raw.0, as_f64_mut(bufs), bufs.len() / self.n) });
    }

    /// Inverse FFTs of buffers stored back to back in host memory, in one call.
    #[track_caller]
    pub fn inv_batch(&self, bufs: &mut [c64]) {
        assert_eq!(bufs.len() % self.n, 0);
        // SAFETY: `bufs` holds a whole number of transforms.
        ffi::check(unsafe { ffi::cfft_unordered_inv_host(self.raw.0, as_f64_mut(bufs), bufs.len() / self.n) });
    }

    /// Serializes a buffer of Fourier-domain data held in the plan's permuted order as
    /// a sequence of `n` c64 in the standard order (`src/unordered.rs:942-970`).
    ///
    /// # Panics
    ///
    /// Panics if the length of `buf` is not equal to the FFT size.
    #[cfg(feature = "serde")]
    #[cfg_attr(docsrs, doc(cfg(feature = "serde")))]
    pub fn serialize_fourier_buffer<S: serde::Serializer>(
        &self,
        serializer: S,
        buf: &[c64],
    ) -> Result<S::Ok, S::Error> {
        use serde::ser::SerializeSeq;

        assert_eq!(buf.len(), self.n);
        let mut standard = alloc::vec![c64::new(0.0, 0.0); self.n];
        // SAFETY: both buffers hold exactly one transform.
        ffi::check(unsafe {
            ffi::cfft_unordered_to_standard_host(self.raw.0, crate::as_f64(buf), as_f64_mut(&mut standard), 1)
        });
        let mut seq = serializer.serialize_seq(Some(self.n))?;
        for z in &standard {
            seq.serialize_element(z)?;
        }
        seq.end()
    }

    /// Deserializes a standard-order sequence of `n` c64 into `buf`, in the plan's
    /// permuted order (`src/unordered.rs:972-1036`).  A sequence of another length is
    /// refused with the deserializer's `invalid_length` error, as in the reference.
    ///
    /// # Panics
    ///
    /// Panics if the length of `buf` is not equal to the FFT size.
    #[cfg(feature = "serde")]
    #[cfg_attr(docsrs, doc(cfg(feature = "serde")))]
    pub fn deserialize_fourier_buffer<'de, D: serde::Deserializer<'de>>(
        &self,
        deserializer: D,
        buf: &mut [c64],
    ) -> Result<(), D::Error> {
        use serde::de::{SeqAccess, Visitor};

        assert_eq!(buf.len(), self.n);

        struct Standard {
            n: usize,
        }

        impl<'de> Visitor<'de> for Standard {
            type Value = Vec<c64>;

            fn expecting(&self, f: &mut core::fmt::Formatter) -> core::fmt::Result {
                write!(f, "a sequence of {} 64-bit complex numbers", self.n)
            }

            fn visit_seq<A: SeqAccess<'de>>(self, mut seq: A) -> Result<Vec<c64>, A::Error> {
                let mut values = Vec::with_capacity(self.n);
                let mut count = 0usize;
                while let Some(z) = seq.next_element::<c64>()? {
                    if count < self.n {
                        values.push(z);
                    }
                    count += 1;
                }
                if count != self.n {
                    return Err(serde::de::Error::invalid_length(count, &self));
                }
                Ok(values)
            }
        }

        let standard = deserializer.deserialize_seq(Standard { n: self.n })?;
        // SAFETY: both buffers hold exactly one transform.
        ffi::check(unsafe {
            ffi::cfft_unordered_from_standard_host(self.raw.0, crate::as_f64(&standard), as_f64_mut(buf), 1)
        });
        Ok(())
    }

    pub(crate) fn raw(&self) -> *const ffi::cfft_unordered_plan {
        self.raw.0
    }
}
