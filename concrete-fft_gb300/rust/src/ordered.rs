//! Ordered FFT: standard order in and out (the reference's `src/ordered.rs`).
//!
//! `Plan::new(n, Method)` chooses one of the eight radix-2/4/8/16 DIF/DIT
//! Stockham algorithms (`Method::Measure` times them all on the GPU and keeps
//! the fastest, with the result kept per GPU model and size); `fwd` and `inv`
//! transform one buffer in place, unnormalised.

use alloc::sync::Arc;
use core::ffi::c_int;
#[cfg(feature = "std")]
use core::time::Duration;

use dyn_stack::{PodStack, SizeOverflow, StackReq};

use crate::ffi;
use crate::{as_f64_mut, c64};

/// Internal FFT algorithm (`src/ordered.rs:22-45`): the discriminant order is the
/// library's `cfft_algo`.
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
#[non_exhaustive]
pub enum FftAlgo {
    /// Decimation in frequency with radix 2
    Dif2,
    /// Decimation in time with radix 2
    Dit2,
    /// Decimation in frequency with radix 4
    Dif4,
    /// Decimation in time with radix 4
    Dit4,
    /// Decimation in frequency with radix 8
    Dif8,
    /// Decimation in time with radix 8
    Dit8,
    /// Decimation in frequency with radix 16
    Dif16,
    /// Decimation in time with radix 16
    Dit16,
}

impl FftAlgo {
    pub(crate) fn to_c(self) -> c_int {
        self as c_int
    }

    pub(crate) fn from_c(v: c_int) -> Self {
        match v {
            0 => FftAlgo::Dif2,
            1 => FftAlgo::Dit2,
            2 => FftAlgo::Dif4,
            3 => FftAlgo::Dit4,
            4 => FftAlgo::Dif8,
            5 => FftAlgo::Dit8,
            6 => FftAlgo::Dif16,
            7 => FftAlgo::Dit16,
            _ => panic!("concrete-fft (GB300): unknown algorithm {v}"),
        }
    }
}

/// Method for selecting the ordered FFT plan (`src/ordered.rs:47-59`).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
#[non_exhaustive]
pub enum Method {
    /// Select the FFT plan by manually providing the underlying algorithm.
    UserProvided(FftAlgo),
    /// Select the FFT plan by timing every algorithm on the GPU for about the given
    /// duration each and keeping the fastest.
    #[cfg(feature = "std")]
    #[cfg_attr(docsrs, doc(cfg(feature = "std")))]
    Measure(Duration),
}

/// The library's plan, destroyed when the last clone of a [`Plan`] goes.
struct Raw(*mut ffi::cfft_ordered_plan);

// SAFETY: the library's plans are immutable after creation and safe to share across
// threads (include/cfft.h).
unsafe impl Send for Raw {}
unsafe impl Sync for Raw {}

impl Drop for Raw {
    fn drop(&mut self) {
        // SAFETY: created by cfft_ordered_plan_create* and destroyed once, here.
        unsafe { ffi::cfft_ordered_plan_destroy(self.0) }
    }
}

/// Ordered FFT plan (`src/ordered.rs:187-373`).  Immutable after creation, so it is
/// `Clone + Send + Sync` like the reference's; its twiddle tables live on the device
/// and are shared by the clones.
#[derive(Clone)]
pub struct Plan {
    raw: Arc<Raw>,
    n: usize,
}

impl core::fmt::Debug for Plan {
    fn fmt(&self, f: &mut core::fmt::Formatter<'_>) -> core::fmt::Result {
        f.debug_struct("Plan")
            .field("algo", &self.algo())
            .field("fft_size", &self.fft_size())
            .finish()
    }
}

impl Plan {
    /// Returns a new FFT plan for the given vector size, selected by the provided method.
    ///
    /// # Panics
    ///
    /// - Panics if `n` is not a power of two, or if it is greater than 1024 (the
    ///   reference's `n.trailing_zeros() < 11`).
    /// - Panics if no usable GB300 (sm_103) device is present.
    #[track_caller]
    pub fn new(n: usize, method: Method) -> Self {
        let mut raw = core::ptr::null_mut();
        // SAFETY: `raw` is a valid out-pointer; the library validates n and the algorithm.
        ffi::check(unsafe {
            match method {
                Method::UserProvided(algo) => ffi::cfft_ordered_plan_create(n, algo.to_c(), &mut raw),
                #[cfg(feature = "std")]
                Method::Measure(duration) => {
                    ffi::cfft_ordered_plan_create_measure(n, duration.as_secs_f64(), &mut raw)
                }
            }
        });
        Self { raw: Arc::new(Raw(raw)), n }
    }

    /// Returns the vector size of the FFT.
    pub fn fft_size(&self) -> usize {
        self.n
    }

    /// Returns the algorithm that's internally used by the FFT.
    pub fn algo(&self) -> FftAlgo {
        // SAFETY: `raw` is a live plan.
        FftAlgo::from_c(unsafe { ffi::cfft_ordered_algo(self.raw.0) })
    }

    /// Returns the size and alignment of the scratch memory needed to perform an FFT.
    /// The GPU keeps its scratch on chip, so nothing is needed from the caller's stack.
    pub fn fft_scratch(&self) -> Result<StackReq, SizeOverflow> {
        Ok(StackReq::empty())
    }

    /// Performs a forward FFT in place, using the provided stack as scratch space
    /// (unused: scratch lives in the GPU's shared memory).
    ///
    /// # Panics
    ///
    /// Panics if the length of `buf` is not equal to the FFT size.
    #[track_caller]
    pub fn fwd(&self, buf: &mut [c64], stack: PodStack) {
        let _ = stack;
        assert_eq!(buf.len(), self.n);
        // SAFETY: `buf` holds n c64 = 2n f64, the length the plan transforms.
        ffi::check(unsafe { ffi::cfft_ordered_fwd_host(self.raw.0, as_f64_mut(buf), 1) });
    }

    /// Performs an inverse FFT in place (unnormalised: `inv(fwd(x)) = n * x`).
    ///
    /// # Panics
    ///
    /// Panics if the length of `buf` is not equal to the FFT size.
    #[track_caller]
    pub fn inv(&self, buf: &mut [c64], stack: PodStack) {
        let _ = stack;
        assert_eq!(buf.len(), self.n);
        // SAFETY: as in `fwd`.
        ffi::check(unsafe { ffi::cfft_ordered_inv_host(self.raw.0, as_f64_mut(buf), 1) });
    }

    /// Forward FFTs of `batch` buffers stored back to back in host memory, in one call.
    /// Page-locked memory is transformed in place by the kernel across the host link.
    #[track_caller]
    pub fn fwd_batch(&self, bufs: &mut [c64]) {
        assert_eq!(bufs.len() % self.n, 0);
        // SAFETY: `bufs` holds a whole number of transforms.
        ffi::check(unsafe { ffi::cfft_ordered_fwd_host(self.raw.0, as_f64_mut(bufs), bufs.len() / self.n) });
    }

    /// Inverse FFTs of `batch` buffers stored back to back in host memory, in one call.
    #[track_caller]
    pub fn inv_batch(&self, bufs: &mut [c64]) {
        assert_eq!(bufs.len() % self.n, 0);
        // SAFETY: `bufs` holds a whole number of transforms.
        ffi::check(unsafe { ffi::cfft_ordered_inv_host(self.raw.0, as_f64_mut(bufs), bufs.len() / self.n) });
    }

    pub(crate) fn raw(&self) -> *const ffi::cfft_ordered_plan {
        self.raw.0
    }
}
