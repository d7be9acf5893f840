//! Double-double arithmetic on the host (the reference's `src/fft128/f128_ops.rs`).
//!
//! A value is the unevaluated sum `self.0 + self.1` of two f64.  The operations are
//! the classic error-free transformations (Knuth's TwoSum, Dekker's Fast2Sum, the
//! FMA product error) composed in the same order as the reference, so every
//! result is bit-identical to the reference's on every target: Rust never fuses
//! a multiply and an add unless `mul_add` is written, which only the product
//! error term does.  The same operations run on the GPU in the library's fft128
//! kernels.  `sincospi` is the library's host routine (`cfft_f128_sincospi`).

use super::f128;
use crate::ffi;
use core::cmp::Ordering;
use core::ops::{Add, AddAssign, Div, DivAssign, Mul, MulAssign, Neg, Sub, SubAssign};

// ---- error-free transformations (src/fft128/f128_ops.rs:3-40)

/// s + e = a + b exactly, for |a| >= |b| (Fast2Sum).
#[inline(always)]
fn fast_two_sum(a: f64, b: f64) -> (f64, f64) {
    let s = a + b;
    let t = s - a;
    (s, b - t)
}

/// s + e = a + b exactly (TwoSum).
#[inline(always)]
fn two_sum(a: f64, b: f64) -> (f64, f64) {
    let s = a + b;
    let b_virtual = s - a;
    let a_virtual = s - b_virtual;
    let a_err = a - a_virtual;
    let b_err = b - b_virtual;
    (s, a_err + b_err)
}

/// s + e = a - b exactly.
#[inline(always)]
fn two_diff(a: f64, b: f64) -> (f64, f64) {
    let s = a - b;
    let b_virtual = s - a;
    let a_virtual = s - b_virtual;
    let a_err = a - a_virtual;
    let b_err = b + b_virtual;
    (s, a_err - b_err)
}

/// p + e = a * b exactly (one FMA).
#[inline(always)]
fn two_prod(a: f64, b: f64) -> (f64, f64) {
    let p = a * b;
    (p, f64::mul_add(a, b, -p))
}

/// Renormalises (hi, lo + extra) through Fast2Sum.
#[inline(always)]
fn renorm(hi: f64, lo: f64) -> f128 {
    let (h, l) = fast_two_sum(hi, lo);
    f128(h, l)
}

impl f128 {
    /// `a + b` of two f64, exact.
    #[inline(always)]
    pub fn add_f64_f64(a: f64, b: f64) -> Self {
        let (s, e) = two_sum(a, b);
        f128(s, e)
    }

    #[inline(always)]
    pub fn add_f128_f64(a: f128, b: f64) -> Self {
        let (s, e) = two_sum(a.0, b);
        renorm(s, e + a.1)
    }

    #[inline(always)]
    pub fn add_f64_f128(a: f64, b: f128) -> Self {
        Self::add_f128_f64(b, a)
    }

    /// The faster "estimate" sum: the low parts are added without their error term.
    #[inline(always)]
    pub fn add_estimate_f128_f128(a: f128, b: f128) -> Self {
        let (s, e) = two_sum(a.0, b.0);
        let lo = a.1 + b.1;
        renorm(s, e + lo)
    }

    #[inline(always)]
    pub fn add_f128_f128(a: f128, b: f128) -> Self {
        let (s, e) = two_sum(a.0, b.0);
        let (t, f) = two_sum(a.1, b.1);
        let r = renorm(s, e + t);
        renorm(r.0, r.1 + f)
    }

    #[inline(always)]
    pub fn sub_f64_f64(a: f64, b: f64) -> Self {
        let (s, e) = two_diff(a, b);
        f128(s, e)
    }

    #[inline(always)]
    pub fn sub_f128_f64(a: f128, b: f64) -> Self {
        let (s, e) = two_diff(a.0, b);
        renorm(s, e + a.1)
    }

    #[inline(always)]
    pub fn sub_f64_f128(a: f64, b: f128) -> Self {
        let (s, e) = two_diff(a, b.0);
        renorm(s, e - b.1)
    }

    #[inline(always)]
    pub fn sub_estimate_f128_f128(a: f128, b: f128) -> Self {
        let (s, e) = two_diff(a.0, b.0);
        let e = e + a.1;
        renorm(s, e - b.1)
    }

    #[inline(always)]
    pub fn sub_f128_f128(a: f128, b: f128) -> Self {
        let (s, e) = two_diff(a.0, b.0);
        let (t, f) = two_diff(a.1, b.1);
        let r = renorm(s, e + t);
        renorm(r.0, r.1 + f)
    }

    #[inline(always)]
    pub fn mul_f64_f64(a: f64, b: f64) -> Self {
        let (p, e) = two_prod(a, b);
        f128(p, e)
    }

    #[inline(always)]
    pub fn mul_f128_f64(a: f128, b: f64) -> Self {
        let (p, e) = two_prod(a.0, b);
        let cross = a.1 * b;
        renorm(p, e + cross)
    }

    #[inline(always)]
    pub fn mul_f64_f128(a: f64, b: f128) -> Self {
        Self::mul_f128_f64(b, a)
    }

    #[inline(always)]
    pub fn mul_f128_f128(a: f128, b: f128) -> Self {
        let (p, e) = two_prod(a.0, b.0);
        let c1 = a.0 * b.1;
        let c2 = a.1 * b.0;
        let cross = c1 + c2;
        renorm(p, e + cross)
    }

    /// `self * self`.
    #[inline(always)]
    pub fn sqr(self) -> Self {
        let (p, e) = two_prod(self.0, self.0);
        let cross = self.0 * self.1;
        let cross2 = 2.0 * cross;
        renorm(p, e + cross2)
    }

    /// `a / b` of two f64 to double-double accuracy (one correction step).
    #[inline(always)]
    pub fn div_f64_f64(a: f64, b: f64) -> Self {
        let q1 = a / b;
        let (p, pe) = two_prod(q1, b);
        let (s, se) = two_diff(a, p);
        let e = se - pe;
        let rem = s + e;
        let q2 = rem / b;
        renorm(q1, q2)
    }

    #[inline(always)]
    pub fn div_f128_f64(a: f128, b: f64) -> Self {
        let q1 = a.0 / b;
        let (p, pe) = two_prod(q1, b);
        let (s, se) = two_diff(a.0, p);
        let e = se + a.1;
        let e = e - pe;
        let rem = s + e;
        let q2 = rem / b;
        renorm(q1, q2)
    }

    #[inline(always)]
    pub fn div_f64_f128(a: f64, b: f128) -> Self {
        Self::div_f128_f128(f128(a, 0.0), b)
    }

    /// The faster "estimate" quotient: one correction step.
    #[inline(always)]
    pub fn div_estimate_f128_f128(a: f128, b: f128) -> Self {
        let q1 = a.0 / b.0;
        let r = Self::mul_f128_f64(b, q1);
        let (s, se) = two_diff(a.0, r.0);
        let e = se - r.1;
        let e = e + a.1;
        let rem = s + e;
        let q2 = rem / b.0;
        renorm(q1, q2)
    }

    /// `a / b` to double-double accuracy (two correction steps).
    #[inline(always)]
    pub fn div_f128_f128(a: f128, b: f128) -> Self {
        let q1 = a.0 / b.0;
        let r = Self::sub_f128_f128(a, Self::mul_f128_f64(b, q1));
        let q2 = r.0 / b.0;
        let r = Self::sub_f128_f128(r, Self::mul_f64_f128(q2, b));
        let q3 = r.0 / b.0;
        let q = renorm(q1, q2);
        Self::add_f128_f64(q, q3)
    }

    /// The high part.
    #[inline(always)]
    pub fn to_f64(self) -> f64 {
        self.0
    }

    /// True when either part is NaN.
    #[inline(always)]
    pub fn is_nan(self) -> bool {
        self.0.is_nan() || self.1.is_nan()
    }

    /// The absolute value (sign of the high part).
    #[inline(always)]
    pub fn abs(self) -> Self {
        if self.0 < 0.0 {
            -self
        } else {
            self
        }
    }

    /// `(sin(pi * self), cos(pi * self))`, bit-identical to the reference
    /// (`src/fft128/f128_ops.rs:534-575`), computed by the library's host routine.
    ///
    /// # Panics
    ///
    /// Panics if `self` is above 1 or below -1, as the reference does.
    #[track_caller]
    pub fn sincospi(self) -> (Self, Self) {
        if self > 1.0 || self < -1.0 {
            panic!("only inputs in [-1, 1] are currently supported, received: {self:?}");
        }
        let mut s = [0.0f64; 2];
        let mut c = [0.0f64; 2];
        // SAFETY: two valid out-arrays of two f64 each.
        ffi::check(unsafe { ffi::cfft_f128_sincospi(self.0, self.1, s.as_mut_ptr(), c.as_mut_ptr()) });
        (f128(s[0], s[1]), f128(c[0], c[1]))
    }

    /// pi to double-double precision (the reference's literal, `src/fft128/f128_ops.rs:580`).
    pub const PI: Self = f128(3.141592653589793, 1.2246467991473532e-16);
}

impl From<f64> for f128 {
    #[inline(always)]
    fn from(value: f64) -> Self {
        f128(value, 0.0)
    }
}

impl Neg for f128 {
    type Output = f128;
    #[inline(always)]
    fn neg(self) -> f128 {
        f128(-self.0, -self.1)
    }
}

/// The binary operators for every mix of f128 and f64 operands, each forwarding to the
/// named operation, plus the compound assignments (`src/fft128/f128_ops.rs:55-217`).
macro_rules! binary_ops {
    ($Op:ident, $op:ident, $OpAssign:ident, $op_assign:ident, $qq:ident, $qd:ident, $dq:ident) => {
        impl $Op<f128> for f128 {
            type Output = f128;
            #[inline(always)]
            fn $op(self, rhs: f128) -> f128 {
                f128::$qq(self, rhs)
            }
        }
        impl $Op<f64> for f128 {
            type Output = f128;
            #[inline(always)]
            fn $op(self, rhs: f64) -> f128 {
                f128::$qd(self, rhs)
            }
        }
        impl $Op<f128> for f64 {
            type Output = f128;
            #[inline(always)]
            fn $op(self, rhs: f128) -> f128 {
                f128::$dq(self, rhs)
            }
        }
        impl $OpAssign<f128> for f128 {
            #[inline(always)]
            fn $op_assign(&mut self, rhs: f128) {
                *self = f128::$qq(*self, rhs);
            }
        }
        impl $OpAssign<f64> for f128 {
            #[inline(always)]
            fn $op_assign(&mut self, rhs: f64) {
                *self = f128::$qd(*self, rhs);
            }
        }
    };
}

binary_ops!(Add, add, AddAssign, add_assign, add_f128_f128, add_f128_f64, add_f64_f128);
binary_ops!(Sub, sub, SubAssign, sub_assign, sub_f128_f128, sub_f128_f64, sub_f64_f128);
binary_ops!(Mul, mul, MulAssign, mul_assign, mul_f128_f128, mul_f128_f64, mul_f64_f128);
binary_ops!(Div, div, DivAssign, div_assign, div_f128_f128, div_f128_f64, div_f64_f128);

// ---- comparisons: equality of both parts, order lexicographic on (hi, lo) and
// unordered when a compared part is NaN (src/fft128/f128_ops.rs:228-275)

impl PartialEq<f128> for f128 {
    #[inline(always)]
    fn eq(&self, other: &f128) -> bool {
        self.0 == other.0 && self.1 == other.1
    }
}
impl PartialEq<f64> for f128 {
    #[inline(always)]
    fn eq(&self, other: &f64) -> bool {
        *self == f128(*other, 0.0)
    }
}
impl PartialEq<f128> for f64 {
    #[inline(always)]
    fn eq(&self, other: &f128) -> bool {
        f128(*self, 0.0) == *other
    }
}

impl PartialOrd<f128> for f128 {
    #[inline(always)]
    fn partial_cmp(&self, other: &f128) -> Option<Ordering> {
        match self.0.partial_cmp(&other.0) {
            Some(Ordering::Equal) => self.1.partial_cmp(&other.1),
            hi => hi,
        }
    }
}
impl PartialOrd<f64> for f128 {
    #[inline(always)]
    fn partial_cmp(&self, other: &f64) -> Option<Ordering> {
        self.partial_cmp(&f128(*other, 0.0))
    }
}
impl PartialOrd<f128> for f64 {
    #[inline(always)]
    fn partial_cmp(&self, other: &f128) -> Option<Ordering> {
        f128(*self, 0.0).partial_cmp(other)
    }
}
