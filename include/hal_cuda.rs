//! `hal::cuda`: the GB300 backend of `libhalcuda.so` behind the crate's `hal::Backend` trait
//! (cyclosubfield-dbfv/src/hal/mod.rs:108-350), so that `ring`, `bfv`, `dbfv` and `bootstrap` run
//! unchanged on the GPU: `RingContext::new(CudaBackend::new(0), field, ...)`.
//!
//! To use it, copy this file to `cyclosubfield-dbfv/src/hal/cuda.rs`, add `pub mod cuda;` to
//! `src/hal/mod.rs`, and link the library (`cargo:rustc-link-lib=halcuda` and a search path in
//! `build.rs`). Every method maps one to one onto the `hc_*` entry point of include/halcuda.h that
//! cites it; the tensor views are the same strided 4-D views as the CPU backend's
//! (src/hal/cpu.rs:66-296), only their memory is device memory. A non-zero status panics with the
//! library's message, like the CPU backend's `assert!`s (`panic = "abort"`, Cargo.toml:28).
//! Work is asynchronous on the context's stream; `hal_import` / `hal_export` return when the host
//! slice may be reused, so the crate's sequential semantics hold.
#![allow(clippy::missing_safety_doc)]

use std::ffi::{c_char, c_int, c_void, CStr};
use std::marker::PhantomData;
use std::ops::{Bound, RangeBounds};
use std::sync::Arc;

use super::{
    Backend, DIMS, DataDim, Dim, Moduli, TensorI128Mut, TensorI128Ref, TensorI64Mut, TensorI64Ref, TensorMut,
    TensorOwned, TensorRef,
};

// ------------------------------------------------------------------------------------------
// FFI (include/halcuda.h)
// ------------------------------------------------------------------------------------------

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct HcView {
    ptr: *mut c_void,
    shape: [i64; 4],
    strides: [i64; 4],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub struct HcModulus {
    n: i64,
    neg_inv_n: i64,
    r2_mod_n: i64,
    r3_mod_n: i64,
}

#[repr(C)]
pub struct HcContext {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct HcNttPlan {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct HcPermPlan {
    _opaque: [u8; 0],
}

const HC_DIM2: c_int = 2;
const HC_DIM3: c_int = 3;

#[link(name = "halcuda")]
extern "C" {
    fn hc_last_error() -> *const c_char;
    fn hc_context_create(device: c_int, out: *mut *mut HcContext) -> c_int;
    fn hc_context_destroy(ctx: *mut HcContext) -> c_int;
    fn hc_allocate_i64(ctx: *mut HcContext, shape: *const i64, out: *mut *mut c_void) -> c_int;
    fn hc_allocate_i128(ctx: *mut HcContext, shape: *const i64, out: *mut *mut c_void) -> c_int;
    fn hc_free(ctx: *mut HcContext, ptr: *mut c_void) -> c_int;
    fn hc_import(ctx: *mut HcContext, dst: HcView, src: *const i64, len: usize) -> c_int;
    fn hc_export(ctx: *mut HcContext, src: HcView, dst: *mut i64, len: usize) -> c_int;
    fn hc_assign(ctx: *mut HcContext, dst: HcView, src: HcView) -> c_int;
    fn hc_assign_narrow(ctx: *mut HcContext, dst: HcView, src: HcView) -> c_int;
    fn hc_assign_i128(ctx: *mut HcContext, dst: HcView, src: HcView) -> c_int;
    fn hc_add_i64(ctx: *mut HcContext, dst: HcView, src: HcView) -> c_int;
    fn hc_sub_i64(ctx: *mut HcContext, dst: HcView, src: HcView) -> c_int;
    fn hc_add_i128(ctx: *mut HcContext, dst: HcView, src: HcView) -> c_int;
    fn hc_fma_i64(ctx: *mut HcContext, dst: HcView, lhs: HcView, rhs: HcView) -> c_int;
    fn hc_mul_i64(ctx: *mut HcContext, dst: HcView, lhs: HcView, rhs: HcView) -> c_int;
    fn hc_inner_product_i64(ctx: *mut HcContext, dst: HcView, lhs: *const HcView, rhs: *const HcView, n: usize)
        -> c_int;
    fn hc_matmul_i64(ctx: *mut HcContext, dst: HcView, lhs: HcView, rhs: HcView) -> c_int;
    fn hc_create_modulus(prime: i64, out: *mut HcModulus) -> c_int;
    fn hc_mul_mont64(ctx: *mut HcContext, dst: HcView, src: HcView, mods: *const HcModulus, n: usize) -> c_int;
    fn hc_add_red_mont64_double(ctx: *mut HcContext, dst: HcView, src: HcView, mods: *const HcModulus, n: usize)
        -> c_int;
    fn hc_red_mont64_double(ctx: *mut HcContext, dst: HcView, src: HcView, mods: *const HcModulus, n: usize) -> c_int;
    fn hc_add_red_mont64(ctx: *mut HcContext, dst: HcView, src: HcView, mods: *const HcModulus, n: usize) -> c_int;
    fn hc_red_mont64(ctx: *mut HcContext, dst: HcView, src: HcView, mods: *const HcModulus, n: usize) -> c_int;
    fn hc_i128_to_mont64(ctx: *mut HcContext, dst: HcView, src: HcView, mods: *const HcModulus, n: usize) -> c_int;
    fn hc_i64_to_mont64(ctx: *mut HcContext, dst: HcView, mods: *const HcModulus, n: usize) -> c_int;
    fn hc_create_ntt_plan(ctx: *mut HcContext, m: *const HcModulus, shape: *const usize, k: usize,
                          out: *mut *mut HcNttPlan) -> c_int;
    fn hc_destroy_ntt_plan(ctx: *mut HcContext, plan: *mut HcNttPlan) -> c_int;
    fn hc_ntt_mont64_dim(ctx: *mut HcContext, dst: HcView, plans: *const *mut HcNttPlan, n: usize, dim: c_int) -> c_int;
    fn hc_intt_mont64_dim(ctx: *mut HcContext, dst: HcView, plans: *const *mut HcNttPlan, n: usize, dim: c_int)
        -> c_int;
    fn hc_ntt_mul_mont64_dim(ctx: *mut HcContext, dst: HcView, plans: *const *mut HcNttPlan, n: usize, dim: c_int,
                             mul: HcView, mods: *const HcModulus, nmods: usize) -> c_int;
    fn hc_bconv_correct_mont64(ctx: *mut HcContext, dst: HcView, lhs: HcView, rhs: HcView, mods: *const HcModulus,
                               n: usize, shift: usize) -> c_int;
    fn hc_bconv_correct_pow2(ctx: *mut HcContext, dst: HcView, src: HcView, factor0: i64, factor1: i64, shift: usize,
                             log2_modulus: usize) -> c_int;
    fn hc_bconv_correct_pow2_wide(ctx: *mut HcContext, dst: HcView, src: HcView, factor0: *const i64,
                                  factor1: *const i64, shift: usize, log2_modulus: usize) -> c_int;
    fn hc_create_permutation(ctx: *mut HcContext, shape: *const usize, shifts: *const usize, k: usize,
                             out: *mut *mut HcPermPlan) -> c_int;
    fn hc_destroy_permutation(ctx: *mut HcContext, plan: *mut HcPermPlan) -> c_int;
    fn hc_permute(ctx: *mut HcContext, dst: HcView, src: HcView, plan: *mut HcPermPlan, dim: c_int) -> c_int;
}

fn check(rc: c_int) {
    if rc != 0 {
        let msg = unsafe { CStr::from_ptr(hc_last_error()) }.to_string_lossy().into_owned();
        panic!("hal::cuda: {} (status {})", msg, rc);
    }
}

fn dim_arg(dim: DataDim) -> c_int {
    match dim {
        DataDim::Dim2 => HC_DIM2,
        DataDim::Dim3 => HC_DIM3,
    }
}

// ------------------------------------------------------------------------------------------
// Context, tensors and views
// ------------------------------------------------------------------------------------------

/// One device context (device + stream); shared by the backend, its tensors and its plans, and
/// destroyed after the last of them.
pub struct Context(*mut HcContext);
unsafe impl Send for Context {}
unsafe impl Sync for Context {}
impl Drop for Context {
    fn drop(&mut self) {
        unsafe { hc_context_destroy(self.0) };
    }
}

fn strides_for(shape: [usize; DIMS]) -> [usize; DIMS] { [shape[1] * shape[2] * shape[3], shape[2] * shape[3], shape[3], 1] }

fn resolve_range<B: RangeBounds<usize>>(bounds: B, len: usize) -> (usize, usize) {
    let start = match bounds.start_bound() {
        Bound::Included(&s) => s,
        Bound::Excluded(&s) => s + 1,
        Bound::Unbounded => 0,
    };
    let end = match bounds.end_bound() {
        Bound::Included(&e) => e + 1,
        Bound::Excluded(&e) => e,
        Bound::Unbounded => len,
    };
    assert!(start <= end && end <= len, "slice bounds {}..{} invalid for dimension of length {}", start, end, len);
    (start, end)
}

fn slice_view<B0: RangeBounds<usize>, B1: RangeBounds<usize>, B2: RangeBounds<usize>, B3: RangeBounds<usize>>(
    shape: [usize; DIMS],
    strides: [usize; DIMS],
    idx0: B0,
    idx1: B1,
    idx2: B2,
    idx3: B3,
) -> (usize, [usize; DIMS]) {
    let (s0, e0) = resolve_range(idx0, shape[0]);
    let (s1, e1) = resolve_range(idx1, shape[1]);
    let (s2, e2) = resolve_range(idx2, shape[2]);
    let (s3, e3) = resolve_range(idx3, shape[3]);
    (s0 * strides[0] + s1 * strides[1] + s2 * strides[2] + s3 * strides[3], [e0 - s0, e1 - s1, e2 - s2, e3 - s3])
}

fn view_of<T>(ptr: *const T, shape: [usize; DIMS], strides: [usize; DIMS]) -> HcView {
    HcView {
        ptr: ptr as *mut c_void,
        shape: shape.map(|x| x as i64),
        strides: strides.map(|x| x as i64),
    }
}

/// An owned device tensor (zero-initialised by the library, like the CPU backend's).
pub struct CudaTensor<T: Copy> {
    ctx: Arc<Context>,
    ptr: *mut T,
    shape: [usize; DIMS],
}
unsafe impl<T: Copy> Send for CudaTensor<T> {}
unsafe impl<T: Copy> Sync for CudaTensor<T> {}
impl<T: Copy> Drop for CudaTensor<T> {
    fn drop(&mut self) {
        unsafe { hc_free(self.ctx.0, self.ptr as *mut c_void) };
    }
}

#[derive(Clone, Copy, Debug)]
pub struct CudaTensorRef<'a, T: Copy> {
    ptr: *const T,
    shape: [usize; DIMS],
    strides: [usize; DIMS],
    tensor: PhantomData<&'a [T]>,
}

#[derive(Debug)]
pub struct CudaTensorMut<'a, T: Copy> {
    ptr: *mut T,
    shape: [usize; DIMS],
    strides: [usize; DIMS],
    tensor: PhantomData<&'a mut [T]>,
}

impl<'a, T: Copy> CudaTensorRef<'a, T> {
    fn hc(self) -> HcView { view_of(self.ptr, self.shape, self.strides) }
}
impl<'a, T: Copy> CudaTensorMut<'a, T> {
    fn hc(&self) -> HcView { view_of(self.ptr, self.shape, self.strides) }
}

impl<'a, T: Copy> TensorRef for CudaTensorRef<'a, T> {
    fn shape(self) -> [usize; DIMS] { self.shape }

    fn slice<B0: RangeBounds<usize>, B1: RangeBounds<usize>, B2: RangeBounds<usize>, B3: RangeBounds<usize>>(
        self,
        idx0: B0,
        idx1: B1,
        idx2: B2,
        idx3: B3,
    ) -> Self {
        let (offset, shape) = slice_view(self.shape, self.strides, idx0, idx1, idx2, idx3);
        Self { ptr: self.ptr.wrapping_add(offset), shape, strides: self.strides, tensor: PhantomData }
    }
}

impl<'b, T: Copy + 'b> TensorMut<'b, T, CudaTensor<T>> for CudaTensorMut<'b, T> {
    fn shape(&self) -> [usize; DIMS] { self.shape }

    fn reborrow<'a>(&'a mut self) -> CudaTensorMut<'a, T> {
        CudaTensorMut { ptr: self.ptr, shape: self.shape, strides: self.strides, tensor: PhantomData }
    }

    fn as_const<'a>(&'a self) -> CudaTensorRef<'a, T> {
        CudaTensorRef { ptr: self.ptr, shape: self.shape, strides: self.strides, tensor: PhantomData }
    }

    fn into_const(self) -> CudaTensorRef<'b, T> {
        CudaTensorRef { ptr: self.ptr, shape: self.shape, strides: self.strides, tensor: PhantomData }
    }

    /// Two views of disjoint elements (src/hal/cpu.rs:267-284); pointer arithmetic only.
    fn split(self, at: usize, dim: Dim) -> (Self, Self) {
        let d = match dim {
            Dim::Dim0 => 0,
            Dim::Dim1 => 1,
            Dim::Dim2 => 2,
            Dim::Dim3 => 3,
        };
        assert!(at <= self.shape[d], "cannot split dimension of length {} at {}", self.shape[d], at);
        let mut first = self.shape;
        first[d] = at;
        let mut second = self.shape;
        second[d] = self.shape[d] - at;
        (
            Self { ptr: self.ptr, shape: first, strides: self.strides, tensor: PhantomData },
            Self { ptr: self.ptr.wrapping_add(at * self.strides[d]), shape: second, strides: self.strides, tensor: PhantomData },
        )
    }

    fn slice<B0: RangeBounds<usize>, B1: RangeBounds<usize>, B2: RangeBounds<usize>, B3: RangeBounds<usize>>(
        self,
        idx0: B0,
        idx1: B1,
        idx2: B2,
        idx3: B3,
    ) -> Self {
        let (offset, shape) = slice_view(self.shape, self.strides, idx0, idx1, idx2, idx3);
        Self { ptr: self.ptr.wrapping_add(offset), shape, strides: self.strides, tensor: PhantomData }
    }
}

impl<T: Copy> TensorOwned<T> for CudaTensor<T> {
    type Ref<'a>
        = CudaTensorRef<'a, T>
    where
        Self: 'a;
    type Mut<'a>
        = CudaTensorMut<'a, T>
    where
        Self: 'a;

    fn shape(self) -> [usize; DIMS] { self.shape }

    fn as_ref<'a>(&'a self) -> Self::Ref<'a> {
        CudaTensorRef { ptr: self.ptr, shape: self.shape, strides: strides_for(self.shape), tensor: PhantomData }
    }

    fn as_mut<'a>(&'a mut self) -> Self::Mut<'a> {
        CudaTensorMut { ptr: self.ptr, shape: self.shape, strides: strides_for(self.shape), tensor: PhantomData }
    }
}

/// A device NTT plan (twiddles and stage programme in HBM), released with its last clone.
pub struct NttPlanHandle {
    ctx: Arc<Context>,
    plan: *mut HcNttPlan,
}
unsafe impl Send for NttPlanHandle {}
unsafe impl Sync for NttPlanHandle {}
impl Drop for NttPlanHandle {
    fn drop(&mut self) {
        unsafe { hc_destroy_ntt_plan(self.ctx.0, self.plan) };
    }
}

/// A device permutation table, released with its last clone.
pub struct PermutationHandle {
    ctx: Arc<Context>,
    plan: *mut HcPermPlan,
}
unsafe impl Send for PermutationHandle {}
unsafe impl Sync for PermutationHandle {}
impl Drop for PermutationHandle {
    fn drop(&mut self) {
        unsafe { hc_destroy_permutation(self.ctx.0, self.plan) };
    }
}

// ------------------------------------------------------------------------------------------
// The backend
// ------------------------------------------------------------------------------------------

/// The GB300 backend: one context (device + stream). Cloning shares the context.
#[derive(Clone)]
pub struct CudaBackend {
    ctx: Arc<Context>,
}

impl CudaBackend {
    pub fn new(device: i32) -> Self {
        let mut ctx = std::ptr::null_mut();
        check(unsafe { hc_context_create(device, &mut ctx) });
        Self { ctx: Arc::new(Context(ctx)) }
    }

    fn c(&self) -> *mut HcContext { self.ctx.0 }

    fn plans(ntt: &[Arc<NttPlanHandle>]) -> Vec<*mut HcNttPlan> { ntt.iter().map(|p| p.plan).collect() }
}

fn words(x: i128) -> [i64; 2] { [x as i64, (x >> 64) as i64] }

impl Backend for CudaBackend {
    type TensorI64 = CudaTensor<i64>;
    type TensorI128 = CudaTensor<i128>;
    type Modulus = HcModulus;
    type NTTPlan = Arc<NttPlanHandle>;
    type PermutationPlan = Arc<PermutationHandle>;

    fn hal_allocate_i64(&self, shape: [usize; DIMS]) -> CudaTensor<i64> {
        let s = shape.map(|x| x as i64);
        let mut p = std::ptr::null_mut();
        check(unsafe { hc_allocate_i64(self.c(), s.as_ptr(), &mut p) });
        CudaTensor { ctx: self.ctx.clone(), ptr: p as *mut i64, shape }
    }

    fn hal_allocate_i128(&self, shape: [usize; DIMS]) -> CudaTensor<i128> {
        let s = shape.map(|x| x as i64);
        let mut p = std::ptr::null_mut();
        check(unsafe { hc_allocate_i128(self.c(), s.as_ptr(), &mut p) });
        CudaTensor { ctx: self.ctx.clone(), ptr: p as *mut i128, shape }
    }

    fn hal_import(&self, dst: TensorI64Mut<Self>, src: &[i64]) {
        check(unsafe { hc_import(self.c(), dst.hc(), src.as_ptr(), src.len()) });
    }

    fn hal_export(&self, src: TensorI64Ref<Self>, dst: &mut [i64]) {
        check(unsafe { hc_export(self.c(), src.hc(), dst.as_mut_ptr(), dst.len()) });
    }

    fn hal_assign(&self, dst: TensorI64Mut<Self>, src: TensorI64Ref<Self>) {
        check(unsafe { hc_assign(self.c(), dst.hc(), src.hc()) });
    }

    fn hal_assign_narrow(&self, dst: TensorI64Mut<Self>, src: TensorI128Ref<Self>) {
        check(unsafe { hc_assign_narrow(self.c(), dst.hc(), src.hc()) });
    }

    fn hal_assign_i128(&self, dst: TensorI128Mut<Self>, src: TensorI128Ref<Self>) {
        check(unsafe { hc_assign_i128(self.c(), dst.hc(), src.hc()) });
    }

    fn hal_add_i64(&self, dst: TensorI64Mut<Self>, src: TensorI64Ref<Self>) {
        check(unsafe { hc_add_i64(self.c(), dst.hc(), src.hc()) });
    }

    fn hal_sub_i64(&self, dst: TensorI64Mut<Self>, src: TensorI64Ref<Self>) {
        check(unsafe { hc_sub_i64(self.c(), dst.hc(), src.hc()) });
    }

    fn hal_add_i128(&self, dst: TensorI128Mut<Self>, src: TensorI128Ref<Self>) {
        check(unsafe { hc_add_i128(self.c(), dst.hc(), src.hc()) });
    }

    fn hal_fma_i64(&self, dst: TensorI128Mut<Self>, lhs: TensorI64Ref<Self>, rhs: TensorI64Ref<Self>) {
        check(unsafe { hc_fma_i64(self.c(), dst.hc(), lhs.hc(), rhs.hc()) });
    }

    fn hal_mul_i64(&self, dst: TensorI128Mut<Self>, lhs: TensorI64Ref<Self>, rhs: TensorI64Ref<Self>) {
        check(unsafe { hc_mul_i64(self.c(), dst.hc(), lhs.hc(), rhs.hc()) });
    }

    fn hal_inner_product_i64(&self, dst: TensorI128Mut<Self>, lhs: &[TensorI64Ref<Self>], rhs: &[TensorI64Ref<Self>]) {
        assert_eq!(lhs.len(), rhs.len());
        let l = lhs.iter().map(|t| t.hc()).collect::<Vec<_>>();
        let r = rhs.iter().map(|t| t.hc()).collect::<Vec<_>>();
        check(unsafe { hc_inner_product_i64(self.c(), dst.hc(), l.as_ptr(), r.as_ptr(), l.len()) });
    }

    fn hal_matmul_i64(&self, dst: TensorI128Mut<Self>, lhs: TensorI64Ref<Self>, rhs: TensorI64Ref<Self>) {
        check(unsafe { hc_matmul_i64(self.c(), dst.hc(), lhs.hc(), rhs.hc()) });
    }

    fn hal_create_modulus(&self, prime: i64) -> HcModulus {
        let mut m = HcModulus { n: 0, neg_inv_n: 0, r2_mod_n: 0, r3_mod_n: 0 };
        check(unsafe { hc_create_modulus(prime, &mut m) });
        m
    }

    fn hal_mul_mont64(&self, dst: TensorI64Mut<Self>, src: TensorI64Ref<Self>, mods: &Moduli<Self>) {
        check(unsafe { hc_mul_mont64(self.c(), dst.hc(), src.hc(), mods.as_ptr(), mods.len()) });
    }

    fn hal_add_red_mont64_double(&self, dst: TensorI64Mut<Self>, src: TensorI128Ref<Self>, mods: &Moduli<Self>) {
        check(unsafe { hc_add_red_mont64_double(self.c(), dst.hc(), src.hc(), mods.as_ptr(), mods.len()) });
    }

    fn hal_red_mont64_double(&self, dst: TensorI64Mut<Self>, src: TensorI128Ref<Self>, mods: &Moduli<Self>) {
        check(unsafe { hc_red_mont64_double(self.c(), dst.hc(), src.hc(), mods.as_ptr(), mods.len()) });
    }

    fn hal_add_red_mont64(&self, dst: TensorI64Mut<Self>, src: TensorI128Ref<Self>, mods: &Moduli<Self>) {
        check(unsafe { hc_add_red_mont64(self.c(), dst.hc(), src.hc(), mods.as_ptr(), mods.len()) });
    }

    fn hal_red_mont64(&self, dst: TensorI64Mut<Self>, src: TensorI128Ref<Self>, mods: &Moduli<Self>) {
        check(unsafe { hc_red_mont64(self.c(), dst.hc(), src.hc(), mods.as_ptr(), mods.len()) });
    }

    fn hal_i128_to_mont64(&self, dst: TensorI64Mut<Self>, src: TensorI128Ref<Self>, mods: &Moduli<Self>) {
        check(unsafe { hc_i128_to_mont64(self.c(), dst.hc(), src.hc(), mods.as_ptr(), mods.len()) });
    }

    fn hal_i64_to_mont64(&self, dst: TensorI64Mut<Self>, mods: &Moduli<Self>) {
        check(unsafe { hc_i64_to_mont64(self.c(), dst.hc(), mods.as_ptr(), mods.len()) });
    }

    fn hal_create_ntt_plan(&self, modulus: &HcModulus, inner_shape: &[usize]) -> Arc<NttPlanHandle> {
        let mut p = std::ptr::null_mut();
        check(unsafe { hc_create_ntt_plan(self.c(), modulus, inner_shape.as_ptr(), inner_shape.len(), &mut p) });
        Arc::new(NttPlanHandle { ctx: self.ctx.clone(), plan: p })
    }

    fn hal_ntt_mont64_dim(&self, dst: TensorI64Mut<Self>, ntt: &[Self::NTTPlan], dim: DataDim) {
        let p = Self::plans(ntt);
        check(unsafe { hc_ntt_mont64_dim(self.c(), dst.hc(), p.as_ptr(), p.len(), dim_arg(dim)) });
    }

    fn hal_intt_mont64_dim(&self, dst: TensorI64Mut<Self>, ntt: &[Self::NTTPlan], dim: DataDim) {
        let p = Self::plans(ntt);
        check(unsafe { hc_intt_mont64_dim(self.c(), dst.hc(), p.as_ptr(), p.len(), dim_arg(dim)) });
    }

    fn hal_ntt_mul_mont64_dim(
        &self,
        dst: TensorI64Mut<Self>,
        ntt: &[Self::NTTPlan],
        dim: DataDim,
        mul: TensorI64Ref<Self>,
        mods: &Moduli<Self>,
    ) {
        let p = Self::plans(ntt);
        check(unsafe {
            hc_ntt_mul_mont64_dim(self.c(), dst.hc(), p.as_ptr(), p.len(), dim_arg(dim), mul.hc(), mods.as_ptr(), mods.len())
        });
    }

    fn hal_bconv_correct_mont64(
        &self,
        dst: TensorI64Mut<Self>,
        lhs: TensorI128Ref<Self>,
        rhs: TensorI64Ref<Self>,
        mods: &Moduli<Self>,
        shift: usize,
    ) {
        check(unsafe { hc_bconv_correct_mont64(self.c(), dst.hc(), lhs.hc(), rhs.hc(), mods.as_ptr(), mods.len(), shift) });
    }

    fn hal_bconv_correct_pow2(
        &self,
        dst: TensorI64Mut<Self>,
        src: TensorI128Ref<Self>,
        factor0: i64,
        factor1: i64,
        shift: usize,
        log2_modulus: usize,
    ) {
        check(unsafe { hc_bconv_correct_pow2(self.c(), dst.hc(), src.hc(), factor0, factor1, shift, log2_modulus) });
    }

    fn hal_bconv_correct_pow2_wide(
        &self,
        dst: TensorI64Mut<Self>,
        src: TensorI128Ref<Self>,
        factor0: i128,
        factor1: i128,
        shift: usize,
        log2_modulus: usize,
    ) {
        let (f0, f1) = (words(factor0), words(factor1));
        check(unsafe {
            hc_bconv_correct_pow2_wide(self.c(), dst.hc(), src.hc(), f0.as_ptr(), f1.as_ptr(), shift, log2_modulus)
        });
    }

    fn hal_create_permutation(&self, inner_shape: &[usize], shifts: &[usize]) -> Arc<PermutationHandle> {
        assert_eq!(inner_shape.len(), shifts.len());
        let mut p = std::ptr::null_mut();
        check(unsafe { hc_create_permutation(self.c(), inner_shape.as_ptr(), shifts.as_ptr(), shifts.len(), &mut p) });
        Arc::new(PermutationHandle { ctx: self.ctx.clone(), plan: p })
    }

    fn hal_permute(&self, dst: TensorI64Mut<Self>, src: TensorI64Ref<Self>, permutation: &Self::PermutationPlan,
                   dim: DataDim) {
        check(unsafe { hc_permute(self.c(), dst.hc(), src.hc(), permutation.plan, dim_arg(dim)) });
    }
}

#[cfg(test)]
mod tests {
    //! The crate's own backend tests, run against this backend: swap `CpuBackend` for
    //! `CudaBackend::new(0)` in src/hal/cpu.rs's test module and src/ring.rs / src/bfv.rs tests.
    use super::*;

    #[test]
    fn import_export_roundtrip() {
        let be = CudaBackend::new(0);
        let mut t = be.hal_allocate_i64([2, 3, 4, 5]);
        let data = (0..120).collect::<Vec<i64>>();
        be.hal_import(t.as_mut(), &data);
        let mut back = vec![0; 120];
        be.hal_export(t.as_ref(), &mut back);
        assert_eq!(data, back);
    }
}
