"""Python binding of the C ABI in include/halcuda.h (ctypes).

Mirrors the reference's tensor HAL trait `hal::Backend` (cyclosubfield-dbfv/src/hal/mod.rs:108-350)
method by method (`hal_*` names, same argument meaning), over device tensors owned by the
library. Errors raise :class:`HalError` carrying the library's message, the counterpart of the
reference's panics. There is no fallback: if ``libhalcuda.so`` cannot be loaded or no GPU is
present, every call raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhalcuda.so")


class HalError(RuntimeError):
    pass


class HcView(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("shape", ctypes.c_int64 * 4), ("strides", ctypes.c_int64 * 4)]


class HcModulus(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("neg_inv_n", ctypes.c_int64), ("r2_mod_n", ctypes.c_int64),
                ("r3_mod_n", ctypes.c_int64)]


_lib = None


def lib_path():
    """Path of libhalcuda.so, built first if it is missing or stale (nothing is loaded)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("_halcuda_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def lib():
    """Loads libhalcuda.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is None:
        import importlib.util

        spec = importlib.util.spec_from_file_location("_halcuda_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
        _lib = ctypes.CDLL(path)
        _lib.hc_last_error.restype = ctypes.c_char_p
        _lib.hc_launch_count.restype = ctypes.c_uint64
        _lib.hc_launch_count.argtypes = [ctypes.c_void_p]
        _lib.hc_context_stream.restype = ctypes.c_void_p
        _lib.hc_context_stream.argtypes = [ctypes.c_void_p]
    return _lib


def check(rc):
    if rc != 0:
        raise HalError("halcuda error %d: %s" % (rc, lib().hc_last_error().decode()))


DIM2, DIM3 = 2, 3


class DeviceTensor:
    """A strided view of device memory; `owner` keeps the allocation alive."""

    def __init__(self, ctx, ptr, shape, strides, wide, owner=None):
        self.ctx, self.ptr, self.shape, self.strides, self.wide = ctx, ptr, tuple(shape), tuple(strides), wide
        self.owner = owner

    @property
    def esize(self):
        return 16 if self.wide else 8

    def view(self):
        v = HcView()
        v.ptr = self.ptr
        for d in range(4):
            v.shape[d] = self.shape[d]
            v.strides[d] = self.strides[d]
        return v

    def numel(self):
        return int(np.prod(self.shape))

    def slice(self, *ranges):
        """Sub-view; ranges are (start, end) pairs per dimension or None for the full range."""
        off = 0
        shape = list(self.shape)
        for d, rg in enumerate(ranges):
            if rg is None:
                continue
            s, e = rg
            assert 0 <= s <= e <= self.shape[d]
            off += s * self.strides[d]
            shape[d] = e - s
        return DeviceTensor(self.ctx, self.ptr + off * self.esize, shape, self.strides, self.wide,
                            self.owner if self.owner is not None else self)

    def rows(self, s, e):
        return self.slice((s, e))

    def base_range(self, s, e):
        return self.slice(None, (s, e))

    def to_numpy(self):
        n = self.numel()
        if self.wide:
            out = np.zeros(tuple(self.shape) + (2,), dtype=np.int64)
            check(lib().hc_export_i128(self.ctx.h, self.view(), out.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.c_size_t(n)))
        else:
            out = np.zeros(self.shape, dtype=np.int64)
            check(lib().hc_export(self.ctx.h, self.view(), out.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(n)))
        return out

    def copy_from(self, arr):
        arr = np.ascontiguousarray(arr, dtype=np.int64)
        n = self.numel()
        if self.wide:
            assert arr.shape == tuple(self.shape) + (2,), (arr.shape, self.shape)
            check(lib().hc_import_i128(self.ctx.h, self.view(), arr.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.c_size_t(n)))
        else:
            assert arr.shape == tuple(self.shape), (arr.shape, self.shape)
            check(lib().hc_import(self.ctx.h, self.view(), arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(n)))
        return self


class _Alloc:
    def __init__(self, ctx, ptr):
        self.ctx, self.ptr = ctx, ptr

    def __del__(self):
        try:
            if self.ctx.h:  # a closed context already released its memory pool
                lib().hc_free(self.ctx.h, ctypes.c_void_p(self.ptr))
        except Exception:
            pass


def _strides(shape):
    return (shape[1] * shape[2] * shape[3], shape[2] * shape[3], shape[3], 1)


def _mods(mods):
    arr = (HcModulus * max(1, len(mods)))(*mods)
    return arr, ctypes.c_size_t(len(mods))


class NttPlan:
    def __init__(self, ctx, handle, modulus, inner_shape):
        self.ctx, self.h, self.modulus, self.inner_shape = ctx, handle, modulus, tuple(inner_shape)

    def __del__(self):
        try:
            if self.ctx.h:
                lib().hc_destroy_ntt_plan(self.ctx.h, self.h)
        except Exception:
            pass


class PermPlan:
    def __init__(self, ctx, handle):
        self.ctx, self.h = ctx, handle

    def __del__(self):
        try:
            if self.ctx.h:
                lib().hc_destroy_permutation(self.ctx.h, self.h)
        except Exception:
            pass


class CudaBackend:
    """The `hal::Backend` trait on the GPU: one method per trait method (src/hal/mod.rs:108-350)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        check(lib().hc_context_create(ctypes.c_int(device), ctypes.byref(h)))
        self.h = h
        self._dependents = []  # weak references to objects that must be released first

    def add_dependent(self, obj):
        import weakref

        self._dependents.append(weakref.ref(obj))

    def close(self):
        """Releases dependents (ring contexts), then the context; later frees are no-ops."""
        if self.h:
            for ref in self._dependents:
                obj = ref()
                if obj is not None:
                    obj.close()
            lib().hc_context_destroy(self.h)
            self.h = None

    def synchronize(self):
        check(lib().hc_synchronize(self.h))

    def set_stream(self, stream):
        """Routes subsequent calls to `stream` (a Stream), or back to the context's own stream (None)."""
        check(lib().hc_context_set_stream(self.h, stream.h if stream is not None else None))

    def on(self, stream):
        be = self

        class _Use:
            def __enter__(self):
                be.set_stream(stream)

            def __exit__(self, *exc):
                be.set_stream(None)

        return _Use()

    def launch_count(self):
        return int(lib().hc_launch_count(self.h))

    # ---- allocation and transfer ----
    def hal_allocate_i64(self, shape):
        return self._alloc(shape, False)

    def hal_allocate_i128(self, shape):
        return self._alloc(shape, True)

    def _alloc(self, shape, wide):
        shape = tuple(int(s) for s in shape)
        ptr = ctypes.c_void_p()
        sh = (ctypes.c_int64 * 4)(*shape)
        fn = lib().hc_allocate_i128 if wide else lib().hc_allocate_i64
        check(fn(self.h, sh, ctypes.byref(ptr)))
        owner = _Alloc(self, ptr.value)
        return DeviceTensor(self, ptr.value, shape, _strides(shape), wide, owner)

    def tensor(self, arr, wide=False):
        arr = np.asarray(arr, dtype=np.int64)
        shape = arr.shape[:4]
        t = self._alloc(shape, wide)
        t.copy_from(arr)
        return t

    def hal_import(self, dst, src):
        dst.copy_from(src)

    def hal_export(self, src):
        return src.to_numpy()

    # ---- copies and integer arithmetic ----
    def hal_assign(self, dst, src):
        check(lib().hc_assign(self.h, dst.view(), src.view()))

    def hal_assign_narrow(self, dst, src):
        check(lib().hc_assign_narrow(self.h, dst.view(), src.view()))

    def hal_assign_i128(self, dst, src):
        check(lib().hc_assign_i128(self.h, dst.view(), src.view()))

    def hal_add_i64(self, dst, src):
        check(lib().hc_add_i64(self.h, dst.view(), src.view()))

    def hal_sub_i64(self, dst, src):
        check(lib().hc_sub_i64(self.h, dst.view(), src.view()))

    def hal_add_i128(self, dst, src):
        check(lib().hc_add_i128(self.h, dst.view(), src.view()))

    def hal_fma_i64(self, dst, lhs, rhs):
        check(lib().hc_fma_i64(self.h, dst.view(), lhs.view(), rhs.view()))

    def hal_mul_i64(self, dst, lhs, rhs):
        check(lib().hc_mul_i64(self.h, dst.view(), lhs.view(), rhs.view()))

    def hal_inner_product_i64(self, dst, lhs, rhs):
        lv = (HcView * len(lhs))(*[t.view() for t in lhs])
        rv = (HcView * len(rhs))(*[t.view() for t in rhs])
        check(lib().hc_inner_product_i64(self.h, dst.view(), lv, rv, ctypes.c_size_t(len(lhs))))

    def hal_matmul_i64(self, dst, lhs, rhs):
        check(lib().hc_matmul_i64(self.h, dst.view(), lhs.view(), rhs.view()))

    # ---- Montgomery arithmetic ----
    def hal_create_modulus(self, prime):
        m = HcModulus()
        check(lib().hc_create_modulus(ctypes.c_int64(prime), ctypes.byref(m)))
        return m

    def hal_mul_mont64(self, dst, src, mods):
        a, n = _mods(mods)
        check(lib().hc_mul_mont64(self.h, dst.view(), src.view(), a, n))

    def _red(self, name, dst, src, mods):
        a, n = _mods(mods)
        check(getattr(lib(), name)(self.h, dst.view(), src.view(), a, n))

    def hal_add_red_mont64_double(self, dst, src, mods):
        self._red("hc_add_red_mont64_double", dst, src, mods)

    def hal_red_mont64_double(self, dst, src, mods):
        self._red("hc_red_mont64_double", dst, src, mods)

    def hal_add_red_mont64(self, dst, src, mods):
        self._red("hc_add_red_mont64", dst, src, mods)

    def hal_red_mont64(self, dst, src, mods):
        self._red("hc_red_mont64", dst, src, mods)

    def hal_i128_to_mont64(self, dst, src, mods):
        self._red("hc_i128_to_mont64", dst, src, mods)

    def hal_i64_to_mont64(self, dst, mods):
        a, n = _mods(mods)
        check(lib().hc_i64_to_mont64(self.h, dst.view(), a, n))

    # ---- NTT ----
    def hal_create_ntt_plan(self, modulus, inner_shape):
        shape = (ctypes.c_size_t * max(1, len(inner_shape)))(*inner_shape)
        h = ctypes.c_void_p()
        check(lib().hc_create_ntt_plan(self.h, ctypes.byref(modulus), shape, ctypes.c_size_t(len(inner_shape)),
                                       ctypes.byref(h)))
        return NttPlan(self, h, modulus, inner_shape)

    @staticmethod
    def _plans(plans):
        return (ctypes.c_void_p * max(1, len(plans)))(*[p.h.value for p in plans]), ctypes.c_size_t(len(plans))

    def hal_ntt_mont64_dim(self, dst, plans, dim):
        p, n = self._plans(plans)
        check(lib().hc_ntt_mont64_dim(self.h, dst.view(), p, n, ctypes.c_int(dim)))

    def hal_intt_mont64_dim(self, dst, plans, dim):
        p, n = self._plans(plans)
        check(lib().hc_intt_mont64_dim(self.h, dst.view(), p, n, ctypes.c_int(dim)))

    def hal_ntt_mul_mont64_dim(self, dst, plans, dim, mul, mods):
        p, n = self._plans(plans)
        a, nm = _mods(mods)
        check(lib().hc_ntt_mul_mont64_dim(self.h, dst.view(), p, n, ctypes.c_int(dim), mul.view(), a, nm))

    def hal_ntt_mont64(self, dst, dim2, dim3):
        self.hal_ntt_mont64_dim(dst, dim2, DIM2)
        self.hal_ntt_mont64_dim(dst, dim3, DIM3)

    def hal_intt_mont64(self, dst, dim2, dim3):
        self.hal_intt_mont64_dim(dst, dim2, DIM2)
        self.hal_intt_mont64_dim(dst, dim3, DIM3)

    # ---- base-conversion corrections ----
    def hal_bconv_correct_mont64(self, dst, lhs, rhs, mods, shift):
        a, n = _mods(mods)
        check(lib().hc_bconv_correct_mont64(self.h, dst.view(), lhs.view(), rhs.view(), a, n, ctypes.c_size_t(shift)))

    def hal_bconv_correct_pow2(self, dst, src, factor0, factor1, shift, log2_modulus):
        check(lib().hc_bconv_correct_pow2(self.h, dst.view(), src.view(), ctypes.c_int64(factor0),
                                          ctypes.c_int64(factor1), ctypes.c_size_t(shift),
                                          ctypes.c_size_t(log2_modulus)))

    def hal_bconv_correct_pow2_wide(self, dst, src, factor0, factor1, shift, log2_modulus):
        def words(x):
            x &= (1 << 128) - 1
            lo, hi = x & ((1 << 64) - 1), x >> 64
            return (ctypes.c_int64 * 2)(lo - (1 << 64) if lo >> 63 else lo, hi - (1 << 64) if hi >> 63 else hi)

        check(lib().hc_bconv_correct_pow2_wide(self.h, dst.view(), src.view(), words(factor0), words(factor1),
                                               ctypes.c_size_t(shift), ctypes.c_size_t(log2_modulus)))

    # ---- permutations ----
    def hal_create_permutation(self, inner_shape, shifts):
        k = len(inner_shape)
        s = (ctypes.c_size_t * max(1, k))(*inner_shape)
        sh = (ctypes.c_size_t * max(1, k))(*shifts)
        h = ctypes.c_void_p()
        check(lib().hc_create_permutation(self.h, s, sh, ctypes.c_size_t(k), ctypes.byref(h)))
        return PermPlan(self, h)

    def hal_permute(self, dst, src, plan, dim):
        check(lib().hc_permute(self.h, dst.view(), src.view(), plan.h, ctypes.c_int(dim)))


# ---------------------------------------------------------------------------------- runtime
def barrett_peak(be):
    """The GPU's rate (products/s) of the transforms' exact 64-bit Barrett product, measured by a
    register-only kernel (hc_barrett_peak)."""
    v = ctypes.c_double()
    check(lib().hc_barrett_peak(be.h, ctypes.byref(v)))
    return float(v.value)


def int8_mma_peak(be):
    """The GPU's int8 tensor-core rate (multiply-adds/s) of warp-level s8 x s8 -> s32 MMAs, measured
    by a register-only kernel (hc_int8_mma_peak)."""
    v = ctypes.c_double()
    check(lib().hc_int8_mma_peak(be.h, ctypes.byref(v)))
    return float(v.value)


class PinnedBuffer:
    """Page-locked host memory viewed as a numpy int64 array."""

    def __init__(self, shape):
        self.shape = tuple(shape)
        nbytes = int(np.prod(self.shape)) * 8
        p = ctypes.c_void_p()
        check(lib().hc_host_alloc(ctypes.c_size_t(nbytes), ctypes.byref(p)))
        self.ptr = p.value
        self.nbytes = nbytes
        self.array = np.ctypeslib.as_array((ctypes.c_int64 * (nbytes // 8)).from_address(self.ptr)).reshape(self.shape)

    def __del__(self):
        try:
            lib().hc_host_free(ctypes.c_void_p(self.ptr))
        except Exception:
            pass


H2D, D2H, D2D = 0, 1, 2


def memcpy_async(be, dst_ptr, src_ptr, nbytes, kind):
    check(lib().hc_memcpy_async(be.h, ctypes.c_void_p(dst_ptr), ctypes.c_void_p(src_ptr), ctypes.c_size_t(nbytes),
                                ctypes.c_int(kind)))


def memset_async(be, dst_ptr, value, nbytes):
    check(lib().hc_memset_async(be.h, ctypes.c_void_p(dst_ptr), ctypes.c_int(value), ctypes.c_size_t(nbytes)))


class Stream:
    """An extra CUDA stream; `with be.on(stream):` routes the calls inside to it."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().hc_stream_create(ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().hc_stream_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Event:
    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().hc_event_create(ctypes.byref(h)))
        self.h = h

    def record(self, be):
        check(lib().hc_event_record(be.h, self.h))

    def wait(self, be):
        """Makes the backend's current stream wait (on the device) for the work before this event."""
        check(lib().hc_stream_wait_event(be.h, self.h))

    def query(self):
        """True once the work recorded before this event has completed (does not block)."""
        done = ctypes.c_int(0)
        check(lib().hc_event_query(self.h, ctypes.byref(done)))
        return bool(done.value)

    def elapsed_ms(self, end, timeout_ms=120000.0):
        ms = ctypes.c_float()
        check(lib().hc_event_elapsed_ms(self.h, end.h, ctypes.c_double(timeout_ms), ctypes.byref(ms)))
        return float(ms.value)

    def __del__(self):
        try:
            lib().hc_event_destroy(self.h)
        except Exception:
            pass


def device_memory(be):
    f, t = ctypes.c_size_t(), ctypes.c_size_t()
    check(lib().hc_device_memory(be.h, ctypes.byref(f), ctypes.byref(t)))
    return int(f.value), int(t.value)


def memory_stats(be, reset_high=False):
    """(allocation calls made by the library so far, bytes in use in the device's default memory
    pool, that pool's high-water mark); `reset_high` first resets the mark to the bytes in use."""
    out = (ctypes.c_uint64 * 3)()
    check(lib().hc_memory_stats(be.h, ctypes.c_int(1 if reset_high else 0), out))
    return int(out[0]), int(out[1]), int(out[2])


class Graph:
    """A captured sequence of calls (hc_graph_*), replayed with launch()."""

    def __init__(self, be, fn):
        self.be = be
        check(lib().hc_graph_begin_capture(be.h))
        try:
            fn()
        finally:
            h = ctypes.c_void_p()
            rc = lib().hc_graph_end_capture(be.h, ctypes.byref(h))
        check(rc)
        self.h = h

    def launch(self):
        check(lib().hc_graph_launch(self.be.h, self.h))

    def __del__(self):
        try:
            lib().hc_graph_destroy(self.h)
        except Exception:
            pass
