"""ctypes bindings of the oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module; the
product library never does. i128 tensors are numpy int64 arrays with a trailing axis of 2
(little-endian low word, then high word), which is the memory layout of ``__int128``.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


class OrView(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("shape", ctypes.c_int64 * 4), ("strides", ctypes.c_int64 * 4)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        _lib.or_last_error.restype = ctypes.c_char_p
        _lib.or_ring_create.restype = ctypes.c_void_p
        _lib.or_ring_create_raw.restype = ctypes.c_void_p
        _lib.or_ring_num_factors.restype = ctypes.c_size_t
        _lib.or_ring_initial_len.restype = ctypes.c_size_t
        _lib.or_ring_prime.restype = ctypes.c_int64
        _lib.or_find_root_of_unity.restype = ctypes.c_int64
        _lib.or_bfv_log2_alpha_for_sigma.restype = ctypes.c_double
        for name in ("or_ring_free", "or_ring_num_factors", "or_ring_initial_len", "or_ring_prime"):
            getattr(_lib, name).argtypes = [ctypes.c_void_p] + ([ctypes.c_size_t] if name == "or_ring_prime" else [])
    return _lib


class OracleError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise OracleError(lib().or_last_error().decode())


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def view(a, i128=False):
    """A strided view of a numpy array holding an i64 tensor (4 dims) or an i128 tensor (4 dims
    plus a trailing axis of 2)."""
    assert a.dtype == np.int64
    if i128:
        assert a.ndim == 5 and a.shape[4] == 2 and a.strides[4] == 8
        strides = [s // 16 for s in a.strides[:4]]
        assert all(s * 16 == o for s, o in zip(strides, a.strides[:4]))
        shape = a.shape[:4]
    else:
        assert a.ndim == 4
        strides = [s // 8 for s in a.strides]
        shape = a.shape
    if a.size == 0:  # numpy reports arbitrary strides for empty arrays
        strides = [shape[1] * shape[2] * shape[3], shape[2] * shape[3], shape[3], 1]
    v = OrView()
    v.ptr = a.ctypes.data
    for d in range(4):
        v.shape[d] = shape[d]
        v.strides[d] = strides[d]
    return v


def _primes(primes):
    return np.ascontiguousarray(np.asarray(primes, dtype=np.int64))


def _sz(values):
    return np.ascontiguousarray(np.asarray(values, dtype=np.uint64))


# ---------------------------------------------------------------- i128 helpers
def to_i128(values, shape=None):
    """Python ints -> numpy (…, 2) int64 array (low, high words)."""
    flat = [int(v) for v in np.asarray(values, dtype=object).reshape(-1)]
    out = np.empty((len(flat), 2), dtype=np.int64)
    for i, v in enumerate(flat):
        v &= (1 << 128) - 1
        lo, hi = v & ((1 << 64) - 1), v >> 64
        out[i, 0] = lo - (1 << 64) if lo >= 1 << 63 else lo
        out[i, 1] = hi - (1 << 64) if hi >= 1 << 63 else hi
    if shape is not None:
        out = out.reshape(tuple(shape) + (2,))
    return out


def from_i128(arr):
    """numpy (…, 2) int64 array -> numpy object array of Python ints."""
    lo = arr[..., 0].astype(object) & ((1 << 64) - 1)
    hi = arr[..., 1].astype(object)
    return hi * (1 << 64) + lo


# ---------------------------------------------------------------- HAL methods
def _call(name, *args):
    _check(getattr(lib(), name)(*args))


def assign(dst, src):
    _call("or_assign", ctypes.byref(view(dst)), ctypes.byref(view(src)))


def assign_narrow(dst, src):
    _call("or_assign_narrow", ctypes.byref(view(dst)), ctypes.byref(view(src, True)))


def assign_i128(dst, src):
    _call("or_assign_i128", ctypes.byref(view(dst, True)), ctypes.byref(view(src, True)))


def add_i64(dst, src):
    _call("or_add_i64", ctypes.byref(view(dst)), ctypes.byref(view(src)))


def sub_i64(dst, src):
    _call("or_sub_i64", ctypes.byref(view(dst)), ctypes.byref(view(src)))


def add_i128(dst, src):
    _call("or_add_i128", ctypes.byref(view(dst, True)), ctypes.byref(view(src, True)))


def fma_i64(dst, lhs, rhs):
    _call("or_fma_i64", ctypes.byref(view(dst, True)), ctypes.byref(view(lhs)), ctypes.byref(view(rhs)))


def mul_i64(dst, lhs, rhs):
    _call("or_mul_i64", ctypes.byref(view(dst, True)), ctypes.byref(view(lhs)), ctypes.byref(view(rhs)))


def inner_product_i64(dst, lhs, rhs):
    lv = (OrView * len(lhs))(*[view(a) for a in lhs])
    rv = (OrView * len(rhs))(*[view(a) for a in rhs])
    _call("or_inner_product_i64", ctypes.byref(view(dst, True)), lv, rv, ctypes.c_size_t(len(lhs)))


def matmul_i64(dst, lhs, rhs):
    _call("or_matmul_i64", ctypes.byref(view(dst, True)), ctypes.byref(view(lhs)), ctypes.byref(view(rhs)))


def mul_mont64(dst, src, primes):
    p = _primes(primes)
    _call("or_mul_mont64", ctypes.byref(view(dst)), ctypes.byref(view(src)), _p(p), ctypes.c_size_t(len(p)))


RED_KINDS = {"add_red_mont64_double": 0, "red_mont64_double": 1, "add_red_mont64": 2, "red_mont64": 3,
             "i128_to_mont64": 4}


def red128(kind, dst, src, primes):
    p = _primes(primes)
    _call("or_red128", ctypes.c_int(RED_KINDS[kind]), ctypes.byref(view(dst)), ctypes.byref(view(src, True)), _p(p),
          ctypes.c_size_t(len(p)))


def i64_to_mont64(dst, primes):
    p = _primes(primes)
    _call("or_i64_to_mont64", ctypes.byref(view(dst)), _p(p), ctypes.c_size_t(len(p)))


def ntt_dim(dst, primes, inner_shape, dim, mode, mul=None):
    """mode: 'ntt', 'intt' or 'ntt_mul' (then `mul` is the kernel tensor)."""
    p = _primes(primes)
    s = _sz(inner_shape)
    mv = view(mul) if mul is not None else view(dst)
    _call("or_ntt_dim", ctypes.byref(view(dst)), _p(p), ctypes.c_size_t(len(p)), _p(s), ctypes.c_size_t(len(s)),
          ctypes.c_int(dim), ctypes.c_int({"ntt": 0, "intt": 1, "ntt_mul": 2}[mode]), ctypes.byref(mv))


def bconv_correct_mont64(dst, lhs, rhs, primes, shift):
    p = _primes(primes)
    _call("or_bconv_correct_mont64", ctypes.byref(view(dst)), ctypes.byref(view(lhs, True)), ctypes.byref(view(rhs)),
          _p(p), ctypes.c_size_t(len(p)), ctypes.c_size_t(shift))


def bconv_correct_pow2(dst, src, f0, f1, shift, log2m):
    _call("or_bconv_correct_pow2", ctypes.byref(view(dst)), ctypes.byref(view(src, True)), ctypes.c_int64(f0),
          ctypes.c_int64(f1), ctypes.c_size_t(shift), ctypes.c_size_t(log2m))


def bconv_correct_pow2_wide(dst, src, f0, f1, shift, log2m):
    a, b = to_i128([f0, f1])
    _call("or_bconv_correct_pow2_wide", ctypes.byref(view(dst)), ctypes.byref(view(src, True)), ctypes.c_int64(a[0]),
          ctypes.c_int64(a[1]), ctypes.c_int64(b[0]), ctypes.c_int64(b[1]), ctypes.c_size_t(shift),
          ctypes.c_size_t(log2m))


def create_permutation(inner_shape, shifts):
    s, sh = _sz(inner_shape), _sz(shifts)
    n = int(np.prod(inner_shape)) if len(inner_shape) else 1
    out = np.zeros(n, dtype=np.uint32)
    _call("or_create_permutation", _p(s), _p(sh), ctypes.c_size_t(len(s)), _p(out))
    return out


def permute(dst, src, inner_shape, shifts, dim):
    s, sh = _sz(inner_shape), _sz(shifts)
    _call("or_permute", ctypes.byref(view(dst)), ctypes.byref(view(src)), _p(s), _p(sh), ctypes.c_size_t(len(s)),
          ctypes.c_int(dim))


def barrett(value, n, xs):
    xs = np.ascontiguousarray(np.asarray(xs, dtype=np.int64))
    out = np.zeros_like(xs)
    zu = np.zeros(2, dtype=np.int64)
    _call("or_barrett", ctypes.c_int64(value), ctypes.c_int64(n), _p(xs), ctypes.c_size_t(len(xs)), _p(out), _p(zu))
    return out, int(zu[0]), int(zu[1])


def mont_constants(prime):
    out = np.zeros(4, dtype=np.int64)
    _call("or_mont_constants", ctypes.c_int64(prime), _p(out))
    return [int(x) for x in out]


def mont_ops(prime, values):
    x = to_i128(values)
    out = np.zeros((len(values), 4), dtype=np.int64)
    _call("or_mont_ops", ctypes.c_int64(prime), _p(x), ctypes.c_size_t(len(values)), _p(out))
    return out


def factor_ntt(q, data, inverse, reduce_output, in_bound):
    data = np.ascontiguousarray(data, dtype=np.int64)
    b = ctypes.c_uint64(0)
    _call("or_factor_ntt", ctypes.c_int64(q), ctypes.c_size_t(len(data)), _p(data), ctypes.c_int(int(inverse)),
          ctypes.c_int(int(reduce_output)), ctypes.c_int64(in_bound), ctypes.byref(b))
    return data, int(b.value)


def plan_apply(q, inner_shape, data, elem_stride, vec_len, inverse, reduce_output):
    s = _sz(inner_shape)
    _call("or_plan_apply", ctypes.c_int64(q), _p(s), ctypes.c_size_t(len(s)), _p(data), ctypes.c_size_t(elem_stride),
          ctypes.c_size_t(vec_len), ctypes.c_int(int(inverse)), ctypes.c_int(int(reduce_output)))


def find_root_of_unity(q, n):
    return int(lib().or_find_root_of_unity(ctypes.c_int64(q), ctypes.c_size_t(n)))


# ---------------------------------------------------------------- field / ring / BFV
def field_info(name):
    out = np.zeros(64, dtype=np.uint64)
    _call("or_field_info", name.encode(), _p(out), ctypes.c_size_t(64))
    k = int(out[5])
    return {
        "m": int(out[0]), "deg_l": int(out[1]), "deg_lprime": int(out[2]), "deg_k": int(out[3]),
        "lprime_factors": int(out[4]), "rou_order": int(out[6]), "gal_ml": int(out[7]),
        "orders": [int(x) for x in out[8:8 + k]], "gens": [int(x) for x in out[8 + k:8 + 2 * k]],
    }


def gal_to_shift(name, g):
    info = field_info(name)
    out = np.zeros(len(info["orders"]), dtype=np.int64)
    _call("or_gal_to_shift", name.encode(), ctypes.c_uint64(g), _p(out))
    return [int(x) for x in out]


def splitmix64(state):
    """The reference's test rng (src/bfv.rs:880-886); `state` is a one-element list."""
    m = (1 << 64) - 1
    state[0] = (state[0] + 0x9E3779B97F4A7C15) & m
    z = state[0]
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    return z ^ (z >> 31)


def pos_repr(x, p):
    return int(x) % int(p)


def montgomery_repr(x, p):
    return (int(x) % p) * ((1 << 64) % p) % p


def from_mont(x, p):
    return (int(x) % p) * pow((1 << 64) % p, p - 2, p) % p


class Ring:
    """The oracle's RingContext (src/ring.rs:594-652) with its BFV layer."""

    def __init__(self, field, lo=None, hi=None, t_bits=0, raw_primes=None):
        self.field = field
        self.info = field_info(field)
        if raw_primes is not None:
            p = _primes(raw_primes)
            self.h = lib().or_ring_create_raw(field.encode(), _p(p), ctypes.c_size_t(len(p)))
        else:
            self.h = lib().or_ring_create(field.encode(), ctypes.c_size_t(lo), ctypes.c_size_t(hi),
                                          ctypes.c_size_t(t_bits))
        if not self.h:
            raise OracleError(lib().or_last_error().decode())
        self.h = ctypes.c_void_p(self.h)
        nf = lib().or_ring_num_factors(self.h)
        self.primes = [int(lib().or_ring_prime(self.h, ctypes.c_size_t(i))) for i in range(nf)]
        self.initial_len = int(lib().or_ring_initial_len(self.h))
        self.n = self.info["deg_l"]
        self.dl = self.info["deg_lprime"]
        self.dk = self.info["deg_k"]

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().or_ring_free(self.h)
        except Exception:
            pass

    def initial_base(self):
        return list(range(self.initial_len))

    def shape(self, count, r):
        return (count, r, self.dl, self.dk)

    def zeros(self, count, r):
        return np.zeros(self.shape(count, r), dtype=np.int64)

    def extension_base(self, base):
        b = _sz(base)
        out = np.zeros(len(self.primes), dtype=np.uint64)
        n = ctypes.c_size_t(0)
        _call("or_ring_extension_base", self.h, _p(b), ctypes.c_size_t(len(b)), _p(out), ctypes.byref(n))
        return [int(x) for x in out[:n.value]]

    def kernels(self, idx):
        out = np.zeros(2 * (self.dl + self.dk), dtype=np.int64)
        _call("or_ring_kernels", self.h, ctypes.c_size_t(idx), _p(out))
        dl, dk = self.dl, self.dk
        return out[:dl], out[dl:dl + dk], out[dl + dk:2 * dl + dk], out[2 * dl + dk:]

    def pb_to_crt(self, data, base, inverse=False):
        data = np.ascontiguousarray(data, dtype=np.int64).copy()
        b = _sz(base)
        _call("or_ring_pb_to_crt", self.h, _p(data), ctypes.c_size_t(data.shape[0]), _p(b), ctypes.c_size_t(len(b)),
              ctypes.c_int(int(inverse)))
        return data

    def crt_to_pb(self, data, base):
        return self.pb_to_crt(data, base, inverse=True)

    def bconv(self, src, src_base, dst_base):
        """Base conversion of a [count, r, ...] tensor (any trailing coefficient shape)."""
        src = np.ascontiguousarray(src, dtype=np.int64).copy()
        count, ncoef = src.shape[0], int(np.prod(src.shape[2:]))
        dst = np.zeros((count, len(dst_base)) + tuple(src.shape[2:]), dtype=np.int64)
        sb, db = _sz(src_base), _sz(dst_base)
        _call("or_ring_bconv", self.h, _p(dst), _p(db), ctypes.c_size_t(len(db)), _p(src), _p(sb),
              ctypes.c_size_t(len(sb)), ctypes.c_size_t(count), ctypes.c_size_t(ncoef))
        return dst

    def bconv_gadget(self, src, base, digits):
        src = np.ascontiguousarray(src, dtype=np.int64).copy()
        ncoef = int(np.prod(src.shape[2:]))
        dst = np.zeros((len(digits), len(base)) + tuple(src.shape[2:]), dtype=np.int64)
        b = _sz(base)
        dg = _sz([x for d in digits for x in d])
        _call("or_ring_bconv_gadget", self.h, _p(dst), _p(src), _p(b), ctypes.c_size_t(len(b)), _p(dg),
              ctypes.c_size_t(len(digits)), ctypes.c_size_t(ncoef))
        return dst

    def apply_galois(self, src, base, g):
        src = np.ascontiguousarray(src, dtype=np.int64)
        dst = np.zeros_like(src)
        b = _sz(base)
        _call("or_ring_apply_galois", self.h, _p(dst), _p(src), ctypes.c_size_t(src.shape[0]), _p(b),
              ctypes.c_size_t(len(b)), ctypes.c_uint64(g))
        return dst

    def mul(self, a, b, base):
        a = np.ascontiguousarray(a, dtype=np.int64)
        b = np.ascontiguousarray(b, dtype=np.int64)
        out = np.zeros_like(a)
        bb = _sz(base)
        _call("or_ring_mul", self.h, _p(a), _p(b), ctypes.c_size_t(a.shape[0]), _p(bb), ctypes.c_size_t(len(bb)),
              _p(out))
        return out

    def wide_freshness(self, data, extra):
        data = np.ascontiguousarray(data, dtype=np.int64)
        out = np.zeros_like(data)
        flags = np.zeros(4, dtype=np.int32)
        _call("or_wide_freshness", self.h, _p(data), ctypes.c_size_t(extra), _p(out), _p(flags))
        return out, [int(f) for f in flags]

    # ---- BFV ----
    def log2_alpha_for_sigma(self, base, sigma):
        b = _sz(base)
        return float(lib().or_bfv_log2_alpha_for_sigma(self.h, _p(b), ctypes.c_size_t(len(b)), ctypes.c_double(sigma)))

    def gen_sk(self, state):
        st = np.array([state[0]], dtype=np.uint64)
        out = self.zeros(1, self.initial_len)
        _call("or_bfv_gen_sk", self.h, _p(st), _p(out))
        state[0] = int(st[0])
        return out

    def enc(self, state, base, t, ptxt, sk, log2_alpha):
        st = np.array([state[0]], dtype=np.uint64)
        tt = to_i128([t])[0]
        m = to_i128(ptxt)
        b = _sz(base)
        out = self.zeros(2, len(base))
        _call("or_bfv_enc", self.h, _p(st), _p(b), ctypes.c_size_t(len(b)), ctypes.c_int64(tt[0]),
              ctypes.c_int64(tt[1]), _p(m), _p(np.ascontiguousarray(sk)), ctypes.c_double(log2_alpha), _p(out))
        state[0] = int(st[0])
        return out

    def _digits(self, digits):
        return _sz([x for d in digits for x in d])

    def gen_rk(self, state, sk, digits, log2_alpha):
        st = np.array([state[0]], dtype=np.uint64)
        out = np.zeros((len(digits), 2, self.initial_len, self.dl, self.dk), dtype=np.int64)
        dg = self._digits(digits)
        _call("or_bfv_gen_rk", self.h, _p(st), _p(np.ascontiguousarray(sk)), _p(dg), ctypes.c_size_t(len(digits)),
              ctypes.c_double(log2_alpha), _p(out))
        state[0] = int(st[0])
        return out

    def gen_ksk(self, state, base, old_sk, new_sk, digits, log2_alpha):
        st = np.array([state[0]], dtype=np.uint64)
        out = np.zeros((len(digits), 2, len(base), self.dl, self.dk), dtype=np.int64)
        b, dg = _sz(base), self._digits(digits)
        _call("or_bfv_gen_ksk", self.h, _p(st), _p(b), ctypes.c_size_t(len(b)), _p(np.ascontiguousarray(old_sk)),
              _p(np.ascontiguousarray(new_sk)), _p(dg), ctypes.c_size_t(len(digits)), ctypes.c_double(log2_alpha),
              _p(out))
        state[0] = int(st[0])
        return out

    def gen_gk(self, state, sk, g, digits, log2_alpha):
        st = np.array([state[0]], dtype=np.uint64)
        out = np.zeros((len(digits), 2, self.initial_len, self.dl, self.dk), dtype=np.int64)
        dg = self._digits(digits)
        _call("or_bfv_gen_gk", self.h, _p(st), _p(np.ascontiguousarray(sk)), ctypes.c_uint64(g), _p(dg),
              ctypes.c_size_t(len(digits)), ctypes.c_double(log2_alpha), _p(out))
        state[0] = int(st[0])
        return out

    def noisy_plaintext(self, ct, base, sk):
        out = self.zeros(1, len(base))
        b = _sz(base)
        _call("or_bfv_noisy_plaintext", self.h, _p(np.ascontiguousarray(ct)), _p(b), ctypes.c_size_t(len(b)),
              _p(np.ascontiguousarray(sk)), _p(out))
        return out

    def hom_mul(self, t, ct1, ct2, base, keys, digits, period_output=False):
        tt = to_i128([t])[0]
        b = _sz(base)
        out = self.zeros(2, len(base))
        dg = self._digits(digits)
        _call("or_bfv_hom_mul", self.h, ctypes.c_int64(tt[0]), ctypes.c_int64(tt[1]), _p(np.ascontiguousarray(ct1)),
              _p(np.ascontiguousarray(ct2)), _p(b), ctypes.c_size_t(len(b)), _p(np.ascontiguousarray(keys)), _p(dg),
              ctypes.c_size_t(len(digits)), ctypes.c_size_t(keys.shape[2]), ctypes.c_int(int(period_output)), _p(out))
        return out

    def hom_gal(self, ct, base, gs, keys, digits):
        b = _sz(base)
        g = np.ascontiguousarray(np.asarray(gs, dtype=np.uint64))
        out = np.zeros((len(gs), 2, len(base), self.dl, self.dk), dtype=np.int64)
        dg = self._digits(digits)
        _call("or_bfv_hom_gal", self.h, _p(np.ascontiguousarray(ct)), _p(b), ctypes.c_size_t(len(b)), _p(g),
              ctypes.c_size_t(len(gs)), _p(np.ascontiguousarray(keys)), _p(dg), ctypes.c_size_t(len(digits)),
              ctypes.c_size_t(keys.shape[3]), _p(out))
        return out

    def dbfv_enc(self, state, log2_b, log2_t, base, ptxt, sk, log2_alpha):
        """dbfv_enc (src/dbfv.rs:661-689): [2 digits, r, ...] CRT basis"""
        st = np.array([state[0]], dtype=np.uint64)
        digits = (log2_t - 1) // log2_b + 1
        m = to_i128(ptxt)
        b = _sz(base)
        out = self.zeros(2 * digits, len(base))
        _call("or_dbfv_enc", self.h, _p(st), ctypes.c_size_t(log2_b), ctypes.c_size_t(log2_t), _p(b),
              ctypes.c_size_t(len(b)), _p(m), _p(np.ascontiguousarray(sk)), ctypes.c_double(log2_alpha), _p(out))
        state[0] = int(st[0])
        return out

    def dbfv_reduce(self, log2_b, log2_t, ct_pb, base, bound=1):
        """dbfv_reduce (src/dbfv.rs:968-1032), period basis in and out"""
        ct = np.ascontiguousarray(ct_pb, dtype=np.int64)
        digits = (log2_t - 1) // log2_b + 1
        out = self.zeros(max(2 * digits, ct.shape[0]), len(base))
        rows = ctypes.c_size_t(0)
        b = _sz(base)
        _call("or_dbfv_reduce", self.h, ctypes.c_size_t(log2_b), ctypes.c_size_t(log2_t), _p(ct),
              ctypes.c_size_t(ct.shape[0] // 2), _p(b), ctypes.c_size_t(len(b)), ctypes.c_uint64(bound), _p(out),
              ctypes.byref(rows))
        return out[:rows.value]

    def dbfv_hom_mul(self, log2_b, log2_t, lhs_pb, rhs_pb, base, rk, digits, period_output=False):
        """dbfv_hom_mul (src/dbfv.rs:1034-1059): period-basis operands"""
        l = np.ascontiguousarray(lhs_pb, dtype=np.int64)
        r = np.ascontiguousarray(rhs_pb, dtype=np.int64)
        md = (log2_t - 1) // log2_b + 1
        out = self.zeros(2 * md, len(base))
        rows = ctypes.c_size_t(0)
        b = _sz(base)
        dg = self._digits(digits)
        _call("or_dbfv_hom_mul", self.h, ctypes.c_size_t(log2_b), ctypes.c_size_t(log2_t), _p(l),
              ctypes.c_size_t(l.shape[0] // 2), _p(r), ctypes.c_size_t(r.shape[0] // 2), _p(b), ctypes.c_size_t(len(b)),
              _p(np.ascontiguousarray(rk)), _p(dg), ctypes.c_size_t(len(digits)), ctypes.c_size_t(rk.shape[2]),
              ctypes.c_int(int(period_output)), _p(out), ctypes.byref(rows))
        return out[:rows.value]

    def dbfv_decrypt(self, ct_crt, base, sk, log2_b, log2_t):
        """dbfv_dec (src/dbfv.rs:699-722) on a CRT-basis ciphertext: centred plaintext coefficients"""
        t = 1 << log2_t
        res = [0] * self.n
        for i in range(ct_crt.shape[0] // 2):
            part = self.decrypt(ct_crt[2 * i:2 * i + 2], base, sk, t)
            mod_i = 1 << (log2_t - i * log2_b)
            for j in range(self.n):
                res[j] += cmod(part[j], mod_i) << (i * log2_b)
        return [cmod(v, t) for v in res]

    def lprime_element_tensor(self, base, coeffs):
        """[1, r, deg_L', 1] CRT-basis tensor of an L' element (src/ring.rs:1227-1250)."""
        b = _sz(base)
        words = np.ascontiguousarray(to_i128(list(coeffs)))
        out = np.zeros((1, len(base), self.dl, 1), dtype=np.int64)
        _call("or_ring_lprime_element_tensor", self.h, _p(b), ctypes.c_size_t(len(b)), _p(words), _p(out))
        return out

    def dbfv_hom_cyclic_transform(self, log2_b, log2_t, g, coeffs, ct, base, gks, digits):
        """hom_cyclic_transform_dbfv (src/bootstrap/homcrt.rs:369-429): ct [2 d, r, ...] CRT basis,
        coeffs a list of deg_L'-long integer lists, gks {automorphism: key [d_key, 2, r_key, ...]}."""
        b = _sz(base)
        ct = np.ascontiguousarray(ct, dtype=np.int64)
        words = np.zeros((max(1, len(coeffs)), self.dl, 2), dtype=np.int64)
        for i, c in enumerate(coeffs):
            for k, v in enumerate(c):
                w = to_i128([v])
                words[i, k] = w[0]
        items = sorted(gks.items())
        keys = np.ascontiguousarray(np.stack([k for _, k in items])) if items else np.zeros((1, 1, 2, 1, 1, 1), np.int64)
        gg = np.ascontiguousarray(np.asarray([g_ for g_, _ in items] or [0], dtype=np.uint64))
        mod_digits = (log2_t - 1) // log2_b + 1
        out = np.zeros((2 * mod_digits, len(base), self.dl, self.dk), dtype=np.int64)
        rows = ctypes.c_size_t(0)
        dg = self._digits(digits)
        _call("or_dbfv_hom_cyclic_transform", self.h, ctypes.c_size_t(log2_b), ctypes.c_size_t(log2_t),
              ctypes.c_uint64(g), _p(words), ctypes.c_size_t(len(coeffs)), _p(ct), ctypes.c_size_t(ct.shape[0] // 2),
              _p(b), ctypes.c_size_t(len(b)), _p(keys), _p(gg), ctypes.c_size_t(len(items)), _p(dg),
              ctypes.c_size_t(len(digits)), ctypes.c_size_t(keys.shape[3]), _p(out), ctypes.byref(rows))
        return out[:rows.value]

    def key_switch(self, c0, c1_pb, base, keys, digits):
        b = _sz(base)
        out = self.zeros(2, len(base))
        dg = self._digits(digits)
        _call("or_bfv_key_switch", self.h, _p(np.ascontiguousarray(c0)), _p(np.ascontiguousarray(c1_pb)), _p(b),
              ctypes.c_size_t(len(b)), _p(np.ascontiguousarray(keys)), _p(dg), ctypes.c_size_t(len(digits)),
              ctypes.c_size_t(keys.shape[2]), _p(out))
        return out

    def lift_to_extended(self, pb, base, crt=None):
        b = _sz(base)
        ext = self.extension_base(base)
        out = self.zeros(pb.shape[0], len(base) + len(ext))
        cp = _p(np.ascontiguousarray(crt)) if crt is not None else ctypes.c_void_p(0)
        _call("or_bfv_lift_to_extended", self.h, _p(np.ascontiguousarray(pb)), cp, ctypes.c_size_t(pb.shape[0]), _p(b),
              ctypes.c_size_t(len(b)), _p(out))
        return out

    def rescale_to_base(self, x, base, base_len, t):
        tt = to_i128([t])[0]
        b = _sz(base)
        out = self.zeros(x.shape[0], base_len)
        _call("or_bfv_rescale_to_base", self.h, _p(np.ascontiguousarray(x)), ctypes.c_size_t(x.shape[0]), _p(b),
              ctypes.c_size_t(len(b)), ctypes.c_size_t(base_len), ctypes.c_int64(tt[0]), ctypes.c_int64(tt[1]),
              _p(out))
        return out

    def mod_switch_down(self, x, base, new_len):
        b = _sz(base)
        out = self.zeros(x.shape[0], new_len)
        _call("or_bfv_mod_switch_down", self.h, _p(np.ascontiguousarray(x)), ctypes.c_size_t(x.shape[0]), _p(b),
              ctypes.c_size_t(len(b)), ctypes.c_size_t(new_len), _p(out))
        return out

    # ---- host-side decoding (src/bfv.rs:249-271, src/ring.rs:1465-1480) ----
    def element_lifts(self, data_mont, base):
        """Smallest lifts modulo Q(base) of all coefficients of one element [1, r, dl, dk]."""
        primes = [self.primes[i] for i in base]
        q = 1
        for p in primes:
            q *= p
        flat = data_mont.reshape(len(base), -1)
        n = flat.shape[1]
        acc = [0] * n
        for i, p in enumerate(primes):
            qi = q // p
            c = qi * pow(qi % p, p - 2, p)
            rinv = pow((1 << 64) % p, p - 2, p)
            col = flat[i]
            for j in range(n):
                acc[j] += (int(col[j]) % p) * rinv % p * c
        lifts = []
        for a in acc:
            a %= q
            if a > (q - 1) // 2:
                a -= q
            lifts.append(a)
        return lifts, q

    def decode_scaled(self, data_mont, base, t):
        lifts, q = self.element_lifts(data_mont, base)
        return [cmod(_rounded_div(lift * t, q), t) for lift in lifts]

    def decrypt(self, ct, base, sk, t):
        return self.decode_scaled(self.noisy_plaintext(ct, base, sk), base, t)

    def encode_scalar(self, x):
        scale = -1 if _num_m_factors(self.info["m"]) % 2 == 1 else 1
        return [x * scale] * self.n

    def decode_scalar(self, t, data_pb):
        val = data_pb[0]
        assert all(v == val for v in data_pb), "ring element doesn't store a scalar"
        scale = -1 if _num_m_factors(self.info["m"]) % 2 == 1 else 1
        return cmod(val * scale, t)


def _num_m_factors(m):
    count, p = 0, 3
    while m > 1:
        if m % p == 0:
            m //= p
            count += 1
        p += 2
    return count


def _rounded_div(a, b):
    return (a + b // 2) // b if a >= 0 else -((-a + b // 2) // b)


def cmod(a, modulus):
    """src/ring.rs:95-106 (truncating remainder, as Rust's `%`)."""
    half = modulus // 2
    r = abs(a) % modulus
    r = -r if a < 0 else r
    if abs(r) >= half:
        if r < 0:
            r += modulus
        elif r > half:
            r -= modulus
    return r


def select_digits(digits, rns_base_len):
    """src/bfv.rs:388-400"""
    per, large, cur, out = rns_base_len // digits, rns_base_len % digits, 0, []
    for i in range(digits):
        ln = per + 1 if i < large else per
        out.append((cur, cur + ln))
        cur += ln
    return out
