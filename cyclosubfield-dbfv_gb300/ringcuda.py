"""Python binding of include/ringcuda.h: the ring (cyclosubfield-dbfv/src/ring.rs) and BFV
(src/bfv.rs) operations of the GB300 backend, with the reference's names and argument meaning.
Tensors are :class:`halcuda.DeviceTensor` views; RNS bases are lists of factor indices."""
import ctypes

import numpy as np

import halcuda
from halcuda import HcModulus, check, lib


def _sz(values):
    return (ctypes.c_size_t * max(1, len(values)))(*[int(v) for v in values])


def _digits(digits):
    return _sz([x for d in digits for x in d]), ctypes.c_size_t(len(digits))


def _i128(v):
    v = int(v) & ((1 << 128) - 1)
    lo, hi = v & ((1 << 64) - 1), v >> 64
    return (ctypes.c_int64 * 2)(lo - (1 << 64) if lo >> 63 else lo, hi - (1 << 64) if hi >> 63 else hi)


def _null_view():
    v = halcuda.HcView()
    v.ptr = None
    return v


def select_digits(digits, rns_base_len):
    """src/bfv.rs:388-400"""
    per, large, cur, out = rns_base_len // digits, rns_base_len % digits, 0, []
    for i in range(digits):
        ln = per + 1 if i < large else per
        out.append((cur, cur + ln))
        cur += ln
    return out


class RingContext:
    """RingContext (src/ring.rs:594-652) on the GPU backend."""

    def __init__(self, field, log2_q_lo=None, log2_q_hi=None, t_bits=0, raw_primes=None, backend=None):
        self.backend = backend or halcuda.CudaBackend(0)
        h = ctypes.c_void_p()
        if raw_primes is not None:
            arr = (ctypes.c_int64 * len(raw_primes))(*raw_primes)
            check(lib().hc_ring_create_raw(self.backend.h, field.encode(), arr, ctypes.c_size_t(len(raw_primes)),
                                           ctypes.byref(h)))
        else:
            check(lib().hc_ring_create(self.backend.h, field.encode(), ctypes.c_size_t(log2_q_lo),
                                       ctypes.c_size_t(log2_q_hi), ctypes.c_size_t(t_bits), ctypes.byref(h)))
        self.h = h
        self.backend.add_dependent(self)
        L = lib()
        L.hc_ring_num_factors.restype = ctypes.c_size_t
        L.hc_ring_num_factors.argtypes = [ctypes.c_void_p]
        L.hc_ring_prime.restype = ctypes.c_int64
        L.hc_ring_prime.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        L.hc_ring_initial_len.restype = ctypes.c_size_t
        L.hc_ring_initial_len.argtypes = [ctypes.c_void_p]
        L.hc_bfv_log2_alpha_for_sigma.restype = ctypes.c_double
        self.primes = [int(L.hc_ring_prime(h, i)) for i in range(L.hc_ring_num_factors(h))]
        self.initial_len = int(L.hc_ring_initial_len(h))
        dims = (ctypes.c_size_t * 3)()
        check(L.hc_ring_dims(h, dims))
        self.n, self.dl, self.dk = int(dims[0]), int(dims[1]), int(dims[2])

    def close(self):
        if self.h and self.backend.h:
            lib().hc_ring_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- bookkeeping ----
    def initial_base(self):
        return list(range(self.initial_len))

    def shape(self, count, r):
        return (count, r, self.dl, self.dk)

    def allocate(self, count, r):
        return self.backend.hal_allocate_i64(self.shape(count, r))

    def tensor(self, arr):
        return self.backend.tensor(arr)

    def modulus(self, idx):
        m = HcModulus()
        check(lib().hc_ring_modulus(self.h, ctypes.c_size_t(idx), ctypes.byref(m)))
        return m

    def mods_for(self, base):
        return [self.modulus(i) for i in base]

    def extension_base(self, base):
        out = (ctypes.c_size_t * len(self.primes))()
        n = ctypes.c_size_t(0)
        check(lib().hc_ring_extension_base(self.h, _sz(base), ctypes.c_size_t(len(base)), out, ctypes.byref(n)))
        return [int(out[i]) for i in range(n.value)]

    def crt_kernels(self, idx):
        out = np.zeros(2 * (self.dl + self.dk), dtype=np.int64)
        check(lib().hc_ring_crt_kernels(self.h, ctypes.c_size_t(idx), out.ctypes.data_as(ctypes.c_void_p)))
        dl, dk = self.dl, self.dk
        return out[:dl], out[dl:dl + dk], out[dl + dk:2 * dl + dk], out[2 * dl + dk:]

    # ---- ring operations ----
    def pb_to_crt(self, t, base):
        check(lib().hc_ring_pb_to_crt(self.h, t.view(), _sz(base), ctypes.c_size_t(len(base))))

    def crt_to_pb(self, t, base):
        check(lib().hc_ring_crt_to_pb(self.h, t.view(), _sz(base), ctypes.c_size_t(len(base))))

    def bconv(self, dst, dst_base, src, src_base):
        check(lib().hc_ring_bconv(self.h, dst.view(), _sz(dst_base), ctypes.c_size_t(len(dst_base)), src.view(),
                                  _sz(src_base), ctypes.c_size_t(len(src_base))))

    def bconv_gadget(self, dst, src, base, digits):
        dg, nd = _digits(digits)
        check(lib().hc_ring_bconv_gadget(self.h, dst.view(), src.view(), _sz(base), ctypes.c_size_t(len(base)), dg,
                                         nd))

    def apply_galois(self, dst, src, base, g):
        check(lib().hc_ring_apply_galois(self.h, dst.view(), src.view(), _sz(base), ctypes.c_size_t(len(base)),
                                         ctypes.c_uint64(g)))

    # ---- BFV ----
    def log2_alpha_for_sigma(self, base, sigma):
        return float(lib().hc_bfv_log2_alpha_for_sigma(self.h, _sz(base), ctypes.c_size_t(len(base)),
                                                       ctypes.c_double(sigma)))

    @staticmethod
    def _state(state):
        return (ctypes.c_uint64 * 1)(state[0])

    def gen_sk(self, state):
        st = self._state(state)
        sk = self.allocate(1, self.initial_len)
        check(lib().hc_bfv_gen_sk(self.h, st, sk.view()))
        state[0] = int(st[0])
        return sk

    def gen_sk_uniform_ternary(self, state):
        """hc_bfv_gen_sk_uniform_ternary: every coefficient uniform in {-1, 0, 1}."""
        st = self._state(state)
        sk = self.allocate(1, self.initial_len)
        check(lib().hc_bfv_gen_sk_uniform_ternary(self.h, st, sk.view()))
        state[0] = int(st[0])
        return sk

    def enc(self, state, base, t, ptxt, sk, log2_alpha):
        st = self._state(state)
        words = np.zeros((self.n, 2), dtype=np.int64)
        for i, v in enumerate(ptxt):
            w = _i128(v)
            words[i, 0], words[i, 1] = w[0], w[1]
        ct = self.allocate(2, len(base))
        check(lib().hc_bfv_enc(self.h, st, _sz(base), ctypes.c_size_t(len(base)), _i128(t),
                               words.ctypes.data_as(ctypes.c_void_p), sk.view(), ctypes.c_double(log2_alpha),
                               ct.view()))
        state[0] = int(st[0])
        return ct

    def gen_ksk(self, state, base, old_sk, new_sk, digits, log2_alpha):
        st = self._state(state)
        keys = self.allocate(2 * len(digits), len(base))
        dg, nd = _digits(digits)
        check(lib().hc_bfv_gen_ksk(self.h, st, _sz(base), ctypes.c_size_t(len(base)), old_sk.view(), new_sk.view(),
                                   dg, nd, ctypes.c_double(log2_alpha), keys.view()))
        state[0] = int(st[0])
        return keys

    def gen_rk(self, state, sk, digits, log2_alpha):
        st = self._state(state)
        keys = self.allocate(2 * len(digits), self.initial_len)
        dg, nd = _digits(digits)
        check(lib().hc_bfv_gen_rk(self.h, st, sk.view(), dg, nd, ctypes.c_double(log2_alpha), keys.view()))
        state[0] = int(st[0])
        return keys

    def gen_gk(self, state, sk, g, digits, log2_alpha):
        st = self._state(state)
        keys = self.allocate(2 * len(digits), self.initial_len)
        dg, nd = _digits(digits)
        check(lib().hc_bfv_gen_gk(self.h, st, sk.view(), ctypes.c_uint64(g), dg, nd, ctypes.c_double(log2_alpha),
                                  keys.view()))
        state[0] = int(st[0])
        return keys

    def noisy_plaintext(self, ct, base, sk):
        out = self.allocate(1, len(base))
        check(lib().hc_bfv_noisy_plaintext(self.h, ct.view(), _sz(base), ctypes.c_size_t(len(base)), sk.view(),
                                           out.view()))
        return out

    def key_switch(self, c0, c1_pb, base, keys, digits):
        out = self.allocate(2, len(base))
        dg, nd = _digits(digits)
        check(lib().hc_bfv_key_switch(self.h, c0.view(), c1_pb.view(), _sz(base), ctypes.c_size_t(len(base)),
                                      keys.view(), dg, nd, out.view()))
        return out

    def key_switch_noalloc(self, c0, c1_pb, base, keys, digits, out):
        """hc_bfv_key_switch_noalloc: key_switch into a caller-provided `out` [2, r] without any
        device allocation (scratch in the library's static array; tables built by an earlier
        key_switch with the same base and digits)."""
        dg, nd = _digits(digits)
        check(lib().hc_bfv_key_switch_noalloc(self.h, c0.view(), c1_pb.view(), _sz(base), ctypes.c_size_t(len(base)),
                                              keys.view(), dg, nd, out.view()))
        return out

    def lift_to_extended(self, pb, base, crt=None):
        ext = self.extension_base(base)
        out = self.allocate(pb.shape[0], len(base) + len(ext))
        check(lib().hc_bfv_lift_to_extended(self.h, pb.view(), crt.view() if crt is not None else _null_view(),
                                            _sz(base), ctypes.c_size_t(len(base)), out.view()))
        return out

    def rescale_to_base(self, x, base, base_len, t):
        out = self.allocate(x.shape[0], base_len)
        check(lib().hc_bfv_rescale_to_base(self.h, x.view(), _sz(base), ctypes.c_size_t(len(base)),
                                           ctypes.c_size_t(base_len), _i128(t), out.view()))
        return out

    def mod_switch_down(self, x, base, new_len):
        out = self.allocate(x.shape[0], new_len)
        check(lib().hc_bfv_mod_switch_down(self.h, x.view(), _sz(base), ctypes.c_size_t(len(base)),
                                           ctypes.c_size_t(new_len), out.view()))
        return out

    def hom_mul(self, t, ct1, ct2, base, rk, digits, period_output=False, out=None):
        out = out if out is not None else self.allocate(ct1.shape[0], len(base))
        dg, nd = _digits(digits)
        check(lib().hc_bfv_hom_mul(self.h, _i128(t), ct1.view(), ct2.view(), _sz(base), ctypes.c_size_t(len(base)),
                                   rk.view(), dg, nd, ctypes.c_int(int(period_output)), out.view()))
        return out

    def hom_gal_batch(self, ct, base, g, gk, digits, out=None):
        """hc_bfv_hom_gal_batch: B ciphertexts [2B, r] under one automorphism g."""
        out = out if out is not None else self.allocate(ct.shape[0], len(base))
        dg, nd = _digits(digits)
        check(lib().hc_bfv_hom_gal_batch(self.h, ct.view(), _sz(base), ctypes.c_size_t(len(base)), ctypes.c_uint64(g),
                                         gk.view(), dg, nd, out.view()))
        return out

    def hom_gal(self, ct, base, gs, gks, digits):
        out = self.allocate(2 * len(gs), len(base))
        dg, nd = _digits(digits)
        garr = (ctypes.c_uint64 * max(1, len(gs)))(*gs)
        check(lib().hc_bfv_hom_gal(self.h, ct.view(), _sz(base), ctypes.c_size_t(len(base)), garr,
                                   ctypes.c_size_t(len(gs)), gks.view(), dg, nd, out.view()))
        return out


CRT_FORWARD, CRT_MUL, CRT_INVERSE = 1, 2, 4
CRT_ONE_LAUNCH = 8  # with the above: all slabs in one persistent launch (default: one per shape class)


class _CrtItem(ctypes.Structure):
    _fields_ = [("ring", ctypes.c_void_p), ("data", halcuda.HcView), ("op", halcuda.HcView),
                ("base", ctypes.POINTER(ctypes.c_size_t)), ("r", ctypes.c_size_t)]


class CrtLaunch(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int), ("ctas_per_sm", ctypes.c_int), ("logv", ctypes.c_int)]

    def as_tuple(self):
        return (self.threads, self.ctas_per_sm, self.logv)


class CrtBatch:
    """hc_crt_batch: batched CRT transforms of (ring, data, op, base) items, one persistent launch
    per shape class of their slabs; `ops` combines CRT_FORWARD, CRT_MUL and CRT_INVERSE. The
    tensors and rings must outlive the batch."""

    def __init__(self, items, ops, backend=None):
        if not items:
            raise ValueError("empty batch")
        self.backend = backend or items[0][0].backend
        # the batch holds device pointers into the items' tensors and rings: keep them alive
        self._items = list(items)
        self._keep = []
        arr = (_CrtItem * len(items))()
        for it, (ring, data, op, base) in enumerate(items):
            b = _sz(base)
            self._keep.append(b)
            arr[it].ring = ring.h
            arr[it].data = data.view()
            arr[it].op = op.view() if op is not None else _null_view()
            arr[it].base = ctypes.cast(b, ctypes.POINTER(ctypes.c_size_t))
            arr[it].r = len(base)
        h = ctypes.c_void_p()
        check(lib().hc_crt_batch_create(self.backend.h, arr, ctypes.c_size_t(len(items)), ctypes.c_int(ops),
                                        ctypes.byref(h)))
        self.h = h
        self.backend.add_dependent(self)
        lib().hc_crt_batch_num_slabs.restype = ctypes.c_size_t
        lib().hc_crt_batch_num_slabs.argtypes = [ctypes.c_void_p]
        self.num_slabs = int(lib().hc_crt_batch_num_slabs(h))

    def run(self):
        check(lib().hc_crt_batch_run(self.h))

    def tune(self, reps=3):
        out = CrtLaunch()
        check(lib().hc_crt_batch_tune(self.h, ctypes.c_int(reps), ctypes.byref(out)))
        return out.as_tuple()

    @property
    def launch(self):
        out = CrtLaunch()
        check(lib().hc_crt_batch_get_launch(self.h, ctypes.byref(out)))
        return out.as_tuple()

    @launch.setter
    def launch(self, shape):
        check(lib().hc_crt_batch_set_launch(self.h, ctypes.byref(CrtLaunch(*shape))))

    def close(self):
        if self.h and self.backend.h:
            lib().hc_crt_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Keyset:
    """hc_keyset: Galois keys of one gadget split, in HBM up to `hbm_budget_bytes`, the rest in
    pinned host memory and streamed in before use (replaces the reference's key offloading)."""

    def __init__(self, ring, digits, r_key, hbm_budget_bytes):
        self.ring, self.digits, self.r_key = ring, list(digits), r_key
        dg, nd = _digits(digits)
        h = ctypes.c_void_p()
        check(lib().hc_keyset_create(ring.h, dg, nd, ctypes.c_size_t(r_key), ctypes.c_size_t(int(hbm_budget_bytes)),
                                     ctypes.byref(h)))
        self.h = h
        ring.backend.add_dependent(self)

    def add(self, g, key):
        check(lib().hc_keyset_add(self.h, ctypes.c_uint64(g), key.view()))

    def stats(self):
        res, strm = ctypes.c_size_t(), ctypes.c_size_t()
        nk, nb = ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().hc_keyset_stats(self.h, ctypes.byref(res), ctypes.byref(strm), ctypes.byref(nk), ctypes.byref(nb)))
        return {"resident": res.value, "streamed": strm.value, "streamed_copies": nk.value,
                "streamed_bytes": nb.value}

    def close(self):
        if self.h and self.ring.backend.h:
            lib().hc_keyset_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def hom_gal_keyset(ring, ct, base, gs, ks):
    out = ring.allocate(2 * len(gs), len(base))
    garr = (ctypes.c_uint64 * max(1, len(gs)))(*gs)
    check(lib().hc_bfv_hom_gal_keyset(ring.h, ct.view(), _sz(base), ctypes.c_size_t(len(base)), garr,
                                      ctypes.c_size_t(len(gs)), ks.h, out.view()))
    return out


def hom_gal_batch_keyset(ring, ct, base, g, ks, out=None):
    """hc_bfv_hom_gal_batch_keyset: B ciphertexts [2B, r] under automorphism g, key from a keyset."""
    out = out if out is not None else ring.allocate(ct.shape[0], len(base))
    check(lib().hc_bfv_hom_gal_batch_keyset(ring.h, ct.view(), _sz(base), ctypes.c_size_t(len(base)),
                                            ctypes.c_uint64(g), ks.h, out.view()))
    return out


def dbfv_hom_cyclic_transform(ring, log2_b, log2_t, g, coeffs, ct, base, ks):
    """hom_cyclic_transform_dbfv on the GPU; returns a [rows, r, ...] device tensor."""
    digits = (log2_t - 1) // log2_b + 1
    words = np.zeros((max(1, len(coeffs)), ring.dl, 2), dtype=np.int64)
    for i, c in enumerate(coeffs):
        for k, v in enumerate(c):
            w = _i128(v)
            words[i, k, 0], words[i, k, 1] = w[0], w[1]
    out = ring.allocate(2 * digits, len(base))
    rows = ctypes.c_size_t(0)
    check(lib().hc_dbfv_hom_cyclic_transform(ring.h, ctypes.c_size_t(log2_b), ctypes.c_size_t(log2_t), ctypes.c_uint64(g),
                                             words.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(len(coeffs)),
                                             ct.view(), _sz(base), ctypes.c_size_t(len(base)), ks.h, out.view(),
                                             ctypes.byref(rows)))
    return out.rows(0, rows.value)


def dbfv_digits(log2_b, log2_t):
    return (log2_t - 1) // log2_b + 1


def dbfv_enc(ring, state, log2_b, log2_t, base, ptxt, sk, log2_alpha):
    """hc_dbfv_enc: [2 digits, r] CRT-basis dBFV ciphertext"""
    st = (ctypes.c_uint64 * 1)(state[0])
    words = np.zeros((ring.n, 2), dtype=np.int64)
    for i, v in enumerate(ptxt):
        w = _i128(v)
        words[i, 0], words[i, 1] = w[0], w[1]
    out = ring.allocate(2 * dbfv_digits(log2_b, log2_t), len(base))
    check(lib().hc_dbfv_enc(ring.h, st, ctypes.c_size_t(log2_b), ctypes.c_size_t(log2_t), _sz(base),
                            ctypes.c_size_t(len(base)), words.ctypes.data_as(ctypes.c_void_p), sk.view(),
                            ctypes.c_double(log2_alpha), out.view()))
    state[0] = int(st[0])
    return out


def dbfv_reduce(ring, log2_b, log2_t, ct_pb, base, bound=1):
    out = ring.allocate(max(2 * dbfv_digits(log2_b, log2_t), ct_pb.shape[0]), len(base))
    rows = ctypes.c_size_t(0)
    check(lib().hc_dbfv_reduce(ring.h, ctypes.c_size_t(log2_b), ctypes.c_size_t(log2_t), ct_pb.view(), _sz(base),
                               ctypes.c_size_t(len(base)), ctypes.c_uint64(bound), out.view(), ctypes.byref(rows)))
    return out.rows(0, rows.value)


def dbfv_hom_mul(ring, log2_b, log2_t, lhs_pb, rhs_pb, base, rk, digits, period_output=False):
    out = ring.allocate(2 * dbfv_digits(log2_b, log2_t), len(base))
    rows = ctypes.c_size_t(0)
    dg, nd = _digits(digits)
    check(lib().hc_dbfv_hom_mul(ring.h, ctypes.c_size_t(log2_b), ctypes.c_size_t(log2_t), lhs_pb.view(), rhs_pb.view(),
                                _sz(base), ctypes.c_size_t(len(base)), rk.view(), dg, nd,
                                ctypes.c_int(int(period_output)), out.view(), ctypes.byref(rows)))
    return out.rows(0, rows.value)
