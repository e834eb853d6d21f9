"""The reference crate's own ring and BFV call sequences, issued through the `hal::Backend` trait
entry points of include/halcuda.h and nothing else.

This is what the unchanged crate runs above a `hal::cuda` backend: `RingContext`
(cyclosubfield-dbfv/src/ring.rs) and `bfv_hom_mul` (src/bfv.rs:747-775) call the trait method by
method, with the crate's caches (transform kernels, BEHZ base-conversion matrices, gadget
matrices), its wide-accumulator bound bookkeeping and its allocations. The fused ring-level
entry points of include/ringcuda.h compute the same integers in far fewer launches; this module
exists to run and time the drop-in path itself, and its results are bit-identical to both.

Only `CudaBackend.hal_*` methods touch device data here. The ring handle supplies host-side facts
the crate keeps in its `RingContext` (the RNS primes, the extension base rule, the CRT kernels of
each prime, src/ring.rs:1338-1415), never device work.
"""
import numpy as np

from halcuda import DIM2, DIM3

# the cyclic orders of L'_q and K_q (FieldDescriptor::lq_cyclic_orders, split after the L' factors;
# src/ring.rs:1318-1326), keyed by (deg_L', deg_K)
NTT_SHAPES = {(12, 3072): ([4, 3], [2, 3, 8, 64]), (4, 12288): ([4], [3, 64, 64])}


def smallest_lift(x, p):
    """The representative of x mod p in [-(p-1)/2, (p-1)/2] (feanor-math's smallest_lift)."""
    x %= p
    return x - p if x > (p - 1) // 2 else x


def mont_repr(x, p):
    """x 2^64 mod p with the sign of x (Rust's truncating %, src/ring.rs:108)."""
    v = x << 64
    r = abs(v) % p
    return r if v >= 0 else -r


def _trunc_mod(a, p):
    r = abs(a) % p
    return r if a >= 0 else -r


def _prod(values):
    out = 1
    for v in values:
        out *= v
    return out


def clip_digits(digits, base_len):
    """src/bfv.rs:120-126"""
    return [(s, min(e, base_len)) for s, e in digits if s < base_len]


class Wide:
    """WideRingEls (src/ring.rs:330-532): an i128 batch, mont(+-1) per factor, the base's extreme
    primes and one worst-case bound per row (0 = fresh, overwritten by the first accumulation)."""

    def __init__(self, data, one, neg_one, max_p, min_p, count):
        self.data, self.one, self.neg_one = data, one, neg_one
        self.max_p, self.min_p = max_p, min_p
        self.bound = [0] * count

    def record_step(self, rows, step):
        for i in range(*rows):
            self.bound[i] += step
            if self.bound[i] > (1 << 127) - 1:
                raise OverflowError("wide ring element overflow: too many accumulation steps")

    def needs_full_reduction(self, row):
        return self.bound[row] > (self.min_p << 63)


class TraitRing:
    """RingContext's call sequences over the trait (src/ring.rs), with its per-base caches."""

    def __init__(self, ring):
        self.ring, self.be = ring, ring.backend
        self.p = ring.primes
        self.dl, self.dk = ring.dl, ring.dk
        self.lprime_shape, self.k_shape = NTT_SHAPES[(ring.dl, ring.dk)]
        self._mods, self._transform, self._bconv, self._gadget, self._scalars = {}, {}, {}, {}, {}

    # ---- bookkeeping (src/ring.rs:774-1060) ----
    def allocate(self, count, base):
        return self.be.hal_allocate_i64((count, len(base), self.dl, self.dk))

    def clone(self, src):
        out = self.be.hal_allocate_i64(src.shape)
        self.be.hal_assign(out, src)
        return out

    def mods_for(self, base):
        key = tuple(base)
        if key not in self._mods:
            self._mods[key] = [self.ring.modulus(i) for i in base]
        return self._mods[key]

    def modulus_of(self, base):
        return _prod(self.p[i] for i in base)

    def _import(self, values, shape):
        t = self.be.hal_allocate_i64(shape)
        self.be.hal_import(t, np.asarray(values, dtype=np.int64).reshape(shape))
        return t

    def scalar_tensor(self, base, scalar):
        """src/ring.rs:884-897: mont(scalar mod p) per factor, [1, r, 1, 1]. Cached per (base,
        scalar): the values are constants, which the crate re-imports on every call."""
        key = ("s", tuple(base), scalar)
        if key not in self._scalars:
            self._scalars[key] = self._import(
                [mont_repr(_trunc_mod(scalar, self.p[i]), self.p[i]) for i in base], (1, len(base), 1, 1))
        return self._scalars[key]

    def inverse_scalar_tensor(self, base, scalar):
        """src/ring.rs:1165-1178: mont(smallest_lift(scalar^-1 mod p)) per factor (cached)."""
        key = ("i", tuple(base), scalar)
        if key not in self._scalars:
            vals = [mont_repr(smallest_lift(pow(scalar % self.p[i], -1, self.p[i]), self.p[i]), self.p[i])
                    for i in base]
            self._scalars[key] = self._import(vals, (1, len(base), 1, 1))
        return self._scalars[key]

    def allocate_wide(self, count, base):
        """src/ring.rs:792-806 (no zeroing: fresh rows are overwritten)"""
        data = self.be.hal_allocate_i128((count, len(base), self.dl, self.dk))
        ps = [self.p[i] for i in base]
        return Wide(data, self.scalar_tensor(base, 1), self.scalar_tensor(base, -1), max(ps), min(ps), count)

    # ---- wide accumulation (src/ring.rs:369-485) ----
    def _accumulate(self, wide, rows, lhs, rhs):
        """Maximal runs of rows with equal freshness, one hal_mul_i64 (fresh) or hal_fma_i64 call
        each; operands of dimension-0 length 1 are broadcast."""
        def operand(t, run):
            return t if t.shape[0] == 1 else t.rows(run[0] - rows[0], run[1] - rows[0])

        start = rows[0]
        while start < rows[1]:
            fresh = wide.bound[start] == 0
            end = start + 1
            while end < rows[1] and (wide.bound[end] == 0) == fresh:
                end += 1
            dst = wide.data.rows(start, end)
            if fresh:
                self.be.hal_mul_i64(dst, operand(lhs, (start, end)), operand(rhs, (start, end)))
            else:
                self.be.hal_fma_i64(dst, operand(lhs, (start, end)), operand(rhs, (start, end)))
            start = end

    def wide_fma(self, wide, rows, lhs, lhs_bound, rhs, rhs_bound):
        self._accumulate(wide, rows, lhs, rhs)
        wide.record_step(rows, lhs_bound * rhs_bound * wide.max_p * wide.max_p)

    def wide_add(self, wide, rows, src, src_bound):
        self._accumulate(wide, rows, src, wide.one)
        wide.record_step(rows, src_bound * wide.max_p * wide.max_p)

    def wide_inner_product(self, wide, rows, terms):
        """src/ring.rs:460-485: one hal_inner_product_i64 over fresh rows."""
        if not all(wide.bound[i] == 0 for i in range(*rows)):
            raise ValueError("WideRingEls::inner_product requires fresh rows")
        self.be.hal_inner_product_i64(wide.data.rows(*rows), [t[0] for t in terms], [t[2] for t in terms])
        wide.record_step(rows, sum(lb * rb * wide.max_p * wide.max_p for _, lb, _, rb in terms))

    def reduce_wide_tensor(self, dst, wide, base, rows):
        """src/ring.rs:846-865"""
        mods = self.mods_for(base)
        start = rows[0]
        while start < rows[1]:
            full = wide.needs_full_reduction(start)
            end = start + 1
            while end < rows[1] and wide.needs_full_reduction(end) == full:
                end += 1
            d = dst.rows(start - rows[0], end - rows[0])
            w = wide.data.rows(start, end)
            if full:
                self.be.hal_red_mont64_double(d, w, mods)
                self.be.hal_i64_to_mont64(d, mods)
            else:
                self.be.hal_red_mont64(d, w, mods)
            start = end

    def reduce_wide(self, wide, base):
        out = self.allocate(len(wide.bound), base)
        self.reduce_wide_tensor(out, wide, base, (0, len(wide.bound)))
        return out

    # ---- basis transforms (src/ring.rs:1115-1161, 1268-1303) ----
    def transform_cache(self, base):
        key = tuple(base)
        if key not in self._transform:
            r = len(base)
            kl, kk, ikl, ikk = [], [], [], []
            pl, pk = [], []
            for i in base:
                m = self.ring.modulus(i)
                pl.append(self.be.hal_create_ntt_plan(m, self.lprime_shape))
                pk.append(self.be.hal_create_ntt_plan(m, self.k_shape))
                a, b, c, d = self.ring.crt_kernels(i)
                kl += list(a)
                kk += list(b)
                ikl += list(c)
                ikk += list(d)
            self._transform[key] = {
                "mods": self.mods_for(base), "lp": pl, "k": pk,
                "kl": self._import(kl, (1, r, self.dl, 1)), "kk": self._import(kk, (1, r, 1, self.dk)),
                "ikl": self._import(ikl, (1, r, self.dl, 1)), "ikk": self._import(ikk, (1, r, 1, self.dk))}
        return self._transform[key]

    def pb_to_crt_tensor(self, data, base):
        c = self.transform_cache(base)
        self.be.hal_ntt_mul_mont64_dim(data, c["lp"], DIM2, c["kl"], c["mods"])
        self.be.hal_ntt_mul_mont64_dim(data, c["k"], DIM3, c["kk"], c["mods"])
        self.be.hal_intt_mont64(data, c["lp"], c["k"])

    def crt_to_pb_tensor(self, data, base):
        c = self.transform_cache(base)
        self.be.hal_ntt_mul_mont64_dim(data, c["lp"], DIM2, c["ikl"], c["mods"])
        self.be.hal_ntt_mul_mont64_dim(data, c["k"], DIM3, c["ikk"], c["mods"])
        self.be.hal_intt_mont64(data, c["lp"], c["k"])

    # ---- BEHZ base conversion (src/ring.rs:1595-1702, 1714-1851) ----
    def bconv_cache(self, src_base, dst_base):
        key = (tuple(src_base), tuple(dst_base))
        if key not in self._bconv:
            r, rd = len(src_base), len(dst_base)
            ps = [self.p[i] for i in src_base]
            pd = [self.p[i] for i in dst_base]
            max_p, min_p = max(ps + pd), min(ps)
            q = _prod(ps)
            shift = max(64, (4 * r * max_p + 1).bit_length())
            qt = 1 << shift
            if (qt - 1) // min_p + 1 >= 1 << 63:
                raise ValueError("coefficients of correction vector don't fit into an i64")
            chunk = ((1 << 127) - 1) // (max_p * max_p)
            qinv = [smallest_lift(pow((q // p) % p, -1, p), p) for p in ps]
            mat = []
            for pj in pd:
                r2 = pow(2, 128, pj)
                mat += [smallest_lift((q // p) % pj * r2, pj) for p in ps]
            mat += [(2 * qt + p) // (2 * p) for p in ps]  # rounded_div(q~, p)
            qm = [smallest_lift(q % pj * (-(1 << 64)), pj) for pj in pd]
            self._bconv[key] = {"qinv": self._import(qinv, (1, r, 1, 1)), "mat": self._import(mat, (1, rd + 1, r, 1)),
                                "qm": self._import(qm, (1, rd, 1, 1)), "shift": shift, "chunk": chunk}
        return self._bconv[key]

    def bconv_tensors(self, dst, dst_base, src, src_base):
        """BConvCache::bconv (src/ring.rs:1663-1702); destroys src."""
        c = self.bconv_cache(src_base, dst_base)
        self._bconv_calls(dst, src, c, self.mods_for(src_base), self.mods_for(dst_base), len(src_base), len(dst_base))

    def _bconv_calls(self, dst, src, c, src_mods, dst_mods, r, rd):
        be = self.be
        be.hal_mul_mont64(src, c["qinv"], src_mods)
        rows = c["mat"].shape[0] if c["mat"].shape[0] > 1 else src.shape[0]
        correction = be.hal_allocate_i128((rows, 1, src.shape[2], src.shape[3]))
        tmp = be.hal_allocate_i128((rows, rd + 1, src.shape[2], src.shape[3]))
        for chunk, j in enumerate(range(0, r, c["chunk"])):
            e = min(j + c["chunk"], r)
            be.hal_matmul_i64(tmp, c["mat"].slice(None, None, (j, e)), src.slice(None, (j, e)))
            if chunk == 0:
                be.hal_red_mont64_double(dst, tmp.slice(None, (0, rd)), dst_mods)
                be.hal_assign_i128(correction, tmp.slice(None, (rd, rd + 1)))
            else:
                be.hal_add_red_mont64_double(dst, tmp.slice(None, (0, rd)), dst_mods)
                be.hal_add_i128(correction, tmp.slice(None, (rd, rd + 1)))
        be.hal_bconv_correct_mont64(dst, correction, c["qm"], dst_mods, c["shift"])
        be.hal_i64_to_mont64(dst, dst_mods)

    def gadget_cache(self, base, digits):
        key = (tuple(base), tuple(digits))
        if key not in self._gadget:
            r, d = len(base), len(digits)
            ps = [self.p[i] for i in base]
            max_p, min_p = max(ps), min(ps)
            maxlen = max(e - s for s, e in digits)
            shift = max(64, (4 * maxlen * max_p + 1).bit_length())
            qt = 1 << shift
            if (qt - 1) // min_p + 1 >= 1 << 63:
                raise ValueError("coefficients of correction vector don't fit into an i64")
            chunk = ((1 << 127) - 1) // (max_p * max_p)
            dinv = [0] * r
            mat = [0] * (d * (r + 1) * r)
            dm = []
            for i, (s, e) in enumerate(digits):
                dmod = _prod(ps[s:e])
                for u in range(s, e):
                    dinv[u] = smallest_lift(pow((dmod // ps[u]) % ps[u], -1, ps[u]), ps[u])
                for j in range(r):
                    pj = ps[j]
                    r2 = pow(2, 128, pj)
                    for u in range(s, e):
                        mat[(i * (r + 1) + j) * r + u] = smallest_lift((dmod // ps[u]) % pj * r2, pj)
                    dm.append(smallest_lift(dmod % pj * (-(1 << 64)), pj))
                for u in range(s, e):
                    mat[(i * (r + 1) + r) * r + u] = (2 * qt + ps[u]) // (2 * ps[u])
            self._gadget[key] = {"qinv": self._import(dinv, (1, r, 1, 1)), "mat": self._import(mat, (d, r + 1, r, 1)),
                                 "qm": self._import(dm, (d, r, 1, 1)), "shift": shift, "chunk": chunk}
        return self._gadget[key]

    def bconv_gadget_tensors(self, dst, src, base, digits):
        """GadgetBConvCache::bconv (src/ring.rs:1814-1851); destroys src."""
        c = self.gadget_cache(base, digits)
        mods = self.mods_for(base)
        self._bconv_calls(dst, src, c, mods, mods, len(base), len(base))


class TraitBfv:
    """The BFV layer's ciphertext multiplication (src/bfv.rs:408-775) over a TraitRing. Inputs
    and outputs are CRT-basis ciphertexts [2, r] with almost-reduced entries (bound 1); a
    relinearisation key is a [2 d, r_key] tensor (rows 2i, 2i + 1 = digit i) over a base that
    the ciphertext's base is a prefix of."""

    def __init__(self, trait_ring):
        self.tr = trait_ring

    def lift_to_extended(self, pb, base, crt):
        """src/bfv.rs:564-592 with the CRT-basis copy given (bound 1)"""
        tr = self.tr
        ext = tr.ring.extension_base(base)
        lifted = list(base) + ext
        r = len(base)
        result = tr.allocate(pb.shape[0], lifted)
        tmp = tr.clone(pb)
        tr.bconv_tensors(result.slice(None, (r, len(lifted))), ext, tmp, base)
        tr.pb_to_crt_tensor(result.slice(None, (r, len(lifted))), ext)
        tr.be.hal_assign(result.slice(None, (0, r)), crt)
        return result, lifted

    def rescale_to_base(self, x, lifted, base_len, t):
        """src/bfv.rs:597-622 (x in period basis over base + extension)"""
        tr = self.tr
        base, ext = lifted[:base_len], lifted[base_len:]
        count = x.shape[0]
        tr.be.hal_mul_mont64(x, tr.scalar_tensor(lifted, t), tr.mods_for(lifted))  # mul_scalar
        tmp = tr.allocate(count, ext)
        tr.bconv_tensors(tmp, ext, x.slice(None, (0, base_len)), base)
        xe = x.slice(None, (base_len, len(lifted)))
        tr.be.hal_sub_i64(xe, tmp)
        tr.be.hal_mul_mont64(xe, tr.inverse_scalar_tensor(ext, tr.modulus_of(base)), tr.mods_for(ext))
        result = tr.allocate(count, base)
        tr.bconv_tensors(result, base, xe, ext)
        return result

    def gadget_decompose(self, c1_pb, base, digits):
        """src/bfv.rs:408-426"""
        tr = self.tr
        result = tr.allocate(len(digits), base)
        tmp = tr.clone(c1_pb)
        tr.bconv_gadget_tensors(result, tmp, base, digits)
        tr.pb_to_crt_tensor(result, base)
        return result

    def key_switch_acc(self, acc, c1_pb, base, keys, digits):
        """src/bfv.rs:498-526: acc[0..2] = sum_i d_i ksk_i, the key restricted to the base"""
        digits = clip_digits(digits, len(base))
        parts = self.gadget_decompose(c1_pb, base, digits)
        terms = [(parts.rows(i, i + 1), 1, keys.slice((2 * i, 2 * i + 2), (0, len(base))), 1)
                 for i in range(len(digits))]
        if terms:
            self.tr.wide_inner_product(acc, (0, 2), terms)

    def relin(self, prod, base, rk, digits):
        """src/bfv.rs:699-741 with a CRT-basis output (prod: [3, r] period basis, bound 1)"""
        tr = self.tr
        acc = tr.allocate_wide(2, base)
        self.key_switch_acc(acc, prod.rows(2, 3), base, rk, digits)
        tr.pb_to_crt_tensor(prod.rows(0, 2), base)
        tr.wide_add(acc, (0, 2), prod.rows(0, 2), 1)
        return tr.reduce_wide(acc, base)

    def hom_mul(self, t, ct1, ct2, base, rk, digits, out=None):
        """bfv_hom_mul (src/bfv.rs:747-775): two CRT-basis ciphertexts [2, r] -> [2, r] (CRT basis).
        With `out`, the result is also copied there (one hal_assign the crate does not make), so
        that every allocation of the call is released before it returns, as a CUDA-graph capture
        of the call requires."""
        tr = self.tr

        def lift(ct):
            ct_pb = tr.clone(ct)
            tr.crt_to_pb_tensor(ct_pb, base)
            return self.lift_to_extended(ct_pb, base, ct)

        lhs, lifted = lift(ct1)
        rhs, _ = lift(ct2)
        acc = tr.allocate_wide(3, lifted)
        l0, l1, r0, r1 = lhs.rows(0, 1), lhs.rows(1, 2), rhs.rows(0, 1), rhs.rows(1, 2)
        tr.wide_fma(acc, (0, 1), l0, 1, r0, 1)  # hom_mul_raw_acc (src/bfv.rs:667-683)
        tr.wide_fma(acc, (1, 2), l0, 1, r1, 1)
        tr.wide_fma(acc, (1, 2), l1, 1, r0, 1)
        tr.wide_fma(acc, (2, 3), l1, 1, r1, 1)
        prod = tr.reduce_wide(acc, lifted)
        tr.crt_to_pb_tensor(prod, lifted)
        rescaled = self.rescale_to_base(prod, lifted, len(base), t)
        result = self.relin(rescaled, base, rk, digits)
        if out is None:
            return result
        tr.be.hal_assign(out, result)
        return out
