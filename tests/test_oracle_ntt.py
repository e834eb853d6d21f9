"""Pins the oracle's Barrett arithmetic and lazy NTT to the reference's own NTT tests
(cyclosubfield-dbfv/src/hal/ntt.rs:660-942), with the same constants, generators and checks."""
import numpy as np
import pytest

Q57 = 144115188075835777          # src/hal/ntt.rs:666
Q62_RADIX2 = 4611686018427379009  # src/hal/ntt.rs:669
Q61_RADIX3 = 3074457345618256921  # src/hal/ntt.rs:672
I64_MAX = (1 << 63) - 1
I64_MIN = -(1 << 63)


class Lcg:
    """src/hal/ntt.rs:674-684"""

    def __init__(self, state):
        self.state = state

    def next(self):
        self.state = (self.state * 6364136223846793005 + 1442695040888963407) & ((1 << 64) - 1)
        return self.state >> 33

    def entry(self, bound):
        a = self.next()
        b = self.next()
        c = self.next()
        r = (a << 62) ^ (b << 31) ^ c
        return r % (2 * bound + 1) - bound


def test_barrett_mul(po):
    """src/hal/ntt.rs:697-717"""
    for n in [97, 65537, Q57, Q62_RADIX2, Q61_RADIX3]:
        rng = Lcg(1)
        values = [0, 1, -1, n - 1, -(n - 1), (n - 1) // 2, -((n - 1) // 2)]
        values += [rng.entry(n - 1) for _ in range(20)]
        inputs = [0, 1, -1, I64_MAX, I64_MIN, I64_MIN + 1, n, -n, 2 * min(n, I64_MAX // 2), 123456789123456789 % n]
        for z in values:
            out, _, _ = po.barrett(z, n, inputs)
            for x, o in zip(inputs, out):
                assert abs(int(o)) <= n
                assert (z * x) % n == int(o) % n, (z, x, n)


def _forward(po, q, data):
    out, bound = po.factor_ntt(q, np.array(data, dtype=np.int64), False, False, 2 * q)
    return out, bound


@pytest.mark.parametrize("q,lens", [(Q57, [2, 4, 16, 128, 3, 9, 81]), (Q62_RADIX2, [2, 4, 16]),
                                    (Q61_RADIX3, [3, 9, 27, 81])])
def test_forward_is_permuted_dft(po, q, lens):
    """src/hal/ntt.rs:724-773"""
    for ln in lens:
        root = po.find_root_of_unity(q, ln)
        roots = [pow(root, e, q) for e in range(ln)]
        x_poly = [0] * ln
        x_poly[1] = 1
        tx, _ = _forward(po, q, x_poly)
        leaf = [roots.index(int(o) % q) for o in tx]
        assert len(set(leaf)) == ln
        rng = Lcg(42 + ln)
        data = [rng.entry(2 * q) for _ in range(ln)]
        tr, out_bound = _forward(po, q, data)
        assert out_bound <= I64_MAX
        for p, e in enumerate(leaf):
            assert abs(int(tr[p])) <= out_bound
            expected = sum((x % q) * roots[(e * j) % ln] for j, x in enumerate(data)) % q
            assert expected == int(tr[p]) % q


@pytest.mark.parametrize("q,lens", [(Q57, [2, 4, 16, 128, 3, 9, 81]), (Q62_RADIX2, [2, 4, 16]),
                                    (Q61_RADIX3, [3, 9, 27, 81])])
def test_factor_roundtrip(po, q, lens):
    """src/hal/ntt.rs:779-804"""
    for ln in lens:
        rng = Lcg(7 + ln)
        extreme = [2 * q, -2 * q] + [[2 * q, -2 * q, 0, q, -q][rng.next() % 5] for _ in range(2, ln)]
        random = [rng.entry(2 * q) for _ in range(ln)]
        for data in (extreme, random):
            fw, bound = _forward(po, q, data)
            bw, bound2 = po.factor_ntt(q, fw, True, False, bound)
            assert bound2 <= I64_MAX
            for pos in range(ln):
                assert (data[pos] * ln) % q == int(bw[pos]) % q


def test_strided_vectorized(po):
    """src/hal/ntt.rs:809-869: strided/vectorised == contiguous, bitwise."""
    q = Q57
    for shape, inverses in (([16], [False]), ([27], [False]), ([4, 3, 2], [False, True])):
        ln = int(np.prod(shape))
        elem_stride, vec_len = 7, 3
        rng = Lcg(99 if shape != [4, 3, 2] else 77)
        strided = np.zeros(ln * elem_stride, dtype=np.int64)
        cols = np.zeros((vec_len, ln), dtype=np.int64)
        for i in range(ln):
            for l in range(vec_len):
                v = rng.entry(2 * q)
                strided[i * elem_stride + l] = v
                cols[l, i] = v
        for inverse in inverses:
            reduce = shape == [4, 3, 2]
            po.plan_apply(q, shape, strided, elem_stride, vec_len, inverse, reduce)
            for l in range(vec_len):
                c = np.ascontiguousarray(cols[l])
                po.plan_apply(q, shape, c, 1, 1, inverse, reduce)
                cols[l] = c
            for i in range(ln):
                for l in range(vec_len):
                    assert cols[l, i] == strided[i * elem_stride + l]


@pytest.mark.parametrize("q,shape", [(Q57, [16, 2]), (Q57, [27, 1]), (Q57, [4, 9]), (Q57, [1, 1]),
                                     (Q62_RADIX2, [16, 2]), (Q61_RADIX3, [27, 1])])
def test_plan_roundtrip_and_convolution(po, q, shape):
    """src/hal/ntt.rs:876-941"""
    ln = shape[0] * shape[1]
    rng = Lcg(5)
    a = [rng.entry(2 * q) for _ in range(ln)]
    b = [rng.entry(q // 4) for _ in range(ln)]
    expected = [0] * ln
    for i0 in range(shape[0]):
        for i1 in range(shape[1]):
            for j0 in range(shape[0]):
                for j1 in range(shape[1]):
                    dst = ((i0 + j0) % shape[0]) * shape[1] + (i1 + j1) % shape[1]
                    expected[dst] += (a[i0 * shape[1] + i1] % q) * b[j0 * shape[1] + j1]
    data = np.array(a, dtype=np.int64)
    po.plan_apply(q, shape, data, 1, 1, False, True)
    assert all(abs(int(x)) <= q for x in data)
    po.plan_apply(q, shape, data, 1, 1, True, True)
    assert all(abs(int(x)) <= q for x in data)
    assert [x % q for x in a] == [int(x) % q for x in data]

    ah, bh = np.array(a, dtype=np.int64), np.array(b, dtype=np.int64)
    po.plan_apply(q, shape, ah, 1, 1, False, True)
    po.plan_apply(q, shape, bh, 1, 1, False, True)
    prod = np.array([(int(x) * int(y)) % q for x, y in zip(ah, bh)], dtype=np.int64)
    po.plan_apply(q, shape, prod, 1, 1, True, True)
    assert [e % q for e in expected] == [int(x) % q for x in prod]

    red, unred = np.array(a, dtype=np.int64), np.array(a, dtype=np.int64)
    po.plan_apply(q, shape, red, 1, 1, False, True)
    po.plan_apply(q, shape, unred, 1, 1, False, False)
    assert [int(x) % q for x in red] == [int(x) % q for x in unred]


def test_mont_constants_match_definitions(po):
    """src/hal/mont.rs:13-33: -N^-1 mod 2^64 and R^2, R^3 mod N in (0, N]."""
    for n in [97, 65537, Q57, 144115188075855859]:
        N, neg_inv, r2, r3 = po.mont_constants(n)
        assert (N * neg_inv) % (1 << 64) == (1 << 64) - 1
        assert r2 == ((1 << 128) % n or n)
        assert r3 == ((1 << 192) % n or n)


def test_mont_reductions(po):
    """src/hal/mont.rs:41-76: congruences and output ranges of the reductions."""
    for n in [97, 65537, 144115188075849889]:
        vals = [0, 1, -1, (1 << 63) * n, -(1 << 63) * n, 12345678901234567890123, -(1 << 126), (1 << 127) - 1,
                -(1 << 127)]
        out = po.mont_ops(n, vals)
        rinv = pow(1 << 64, -1, n)
        for v, (r1, r2, tm, tm64) in zip(vals, out):
            if abs(v) <= (1 << 63) * n + n:
                assert abs(int(r1)) <= n and int(r1) % n == v * rinv % n
                assert abs(int(tm)) <= n and int(tm) % n == v * (1 << 64) % n
            assert abs(int(r2)) <= n and int(r2) % n == v * rinv * rinv % n
            lo = ((v % (1 << 64)) ^ (1 << 63)) - (1 << 63)
            assert abs(int(tm64)) <= n and int(tm64) % n == lo * (1 << 64) % n
