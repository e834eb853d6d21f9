"""Pins the oracle's backend methods to the reference's CPU-backend tests
(cyclosubfield-dbfv/src/hal/cpu.rs:1127-1876)."""
import numpy as np

from test_oracle_ntt import Lcg


def flat(shape, idx):
    return ((idx[0] * shape[1] + idx[1]) * shape[2] + idx[2]) * shape[3] + idx[3]


def lcg_vals(rng, n, mod, off):
    return np.array([rng.next() % mod - off for _ in range(n)], dtype=np.int64)


def test_add_sub_broadcast(po):
    """src/hal/cpu.rs:1218-1262"""
    shape = (2, 2, 3, 4)
    data = np.arange(48, dtype=np.int64).reshape(shape)
    dst = data.copy()
    po.add_i64(dst, np.array([10, 20], dtype=np.int64).reshape(1, 2, 1, 1))
    assert (dst == data + np.array([10, 20]).reshape(1, 2, 1, 1)).all()
    src_l = (np.arange(12, dtype=np.int64) * 100).reshape(2, 2, 3, 1)
    po.sub_i64(dst, src_l)
    assert (dst == data + np.array([10, 20]).reshape(1, 2, 1, 1) - src_l).all()
    d128 = po.to_i128([1] * 8, (2, 1, 2, 2))
    po.add_i128(d128, po.to_i128([5, 6, 7, 8], (1, 1, 2, 2)))
    assert list(po.from_i128(d128).reshape(-1)) == [6, 7, 8, 9, 6, 7, 8, 9]


def test_fma_and_matmul(po):
    """src/hal/cpu.rs:1264-1350"""
    shape = (2, 2, 3, 4)
    rng = Lcg(42)
    lhs = lcg_vals(rng, 48, 1000, 500).reshape(shape)
    rhs = lcg_vals(rng, 48, 1000, 500).reshape(shape)
    acc = po.to_i128([0] * 48, shape)
    po.fma_i64(acc, lhs, rhs)
    po.fma_i64(acc, lhs, rhs)
    assert (po.from_i128(acc) == 2 * lhs.astype(object) * rhs.astype(object)).all()
    prod = po.to_i128([-77] * 48, shape)
    po.mul_i64(prod, lhs, rhs)
    assert (po.from_i128(prod) == lhs.astype(object) * rhs.astype(object)).all()
    i_len, j_len, k_len, l_len, u_len = 2, 3, 2, 4, 5
    mm_l = lcg_vals(rng, j_len * u_len, 100, 50).reshape(1, j_len, u_len, 1)
    mm_r = lcg_vals(rng, i_len * u_len * k_len * l_len, 100, 50).reshape(i_len, u_len, k_len, l_len)
    dst = po.to_i128([-1] * 48, (i_len, j_len, k_len, l_len))
    po.matmul_i64(dst, mm_l, mm_r)
    po.matmul_i64(dst, mm_l, mm_r)
    exp = np.einsum("ju,iukl->ijkl", mm_l[0, :, :, 0].astype(object), mm_r.astype(object))
    assert (po.from_i128(dst) == exp).all()
    mm_lr = lcg_vals(rng, i_len * j_len * u_len, 100, 50).reshape(i_len, j_len, u_len, 1)
    mm_rb = lcg_vals(rng, u_len * k_len * l_len, 100, 50).reshape(1, u_len, k_len, l_len)
    po.matmul_i64(dst, mm_lr, mm_rb)
    exp = np.einsum("iju,ukl->ijkl", mm_lr[:, :, :, 0].astype(object), mm_rb[0].astype(object))
    assert (po.from_i128(dst) == exp).all()


def test_inner_product(po):
    """src/hal/cpu.rs:1352-1454"""
    shape = (2, 2, 3, 4)
    rng = Lcg(99)
    lhs = [lcg_vals(rng, 48, 1000, 500).reshape(shape) for _ in range(5)]
    rhs = [lcg_vals(rng, 48, 1000, 500).reshape(shape) for _ in range(5)]
    dst = po.to_i128([-123] * 48, shape)
    po.inner_product_i64(dst, lhs, rhs)
    exp = sum(l.astype(object) * r.astype(object) for l, r in zip(lhs, rhs))
    assert (po.from_i128(dst) == exp).all()
    chain = po.to_i128([7] * 48, shape)
    po.mul_i64(chain, lhs[0], rhs[0])
    for t in range(1, 5):
        po.fma_i64(chain, lhs[t], rhs[t])
    assert (chain == dst).all()
    lb = lcg_vals(rng, 24, 200, 100).reshape(1, 2, 3, 4)
    rb = lcg_vals(rng, 12, 200, 100).reshape(2, 2, 3, 1)
    bd = po.to_i128([0] * 48, shape)
    po.inner_product_i64(bd, [lb, lhs[0]], [rb, rhs[0]])
    exp = lb.astype(object) * rb.astype(object) + lhs[0].astype(object) * rhs[0].astype(object)
    assert (po.from_i128(bd) == exp).all()
    la, lb2, ra, rb2 = [lcg_vals(rng, 600, 1000, 500).reshape(1, 1, 1, 600) for _ in range(4)]
    ld = po.to_i128([-9] * 600, (1, 1, 1, 600))
    po.inner_product_i64(ld, [la, lb2], [ra, rb2])
    assert (po.from_i128(ld) == la.astype(object) * ra.astype(object) + lb2.astype(object) * rb2.astype(object)).all()


def test_mont_ops(po):
    """src/hal/cpu.rs:1456-1581"""
    primes = [97, 65537]
    shape = (2, 2, 3, 4)
    rng = Lcg(17)
    a = lcg_vals(rng, 48, 200, 100).reshape(shape)
    b = lcg_vals(rng, 48, 200, 100).reshape(shape)
    jidx = np.arange(48).reshape(shape)
    jp = lambda pos: primes[(pos // 12) % 2]
    a_mont = np.array([int(po.mont_ops(jp(p), [int(a.reshape(-1)[p])])[0, 2]) for p in range(48)],
                      dtype=np.int64).reshape(shape)
    dst = a_mont.copy()
    po.mul_mont64(dst, b, primes)
    for p in range(48):
        q = jp(p)
        assert abs(int(dst.reshape(-1)[p])) <= q
        assert int(dst.reshape(-1)[p]) % q == (int(a.reshape(-1)[p]) * int(b.reshape(-1)[p])) % q
    src = po.to_i128([(x - 24) * 1000000007 * 1000000007 for x in range(48)], shape)
    vals = po.from_i128(src).reshape(-1)
    acc = np.full(shape, 1000, dtype=np.int64)
    po.red128("add_red_mont64_double", acc, src, primes)
    over = np.full(shape, 1000, dtype=np.int64)
    po.red128("red_mont64_double", over, src, primes)
    assert (over == acc - 1000).all()
    for p in range(48):
        q = jp(p)
        red = int(acc.reshape(-1)[p]) - 1000
        assert abs(red) <= q and red * (1 << 128) % q == int(vals[p]) % q
    mont = np.zeros(shape, dtype=np.int64)
    po.red128("i128_to_mont64", mont, src, primes)
    acc2 = np.full(shape, 1000, dtype=np.int64)
    po.red128("add_red_mont64", acc2, src, primes)
    over2 = np.full(shape, 1000, dtype=np.int64)
    po.red128("red_mont64", over2, src, primes)
    assert (over2 == acc2 - 1000).all()
    for p in range(48):
        q = jp(p)
        assert abs(int(mont.reshape(-1)[p])) <= q
        assert int(mont.reshape(-1)[p]) % q == int(vals[p]) * (1 << 64) % q
        red = int(acc2.reshape(-1)[p]) - 1000
        assert abs(red) <= q and red * (1 << 64) % q == int(vals[p]) % q
    plain = np.array([(x - 24) * 187654321987654321 for x in range(48)], dtype=np.int64).reshape(shape)
    inp = plain.copy()
    po.i64_to_mont64(inp, primes)
    for p in range(48):
        q = jp(p)
        assert abs(int(inp.reshape(-1)[p])) <= q and int(inp.reshape(-1)[p]) % q == int(plain.reshape(-1)[p]) * (1 << 64) % q
    del jidx


def test_assign_narrow(po):
    """src/hal/cpu.rs:1583-1627"""
    shape = (2, 2, 3, 4)
    vals = [(x - 24) * 123456789123 for x in range(48)]
    src = po.to_i128(vals, shape)
    dst = np.zeros(shape, dtype=np.int64)
    po.assign_narrow(dst, src)
    assert list(dst.reshape(-1)) == vals
    bc = po.to_i128([x + 100 for x in range(6)], (1, 2, 3, 1))
    po.assign_narrow(dst, bc)
    for i in range(2):
        for j in range(2):
            for k in range(3):
                assert (dst[i, j, k] == j * 3 + k + 100).all()
    d128 = po.to_i128([-1] * 48, shape)
    po.assign_i128(d128, src)
    assert list(po.from_i128(d128).reshape(-1)) == vals
    big = po.to_i128([(x + 100) << 80 for x in range(6)], (1, 2, 3, 1))
    po.assign_i128(d128, big)
    out = po.from_i128(d128)
    for j in range(2):
        for k in range(3):
            assert (out[:, j, k] == (j * 3 + k + 100) << 80).all()


def test_bconv_correct_mont(po):
    """src/hal/cpu.rs:1629-1690"""
    primes = [97, 65537]
    shape = (2, 2, 2, 3)
    shift = 66
    small = [3, -7, 12, 0, 25, -1, 8, 4, -13, 6, 2, 9]
    lhs = po.to_i128([(s << shift) + ((s % 5) << 20) + 12345 for s in small], (2, 1, 2, 3))
    for rhs_vals, rshape in (([1001, -4242], (1, 2, 1, 1)), ([1001, -4242, 77, -33], (2, 2, 1, 1))):
        rhs = np.array(rhs_vals, dtype=np.int64).reshape(rshape)
        dst = np.full(shape, 500, dtype=np.int64)
        po.bconv_correct_mont64(dst, lhs, rhs, primes, shift)
        for i in range(2):
            for j in range(2):
                q = primes[j]
                for k in range(2):
                    for l in range(3):
                        out = int(dst[i, j, k, l]) - 500
                        r = rhs_vals[j] if rshape[0] == 1 else rhs_vals[i * 2 + j]
                        assert abs(out) <= q
                        assert out * (1 << 64) % q == small[(i * 2 + k) * 3 + l] * r % q


Q_NTT = 144115188075849889  # src/hal/cpu.rs:1696


def test_ntt_roundtrip(po):
    """src/hal/cpu.rs:1692-1724"""
    q = Q_NTT
    rng = Lcg(7)
    data = np.array([rng.next() % (2 * q) - q for _ in range(240)], dtype=np.int64)
    for shape, dim in (((2, 2, 12, 5), 2), ((2, 2, 5, 12), 3)):
        t = data.reshape(shape).copy()
        po.ntt_dim(t, [q, q], [4, 3], dim, "ntt")
        po.ntt_dim(t, [q, q], [4, 3], dim, "intt")
        assert all(int(a) % q == int(b) % q for a, b in zip(data, t.reshape(-1)))


def test_ntt_convolution_theorem(po):
    """src/hal/cpu.rs:1728-1772"""
    q = Q_NTT
    inner = [8, 9, 2]
    n = 144
    rng = Lcg(42)
    a = [rng.next() % 1000 - 500 for _ in range(n)]
    b = [rng.next() % 1000 - 500 for _ in range(n)]
    exp = [0] * n
    for i0 in range(8):
        for i1 in range(9):
            for i2 in range(2):
                for j0 in range(8):
                    for j1 in range(9):
                        for j2 in range(2):
                            d = (((i0 + j0) % 8) * 9 + (i1 + j1) % 9) * 2 + (i2 + j2) % 2
                            exp[d] += a[(i0 * 9 + i1) * 2 + i2] * b[(j0 * 9 + j1) * 2 + j2]
    at = np.array([po.montgomery_repr(x, q) for x in a], dtype=np.int64).reshape(1, 1, n, 1)
    bt = np.array([po.montgomery_repr(x, q) for x in b], dtype=np.int64).reshape(1, 1, n, 1)
    po.ntt_dim(at, [q], inner, 2, "ntt")
    po.ntt_dim(bt, [q], inner, 2, "ntt")
    po.mul_mont64(at, bt, [q])
    po.ntt_dim(at, [q], inner, 2, "intt")
    assert [po.montgomery_repr(e, q) for e in exp] == [int(x) % q for x in at.reshape(-1)]


def test_ntt_mul_mont64_dim(po):
    """src/hal/cpu.rs:1776-1827: the fused form equals transform-then-multiply, raw."""
    q = Q_NTT
    rng = Lcg(123)
    n = 24
    for dim, shape, kshape in ((2, (2, 2, n, 3), (1, 2, n, 1)), (3, (2, 2, 3, n), (1, 2, 1, n))):
        data = np.array([rng.next() % (4 * q) - 2 * q for _ in range(int(np.prod(shape)))], dtype=np.int64)
        data = data.reshape(shape)
        kern = np.array([po.montgomery_repr(rng.next() % (2 * q) - q, q) for _ in range(int(np.prod(kshape)))],
                        dtype=np.int64).reshape(kshape)
        ref = data.copy()
        po.ntt_dim(ref, [q, q], [8, 3], dim, "ntt")
        po.mul_mont64(ref, kern, [q, q])
        fused = data.copy()
        po.ntt_dim(fused, [q, q], [8, 3], dim, "ntt_mul", kern)
        assert (np.abs(fused) <= q).all()
        assert (ref == fused).all()


def test_permute(po):
    """src/hal/cpu.rs:1829-1875"""
    inner, shifts = [3, 4], [1, 2]
    data = np.arange(48, dtype=np.int64)
    s3 = data.reshape(1, 2, 2, 12)
    d3 = np.zeros_like(s3)
    po.permute(d3, s3, inner, shifts, 3)
    for j in range(2):
        for k in range(2):
            for a0 in range(3):
                for a1 in range(4):
                    assert d3[0, j, k, ((a0 + 1) % 3) * 4 + (a1 + 2) % 4] == s3[0, j, k, a0 * 4 + a1]
    s2 = data.reshape(1, 2, 12, 2)
    d2 = np.zeros_like(s2)
    po.permute(d2, s2, inner, shifts, 2)
    for j in range(2):
        for a0 in range(3):
            for a1 in range(4):
                assert (d2[0, j, ((a0 + 1) % 3) * 4 + (a1 + 2) % 4] == s2[0, j, a0 * 4 + a1]).all()
