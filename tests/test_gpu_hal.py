"""Bit-exact parity of every Backend method on the GPU (C-ABI library) against the oracle's
restatement of the reference's CPU backend, on the same seeded inputs: full-size field shapes,
broadcasting, strided views, empty and ragged shapes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Q57 = 144115188075835777
Q_NTT = 144115188075849889
Q62 = 4611686018427379009
Q61 = 3074457345618256921


@pytest.fixture(scope="module")
def primes36864(po):
    ring = po.Ring("field_36864", 900, 930, 8)
    return ring.primes


@pytest.fixture(scope="module")
def primes49152(po):
    ring = po.Ring("field_49152", 1280, 1310, 2)
    return ring.primes


def rng(seed):
    return np.random.default_rng(seed)


def residues(g, shape, primes, bound=1):
    """Entries of row j uniform in [-bound p_j, bound p_j]."""
    out = np.empty(shape, dtype=np.int64)
    for j in range(shape[1]):
        p = primes[j]
        out[:, j] = g.integers(-bound * p, bound * p, size=(shape[0],) + tuple(shape[2:]), endpoint=True)
    return out


def rand_i64(g, shape, lo=-(1 << 63), hi=(1 << 63) - 1):
    return g.integers(lo, hi, size=shape, dtype=np.int64, endpoint=True)


def rand_i128(g, shape, bits=127):
    lo = g.integers(-(1 << 63), (1 << 63) - 1, size=shape, dtype=np.int64, endpoint=True)
    if bits >= 127:
        hi = g.integers(-(1 << 63), (1 << 63) - 1, size=shape, dtype=np.int64, endpoint=True)
    else:
        hi = g.integers(-(1 << (bits - 64)), (1 << (bits - 64)) - 1, size=shape, dtype=np.int64, endpoint=True)
    return np.stack([lo, hi], axis=-1)


def mods(be, primes):
    return [be.hal_create_modulus(p) for p in primes]


def test_create_modulus_matches(be, po):
    for p in [97, 65537, Q57, Q_NTT, 144115188075855859, (1 << 61) - 1]:
        m = be.hal_create_modulus(p)
        assert [m.n, m.neg_inv_n, m.r2_mod_n, m.r3_mod_n] == po.mont_constants(p)


@pytest.mark.parametrize("dshape,sshape", [((2, 3, 4, 37), (2, 3, 4, 37)), ((2, 3, 4, 37), (1, 3, 1, 1)),
                                           ((2, 3, 4, 37), (2, 1, 4, 1)), ((3, 16, 12, 3072), (1, 16, 1, 3072)),
                                           ((0, 3, 4, 5), (1, 3, 4, 5))])
def test_add_sub_assign(be, po, dshape, sshape):
    g = rng(1)
    d0, s = rand_i64(g, dshape), rand_i64(g, sshape)
    for op in ("add_i64", "sub_i64", "assign"):
        exp = d0.copy()
        getattr(po, op)(exp, s)
        d = be.tensor(d0)
        getattr(be, "hal_" + op)(d, be.tensor(s))
        assert (d.to_numpy() == exp).all(), op


@pytest.mark.parametrize("dshape,sshape", [((2, 3, 4, 37), (2, 3, 4, 37)), ((2, 3, 4, 37), (1, 3, 4, 1))])
def test_i128_copies(be, po, dshape, sshape):
    g = rng(2)
    d0, s = rand_i128(g, dshape), rand_i128(g, sshape)
    exp = d0.copy()
    po.add_i128(exp, s)
    d = be.tensor(d0, wide=True)
    be.hal_add_i128(d, be.tensor(s, wide=True))
    assert (d.to_numpy() == exp).all()
    exp = d0.copy()
    po.assign_i128(exp, s)
    d = be.tensor(d0, wide=True)
    be.hal_assign_i128(d, be.tensor(s, wide=True))
    assert (d.to_numpy() == exp).all()
    n0 = rand_i64(g, dshape)
    exp = n0.copy()
    po.assign_narrow(exp, s)
    d = be.tensor(n0)
    be.hal_assign_narrow(d, be.tensor(s, wide=True))
    assert (d.to_numpy() == exp).all()


@pytest.mark.parametrize("lshape,rshape", [((2, 3, 4, 40), (2, 3, 4, 40)), ((1, 3, 4, 40), (2, 3, 4, 1)),
                                           ((1, 1, 1, 1), (2, 3, 4, 40))])
def test_fma_mul(be, po, lshape, rshape):
    g = rng(3)
    dshape = (2, 3, 4, 40)
    d0 = rand_i128(g, dshape)
    l, r = rand_i64(g, lshape), rand_i64(g, rshape)
    for op in ("fma_i64", "mul_i64"):
        exp = d0.copy()
        getattr(po, op)(exp, l, r)
        d = be.tensor(d0, wide=True)
        getattr(be, "hal_" + op)(d, be.tensor(l), be.tensor(r))
        assert (d.to_numpy() == exp).all(), op


def test_inner_product(be, po):
    g = rng(4)
    dshape = (2, 4, 12, 3072)
    terms = [((1, 4, 12, 3072), (2, 4, 12, 3072))] * 5 + [((2, 4, 12, 1), (1, 4, 1, 3072))]
    ls = [rand_i64(g, a) for a, _ in terms]
    rs = [rand_i64(g, b) for _, b in terms]
    exp = rand_i128(g, dshape)
    po.inner_product_i64(exp, ls, rs)
    d = be.tensor(rand_i128(g, dshape), wide=True)
    be.hal_inner_product_i64(d, [be.tensor(x) for x in ls], [be.tensor(x) for x in rs])
    assert (d.to_numpy() == exp).all()


@pytest.mark.parametrize("shapes", [((1, 35, 16, 1), (3, 16, 12, 3072)), ((2, 3, 5, 1), (2, 5, 2, 7)),
                                    ((2, 3, 5, 1), (1, 5, 2, 7)), ((4, 17, 16, 1), (1, 16, 3, 37))])
def test_matmul(be, po, shapes):
    g = rng(5)
    lshape, rshape = shapes
    I = max(lshape[0], rshape[0])
    dshape = (I, lshape[1], rshape[2], rshape[3])
    l = rand_i64(g, lshape, -(1 << 57), 1 << 57)
    r = rand_i64(g, rshape, -(1 << 57), 1 << 57)
    exp = rand_i128(g, dshape)
    po.matmul_i64(exp, l, r)
    d = be.tensor(rand_i128(g, dshape), wide=True)
    be.hal_matmul_i64(d, be.tensor(l), be.tensor(r))
    assert (d.to_numpy() == exp).all()


def test_montgomery_family(be, po, primes36864):
    g = rng(6)
    pr = primes36864[:16]
    M = mods(be, pr)
    shape = (3, 16, 12, 3072)
    # mul_mont64: products within 2^63 N (one factor reduced, the other arbitrary i64)
    d0 = rand_i64(g, shape)
    for sshape in [(1, 16, 1, 3072), (1, 16, 12, 1), (3, 16, 12, 3072)]:
        s = residues(g, sshape, pr)
        exp = d0.copy()
        po.mul_mont64(exp, s, pr)
        d = be.tensor(d0)
        be.hal_mul_mont64(d, be.tensor(s), M)
        assert (d.to_numpy() == exp).all(), sshape
    # reductions of i128 sources
    s128 = rand_i128(g, shape)
    s128_small = np.stack([rand_i64(g, shape), rand_i64(g, shape, -(1 << 55), 1 << 55)], axis=-1)
    for kind, src in (("add_red_mont64_double", s128), ("red_mont64_double", s128), ("add_red_mont64", s128_small),
                      ("red_mont64", s128_small), ("i128_to_mont64", s128_small)):
        exp = d0.copy()
        po.red128(kind, exp, src, pr)
        d = be.tensor(d0)
        getattr(be, "hal_" + kind)(d, be.tensor(src, wide=True), M)
        assert (d.to_numpy() == exp).all(), kind
    exp = d0.copy()
    po.i64_to_mont64(exp, pr)
    d = be.tensor(d0)
    be.hal_i64_to_mont64(d, M)
    assert (d.to_numpy() == exp).all()


# primes = 1 mod 192 of 40, 47, 52, 55, 58, 60, 61 and 61.4 bits
FAST_PRIMES = [1099511625409, 140737488355201, 4503599627367553, 36028797018963841, 288230376151711681,
               1152921504606844417, 2305843009213692097, 3074457345618256321]

NTT_CASES = [
    # (primes fixture or list, inner shape, tensor shape, dim)
    ("36864", [4, 3], (2, 16, 12, 3072), 2),
    ("36864", [2, 3, 8, 64], (2, 16, 12, 3072), 3),
    ("49152", [4], (2, 8, 4, 12288), 2),
    ("49152", [3, 64, 64], (1, 8, 4, 12288), 3),
    ([Q_NTT, Q_NTT], [4, 3], (2, 2, 12, 5), 2),
    ([Q_NTT, Q_NTT], [4, 3], (2, 2, 5, 12), 3),
    ([Q_NTT], [8, 9, 2], (1, 1, 144, 1), 2),
    ([Q_NTT, Q_NTT], [8, 3], (2, 2, 3, 24), 3),
    ([Q57, Q57], [16, 2], (2, 2, 3, 32), 3),
    ([Q57], [27, 1], (2, 1, 27, 9), 2),
    ([Q57], [4, 9], (3, 1, 5, 36), 3),
    ([Q57], [1, 1], (2, 1, 3, 1), 3),
    ([Q57], [], (2, 1, 1, 4), 2),
    ([Q62, Q62], [16, 2], (2, 2, 32, 3), 2),
    ([Q61], [27, 1], (2, 1, 4, 27), 3),
    ([Q61], [81], (1, 1, 81, 70), 2),
] + [
    # the factorisations with specialised kernels, over primes of 40..61.4 bits: the reduction
    # and skip schedule of the plan differs with the prime's size
    (FAST_PRIMES, [2, 3, 8, 64], (1, 8, 12, 3072), 3),
    (FAST_PRIMES, [4, 3], (2, 8, 12, 3072), 2),
    (FAST_PRIMES, [3, 64, 64], (1, 8, 4, 12288), 3),
    (FAST_PRIMES, [4], (1, 8, 4, 12288), 2),
    (FAST_PRIMES[:3], [4, 3], (1, 3, 12, 300), 2),
]


@pytest.mark.parametrize("case", NTT_CASES, ids=lambda c: "%s-%s-dim%d" % (c[1], c[2], c[3]))
def test_ntt_family(be, po, case, primes36864, primes49152):
    src, inner, shape, dim = case
    pr = {"36864": primes36864, "49152": primes49152}.get(src, src) if isinstance(src, str) else src
    pr = list(pr[:shape[1]])
    g = rng(7)
    data = residues(g, shape, pr, bound=2)
    M = mods(be, pr)
    plans = [be.hal_create_ntt_plan(m, inner) for m in M]
    kshape = (1, shape[1], shape[2], 1) if dim == 2 else (1, shape[1], 1, shape[3])
    kern = residues(g, kshape, pr)
    for mode in ("ntt", "intt", "ntt_mul"):
        exp = data.copy()
        po.ntt_dim(exp, pr, inner, dim, mode, kern if mode == "ntt_mul" else None)
        d = be.tensor(data)
        if mode == "ntt":
            be.hal_ntt_mont64_dim(d, plans, dim)
        elif mode == "intt":
            be.hal_intt_mont64_dim(d, plans, dim)
        else:
            be.hal_ntt_mul_mont64_dim(d, plans, dim, be.tensor(kern), M)
        got = d.to_numpy()
        assert (got == exp).all(), (mode, np.argwhere(got != exp)[:5])


@pytest.mark.parametrize("inner,shape,dim", [([2, 3, 8, 64], (2, 4, 12, 3072), 3), ([4, 3], (2, 4, 12, 3072), 2),
                                             ([3, 64, 64], (1, 4, 4, 12288), 3), ([4], (2, 4, 4, 12288), 2)])
def test_ntt_mul_full_operand(be, po, inner, shape, dim, primes36864, primes49152):
    """ntt_mul with a multiplier of the full tensor shape (no broadcasting) on the specialised shapes."""
    pr = list((primes36864 if shape[3] == 3072 else primes49152)[:shape[1]])
    g = rng(17)
    data = residues(g, shape, pr, bound=2)
    kern = residues(g, shape, pr)
    M = mods(be, pr)
    plans = [be.hal_create_ntt_plan(m, inner) for m in M]
    exp = data.copy()
    po.ntt_dim(exp, pr, inner, dim, "ntt_mul", kern)
    d = be.tensor(data)
    be.hal_ntt_mul_mont64_dim(d, plans, dim, be.tensor(kern), M)
    assert (d.to_numpy() == exp).all()


def test_ntt_strided_view(be, po, primes36864):
    """A transform on a strided sub-view (a slice of the RNS rows and of dimension 0) touches only
    the view, exactly like the reference's views (src/hal/cpu.rs:187-296)."""
    pr = primes36864[:20]
    g = rng(8)
    full = residues(g, (3, 20, 12, 3072), pr, bound=2)
    sub_pr = pr[4:12]
    M = mods(be, sub_pr)
    p2 = [be.hal_create_ntt_plan(m, [4, 3]) for m in M]
    p3 = [be.hal_create_ntt_plan(m, [2, 3, 8, 64]) for m in M]
    exp = full.copy()
    view = exp[1:3, 4:12]
    po.ntt_dim(view, sub_pr, [4, 3], 2, "ntt")
    po.ntt_dim(view, sub_pr, [2, 3, 8, 64], 3, "intt")
    d = be.tensor(full)
    dv = d.slice((1, 3), (4, 12))
    be.hal_ntt_mont64_dim(dv, p2, 2)
    be.hal_intt_mont64_dim(dv, p3, 3)
    assert (d.to_numpy() == exp).all()


def test_bconv_corrections(be, po):
    g = rng(9)
    pr = [144115188075855859, 144115188075855847, 144115188075855823]
    M = mods(be, pr)
    shape = (2, 3, 4, 50)
    lhs = rand_i128(g, (2, 1, 4, 50), bits=126)
    for rshape in [(1, 3, 1, 1), (2, 3, 1, 1)]:
        rhs = residues(g, rshape, pr)
        for shift in (64, 66, 100, 126):
            d0 = residues(g, shape, pr)
            exp = d0.copy()
            po.bconv_correct_mont64(exp, lhs, rhs, pr, shift)
            d = be.tensor(d0)
            be.hal_bconv_correct_mont64(d, be.tensor(lhs, wide=True), be.tensor(rhs), M, shift)
            assert (d.to_numpy() == exp).all(), (rshape, shift)
    src = rand_i128(g, (2, 2, 4, 50), bits=120)
    for shift, log2m in ((1, 1), (30, 62), (64, 20), (126, 40)):
        exp = rand_i64(g, (2, 1, 4, 50))
        d = be.tensor(exp)
        po.bconv_correct_pow2(exp, src, -123456789, 987654321, shift, log2m)
        be.hal_bconv_correct_pow2(d, be.tensor(src, wide=True), -123456789, 987654321, shift, log2m)
        assert (d.to_numpy() == exp).all(), (shift, log2m)
    src3 = rand_i128(g, (2, 3, 4, 50), bits=120)
    for shift, log2m in ((1, 64), (70, 126), (100, 90)):
        exp = rand_i64(g, (2, 2, 4, 50))
        d = be.tensor(exp)
        f0, f1 = -(3 << 90) + 12345, (5 << 70) + 77
        po.bconv_correct_pow2_wide(exp, src3, f0, f1, shift, log2m)
        be.hal_bconv_correct_pow2_wide(d, be.tensor(src3, wide=True), f0, f1, shift, log2m)
        assert (d.to_numpy() == exp).all(), (shift, log2m)


@pytest.mark.parametrize("inner,shifts,shape,dim", [([3, 4], [1, 2], (1, 2, 2, 12), 3), ([3, 4], [1, 2], (1, 2, 12, 2), 2),
                                                    ([2, 3, 8, 64], [1, 2, 5, 33], (2, 3, 12, 3072), 3),
                                                    ([4, 3], [3, 1], (2, 3, 12, 3072), 2),
                                                    ([3, 64, 64], [2, 17, 63], (1, 2, 4, 12288), 3)])
def test_permute(be, po, inner, shifts, shape, dim):
    g = rng(10)
    src = rand_i64(g, shape)
    exp = np.zeros_like(src)
    po.permute(exp, src, inner, shifts, dim)
    d = be.tensor(np.zeros_like(src))
    be.hal_permute(d, be.tensor(src), be.hal_create_permutation(inner, shifts), dim)
    assert (d.to_numpy() == exp).all()


def test_import_export_strided(be):
    """src/hal/cpu.rs:1141-1186: import into / export from a strided view touches only the view."""
    data = np.arange(120, dtype=np.int64).reshape(2, 3, 4, 5)
    t = be.tensor(data)
    v = t.slice((1, 2), (0, 2), (2, 4), (1, 4))
    assert (v.to_numpy() == data[1:2, 0:2, 2:4, 1:4]).all()
    patch = np.arange(1000, 1012, dtype=np.int64).reshape(1, 2, 2, 3)
    v.copy_from(patch)
    exp = data.copy()
    exp[1:2, 0:2, 2:4, 1:4] = patch
    assert (t.to_numpy() == exp).all()


def test_errors_are_reported(be):
    import halcuda

    a = be.hal_allocate_i64((2, 3, 4, 5))
    b = be.hal_allocate_i64((2, 2, 4, 5))
    with pytest.raises(halcuda.HalError, match="broadcast"):
        be.hal_add_i64(a, b)
    with pytest.raises(halcuda.HalError, match="modulus"):
        be.hal_mul_mont64(a, a, [be.hal_create_modulus(97)] * 2)


def test_runtime_stream_wait_and_barrett_peak(be):
    """hc_stream_wait_event orders work across streams (a copy on a second stream waits for a fill
    on the first); hc_barrett_peak returns a positive finite rate."""
    import math

    import halcuda

    n = 1 << 20
    src = be.hal_allocate_i64((1, 1, 1, n))
    dst = be.hal_allocate_i64((1, 1, 1, n))
    be.synchronize()
    halcuda.memset_async(be, src.ptr, 0x11, n * 8)
    ev = halcuda.Event()
    ev.record(be)
    s = halcuda.Stream()
    with be.on(s):
        ev.wait(be)
        halcuda.memcpy_async(be, dst.ptr, src.ptr, n * 8, halcuda.D2D)
        done = halcuda.Event()
        done.record(be)
    be.synchronize()
    done.elapsed_ms(done)
    assert (dst.to_numpy() == 0x1111111111111111).all()
    s.close()
    rate = halcuda.barrett_peak(be)
    assert math.isfinite(rate) and rate > 1e9


def test_int8_mma_peak(be):
    """hc_int8_mma_peak returns a positive finite multiply-add rate."""
    import math

    import halcuda

    rate = halcuda.int8_mma_peak(be)
    assert math.isfinite(rate) and rate > 1e11


def test_matmul_zero_columns_and_row_remainders(be, po):
    """A gadget-style conversion matrix [d, r + 1, r, 1], zero outside each digit's columns (the
    kernel skips all-zero column groups), with output row counts that are not multiples of four,
    57-bit and 63-bit right-hand values, against the oracle."""
    g = rng(41)
    d, r = 4, 16
    for rows, xbits in ((r + 1, 57), (6, 57), (3, 57), (r + 1, 63)):
        lhs = np.zeros((d, rows, r, 1), dtype=np.int64)
        for i in range(d):
            lhs[i, :, 4 * i:4 * i + 4, 0] = rand_i64(g, (rows, 4), -(1 << 56), (1 << 56) - 1)
        rhs = rand_i64(g, (1, r, 12, 64), -(1 << xbits), (1 << xbits) - 1)
        exp = rand_i128(g, (d, rows, 12, 64))
        po.matmul_i64(exp, lhs, rhs)
        out = be.tensor(rand_i128(g, (d, rows, 12, 64)), wide=True)
        be.hal_matmul_i64(out, be.tensor(lhs), be.tensor(rhs))
        assert (out.to_numpy() == exp).all(), rows


def test_line_grid_and_tile_paths_agree(be, po, primes36864):
    """The pointwise, inner-product and correction kernels run over a grid of destination lines
    while the line count fits the grid, and over tiles beyond it: both forms against the oracle
    (70000 lines of 4 positions, and 200 lines of 3072)."""
    g = rng(42)
    for shape in ((1, 70000, 1, 4), (2, 4, 25, 3072)):
        a, b = rand_i64(g, shape), rand_i64(g, shape)
        exp = a.copy()
        po.sub_i64(exp, b)
        da = be.tensor(a)
        be.hal_sub_i64(da, be.tensor(b))
        assert (da.to_numpy() == exp).all(), shape
        ls = [rand_i64(g, shape, -(1 << 57), 1 << 57) for _ in range(3)]
        rs = [rand_i64(g, shape, -(1 << 57), 1 << 57) for _ in range(3)]
        wexp = rand_i128(g, shape)
        po.inner_product_i64(wexp, ls, rs)
        dw = be.tensor(rand_i128(g, shape), wide=True)
        be.hal_inner_product_i64(dw, [be.tensor(x) for x in ls], [be.tensor(x) for x in rs])
        assert (dw.to_numpy() == wexp).all(), shape
    # the base-conversion correction over > 65535 destination lines
    pr = primes36864[:2]
    shape = (35000, 2, 1, 4)
    lhs = rand_i128(g, (35000, 1, 1, 4))
    rhs = residues(g, (1, 2, 1, 1), pr)
    dst = residues(g, shape, pr)
    exp = dst.copy()
    po.bconv_correct_mont64(exp, lhs, rhs, pr, 70)
    d = be.tensor(dst)
    be.hal_bconv_correct_mont64(d, be.tensor(lhs, wide=True), be.tensor(rhs), mods(be, pr), 70)
    assert (d.to_numpy() == exp).all()
