"""Pins the oracle's ring and BFV layers to the reference's known-answer tests
(cyclosubfield-dbfv/src/ring.rs:1854-2213, src/bfv.rs:888-1194)."""
import numpy as np
import pytest

BCONV_PRIMES = [  # src/ring.rs:1862-1876
    144115188075855859, 144115188075855847, 144115188075855823, 144115188075855811, 144115188075855803,
    144115188075855761, 144115188075855677, 144115188075855599, 144115188075855509, 144115188075855449,
    144115188075855439, 144115188075855421, 144115188075855413,
]


def trunc_mod(v, p):
    r = abs(v) % p
    return -r if v < 0 else r


def test_bconv_known_answers(po):
    """src/ring.rs:1859-1917"""
    rf = BCONV_PRIMES
    ring = po.Ring("field_2", raw_primes=rf)
    d1 = [0, 1, 2, 3, 4, 5, 6, 7]
    d2 = [1 << 64, 3 << 100, -7 << 100, 9 << 120, -1 << 120, 5 << 120, 0, 7 << 120]
    src = np.zeros((2, 7, 8, 1), dtype=np.int64)
    for i in range(7):
        for j in range(8):
            src[0, i, j, 0] = po.montgomery_repr(trunc_mod(d1[j], rf[i]), rf[i])
            src[1, i, j, 0] = po.montgomery_repr(trunc_mod(d2[j], rf[i]), rf[i])
    dst = ring.bconv(src, list(range(7)), list(range(7, 13)))
    for i in range(6):
        for j in range(8):
            assert int(dst[0, i, j, 0]) % rf[7 + i] == po.montgomery_repr(d1[j], rf[7 + i])
            assert int(dst[1, i, j, 0]) % rf[7 + i] == po.montgomery_repr(d2[j], rf[7 + i])


def test_bconv_gadget(po):
    """src/ring.rs:1919-1972: batched digit conversion == per-digit conversion."""
    rf = BCONV_PRIMES[:7]
    ring = po.Ring("field_2", raw_primes=rf)
    digits = [(0, 3), (3, 5), (5, 7)]
    data = [0, 1, -1 << 100, 3 << 100, -7 << 90, 9 << 120, 12345, 7 << 120]
    src = np.zeros((1, 7, 8, 1), dtype=np.int64)
    for i in range(7):
        for j in range(8):
            src[0, i, j, 0] = po.montgomery_repr(trunc_mod(data[j], rf[i]), rf[i])
    out = ring.bconv_gadget(src, list(range(7)), digits)
    for di, (s, e) in enumerate(digits):
        exp = ring.bconv(src[:, s:e], list(range(s, e)), list(range(7)))
        for i in range(7):
            assert [int(x) % rf[i] for x in exp[0, i, :, 0]] == [int(x) % rf[i] for x in out[di, i, :, 0]]


def test_pb_crt_transform_period_basis_relation(po):
    """src/ring.rs:1977-2012 (known answer computed with sage by the reference's authors)."""
    ring = po.Ring("field_18", 100, 120, 4)
    p = ring.primes[0]
    data = np.zeros((1, 1, 3, 6), dtype=np.int64)
    for block in range(3):
        data.reshape(-1)[block * 6] = po.montgomery_repr(1, p)
    crt = ring.pb_to_crt(data, [0])
    sq = ring.mul(crt, crt, [0])
    out = ring.crt_to_pb(sq, [0]).reshape(-1)
    exp = [3, 4, 2, -2, -4, -2]
    for block in range(3):
        for j in range(6):
            assert po.montgomery_repr(exp[j], p) == int(out[block * 6 + j]) % p


def test_pb_crt_roundtrip(po):
    """src/ring.rs:2014-2035"""
    ring = po.Ring("field_18", 100, 120, 4)
    base = ring.initial_base()
    state = 123
    vals = []
    for _ in range(2 * len(base) * 18):
        state = (state * 6364136223846793005 + 1442695040888963407) & ((1 << 64) - 1)
        vals.append((state >> 12) % 1000000)
    data = np.array(vals, dtype=np.int64).reshape(ring.shape(2, len(base)))
    out = ring.crt_to_pb(ring.pb_to_crt(data, base), base)
    for pos, (e, a) in enumerate(zip(data.reshape(-1), out.reshape(-1))):
        p = ring.primes[base[(pos // 18) % len(base)]]
        assert int(e) % p == int(a) % p


def test_crt_transform_multiply_small(po):
    """src/ring.rs:2037-2067"""
    ring = po.Ring("field_18", 100, 120, 4)
    p = ring.primes[0]
    data = np.zeros((1, 1, 3, 6), dtype=np.int64)
    data.reshape(-1)[0] = po.montgomery_repr(1, p)
    crt = ring.pb_to_crt(data, [0])
    out = ring.crt_to_pb(ring.mul(crt, crt, [0]), [0]).reshape(-1)
    for x in out:
        plain = po.from_mont(int(x), p)
        assert min(plain, p - plain) <= ring.info["m"]


def test_wide_freshness(po):
    """src/ring.rs:2118-2169"""
    ring = po.Ring("field_18", 100, 120, 4)
    base = ring.initial_base()
    r = len(base)
    values = [(pos % 50) + 1 for pos in range(4 * r * 18)]
    mont = [po.montgomery_repr(v, ring.primes[base[(pos // 18) % r]]) for pos, v in enumerate(values)]
    out, flags = ring.wide_freshness(np.array(mont, dtype=np.int64).reshape(ring.shape(4, r)), 100)
    assert flags[0] == 1 and flags[1] == 0
    for pos in range(4 * r * 18):
        p = ring.primes[base[(pos // 18) % r]]
        x = int(out.reshape(-1)[pos])
        assert abs(x) <= p
        mult = {0: 101, 1: 2, 2: 2}.get(pos // (r * 18), 1)
        assert (mult * values[pos]) % p == po.from_mont(x, p)


def test_apply_galois(po):
    """src/ring.rs:2171-2212"""
    ring = po.Ring("field_18", 100, 120, 4)
    base = [0, 1]
    data = np.arange(36, dtype=np.int64).reshape(1, 2, 3, 6)
    gens = ring.info["gens"]
    out = ring.apply_galois(data, base, gens[1]).reshape(-1)
    for j in range(2):
        for a0 in range(3):
            for a1 in range(2):
                for a2 in range(3):
                    src = j * 18 + (a0 * 2 + a1) * 3 + a2
                    dst = j * 18 + (a0 * 2 + (a1 + 1) % 2) * 3 + a2
                    assert data.reshape(-1)[src] == out[dst]
    g1, g2 = gens[0], gens[2]
    two = ring.apply_galois(ring.apply_galois(data, base, g1), base, g2)
    one = ring.apply_galois(data, base, g1 * g2 % ring.info["m"])
    assert (two == one).all()


# ------------------------------------------------------------------------------------- BFV
def _setup(po, field, lo, hi, t_bits, seed, digits_fn=None):
    ring = po.Ring(field, lo, hi, t_bits)
    base = ring.initial_base()
    la = ring.log2_alpha_for_sigma(base, 3.2)
    st = [seed]
    sk = ring.gen_sk(st)
    return ring, base, la, st, sk


def test_enc_dec(po):
    """src/bfv.rs:895-911"""
    ring, base, la, st, sk = _setup(po, "field_192", 100, 120, 8, 1)
    m = [(i % 255) - 127 for i in range(ring.n)]
    ct = ring.enc(st, base, 256, m, sk, la)
    assert ring.decrypt(ct, base, sk, 256) == m
    m2 = [2] * ring.n
    ct = ring.enc(st, base, 4, m2, sk, la)
    assert ring.decrypt(ct, base, sk, 4) == [po.cmod(2, 4)] * ring.n


def test_key_switch(po):
    """src/bfv.rs:977-996"""
    ring, base, la, st, sk1 = _setup(po, "field_192", 100, 120, 8, 2)
    m = [(i % 255) - 127 for i in range(ring.n)]
    sk2 = ring.gen_sk(st)
    ct1 = ring.enc(st, base, 256, m, sk1, la)
    digits = po.select_digits(len(base), len(base))
    ksk = ring.gen_ksk(st, base, sk1, sk2, digits, la)
    c1 = ring.crt_to_pb(ct1[1:2], base)
    ct2 = ring.key_switch(ct1[0:1], c1, base, ksk, digits)
    assert ring.decrypt(ct2, base, sk2, 256) == m


def test_hom_mul_scalar(po):
    """src/bfv.rs:998-1013"""
    ring, base, la, st, sk = _setup(po, "field_192", 100, 120, 8, 3)
    digits = po.select_digits(len(base), len(base))
    rk = ring.gen_rk(st, sk, digits, la)
    ct1 = ring.enc(st, base, 256, ring.encode_scalar(5), sk, la)
    ct2 = ring.enc(st, base, 256, ring.encode_scalar(7), sk, la)
    res = ring.hom_mul(256, ct1, ct2, base, rk, digits)
    assert ring.decode_scalar(256, ring.decrypt(res, base, sk, 256)) == 35


def test_hom_mul_large_t(po):
    """src/bfv.rs:1037-1057 (t = 2^64)."""
    ring, base, la, st, sk = _setup(po, "field_192", 200, 220, 64, 5)
    digits = po.select_digits(len(base) // 2, len(base))
    rk = ring.gen_rk(st, sk, digits, la)
    t = 1 << 64
    ct1 = ring.enc(st, base, t, ring.encode_scalar(3 << 24), sk, la)
    ct2 = ring.enc(st, base, t, ring.encode_scalar(5 << 23), sk, la)
    res = ring.hom_mul(t, ct1, ct2, base, rk, digits)
    assert ring.decode_scalar(t, ring.decrypt(res, base, sk, t)) == po.cmod(15 << 47, t)


def test_hom_gal_known_answer(po):
    """src/bfv.rs:1121-1140"""
    ring, base, la, st, sk = _setup(po, "field_18", 300, 320, 4, 6)
    digits = po.select_digits(len(base), len(base))
    g = ring.info["gens"][ring.info["lprime_factors"]]
    gk = ring.gen_gk(st, sk, g, digits, la)
    ptxt = [1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0]
    ct = ring.enc(st, base, 16, ptxt, sk, la)
    res = ring.hom_gal(ct, base, [g], gk[None], digits)
    assert ring.decrypt(res[0], base, sk, 16) == [0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0]


def test_mod_switch_down_dynamic_scaling(po):
    """src/bfv.rs:1164-1193"""
    ring, base, la, st, sk = _setup(po, "field_18", 300, 320, 16, 7)
    digits = po.select_digits(len(base), len(base))
    rk = ring.gen_rk(st, sk, digits, la)
    t = 1 << 16
    ct = ring.enc(st, base, t, ring.encode_scalar(2025), sk, la)
    ct_pb = ring.crt_to_pb(ct, base)
    small = min(3, len(base))
    sw = ring.pb_to_crt(ring.mod_switch_down(ct_pb, base, small), base[:small])
    assert ring.decode_scalar(t, ring.decrypt(sw, base[:small], sk, t)) == 2025
    mid = len(base) - 2
    swm = ring.pb_to_crt(ring.mod_switch_down(ct_pb, base, mid), base[:mid])
    res = ring.hom_mul(t, swm, swm, base[:mid], rk, digits)
    assert ring.decode_scalar(t, ring.decrypt(res, base[:mid], sk, t)) == po.cmod(2025 * 2025, t)


@pytest.mark.slow
def test_enc_dec_hom_mul_field_36864(po):
    """src/bfv.rs:1142-1162: the full-degree field."""
    ring, base, la, st, sk = _setup(po, "field_36864", 100, 120, 8, 8)
    m = [(i % 255) - 127 for i in range(ring.n)]
    ct = ring.enc(st, base, 256, m, sk, la)
    assert ring.decrypt(ct, base, sk, 256) == m
    digits = po.select_digits(len(base), len(base))
    rk = ring.gen_rk(st, sk, digits, la)
    ct1 = ring.enc(st, base, 256, ring.encode_scalar(5), sk, la)
    ct2 = ring.enc(st, base, 256, ring.encode_scalar(7), sk, la)
    res = ring.hom_mul(256, ct1, ct2, base, rk, digits)
    assert ring.decode_scalar(256, ring.decrypt(res, base, sk, 256)) == 35
