"""The oracle's restatement of the homomorphic CRT transform step (hom_cyclic_transform_dbfv,
src/bootstrap/homcrt.rs:369-429), checked by decryption: the homomorphic result on a real
dBFV encryption must decrypt to the plaintext transform sum_i c_i sigma^i(m), computed without
keys on a noiseless encoding of m. Also the baby-step / giant-step split of the reference."""
import numpy as np
import pytest


def bsgs_split(n):
    """src/bootstrap/homcrt.rs:335-339"""
    best = min(range(1, n + 1), key=lambda c: (c + 3 * ((n - 1) // c + 1), c))
    return best, (n - 1) // best + 1


def pow_mod(g, e, m):
    r = 1
    for _ in range(e):
        r = r * g % m
    return r


def test_bsgs_split_matches_reference_rule():
    # first minimum of count + 3 * ceil(len / count), as Iterator::min_by_key returns it
    assert bsgs_split(1) == (1, 1)
    assert bsgs_split(3) == (3, 1)
    assert bsgs_split(8) == (4, 2)
    assert bsgs_split(64) == (13, 5)


def cmod(x, t):
    r = int(x) % t
    return r - t if r > t // 2 else r


def dbfv_decrypt(o, ct, base, sk, log2_b, log2_t):
    """dbfv_dec (src/dbfv.rs:699-722)"""
    t = 1 << log2_t
    d = ct.shape[0] // 2
    res = [0] * o.n
    for i in range(d):
        part = o.decrypt(ct[2 * i:2 * i + 2], base, sk, t)
        for j in range(o.n):
            res[j] += cmod(part[j], 1 << (log2_t - i * log2_b)) << (i * log2_b)
    return [cmod(v, t) for v in res]


@pytest.mark.parametrize("length,log2_b,log2_t,digits_ct", [(8, 4, 8, 2), (1, 4, 8, 2), (3, 3, 9, 1), (10, 8, 8, 1)])
def test_hom_cyclic_transform_decrypts_to_plain_transform(po, length, log2_b, log2_t, digits_ct):
    o = po.Ring("field_18", 300, 320, 4)
    base = o.initial_base()
    t = 1 << log2_t
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [41 + length]
    sk = o.gen_sk(st)
    g = 932  # generator of order 3 of the Galois group of field_18 (src/field.rs, field_18())
    m_field = o.info["m"]
    rng = np.random.default_rng(length)
    msg = [int(v) for v in rng.integers(0, t, size=o.n)]
    coeffs = [[int(v) for v in rng.integers(-300, 300, size=o.dl)] for _ in range(length)]
    # dBFV encryption without the canonical reduction: digit 0 encrypts m, the others zero
    parts = [o.enc(st, base, t, msg, sk, la)] + [o.enc(st, base, t, [0] * o.n, sk, la) for _ in range(digits_ct - 1)]
    ct = np.concatenate(parts, axis=0)
    baby, giant = bsgs_split(length)
    gs = [pow_mod(g, j, m_field) for j in range(1, baby)] + ([pow_mod(g, baby, m_field)] if giant > 1 else [])
    digits = po.select_digits(3, len(base))
    gks = {gg: o.gen_gk(st, sk, gg, digits, la) for gg in sorted(set(gs))}
    res = o.dbfv_hom_cyclic_transform(log2_b, log2_t, g, coeffs, ct, base, gks, digits)
    got = dbfv_decrypt(o, res, base, sk, log2_b, log2_t)

    # the plain transform on a noiseless encoding: c0 of an encryption under the zero key with a
    # vanishing error is exactly Delta m; sum_i c_i sigma^i(Delta m), decrypted with c1 = 0
    zero_sk = np.zeros_like(sk)
    x = o.enc([7], base, t, msg, zero_sk, -200.0)[0:1]
    primes = [o.primes[i] for i in base]
    acc = np.zeros_like(x)
    for i, c in enumerate(coeffs):
        term = o.apply_galois(x, base, pow_mod(g, i, m_field)) if i else x.copy()
        po.mul_mont64(term, o.lprime_element_tensor(base, c), primes)
        acc = acc + term
        for j, p in enumerate(primes):
            acc[:, j] %= p
    plain = np.concatenate([acc, np.zeros_like(acc)], axis=0)
    exp = [cmod(v, t) for v in o.decrypt(plain, base, sk, t)]
    assert got == exp


# ---- the dBFV reduction path (src/dbfv.rs:735-1143), pinned by decryption ----

DBFV_CASES = [("field_192", 200, 220, 4, 8), ("field_192", 300, 320, 8, 24), ("field_18", 400, 420, 16, 64),
              ("field_18", 520, 540, 32, 96)]


def _dbfv_setup(po, field, lo, hi, seed):
    o = po.Ring(field, lo, hi, 4)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [seed]
    sk = o.gen_sk(st)
    return o, base, la, st, sk


@pytest.mark.parametrize("field,lo,hi,log2_b,log2_t", DBFV_CASES)
def test_dbfv_enc_dec_and_reduce(po, field, lo, hi, log2_b, log2_t):
    o, base, la, st, sk = _dbfv_setup(po, field, lo, hi, 31)
    t = 1 << log2_t
    rng = np.random.default_rng(log2_t)
    msg = [int(v) for v in rng.integers(0, 1 << min(62, log2_t), size=o.n)]
    if log2_t > 62:
        msg = [(v << (log2_t - 62)) + 12345 for v in msg]
    ct = o.dbfv_enc(st, log2_b, log2_t, base, msg, sk, la)
    assert ct.shape[0] == 2 * ((log2_t - 1) // log2_b + 1)
    assert o.dbfv_decrypt(ct, base, sk, log2_b, log2_t) == [cmod(v, t) for v in msg]
    # reducing again (from period basis) keeps the plaintext
    red = o.dbfv_reduce(log2_b, log2_t, o.crt_to_pb(ct, base), base)
    assert o.dbfv_decrypt(o.pb_to_crt(red, base), base, sk, log2_b, log2_t) == [cmod(v, t) for v in msg]


@pytest.mark.parametrize("field,lo,hi,log2_b,log2_t", DBFV_CASES)
def test_dbfv_hom_mul_decrypts_to_the_product(po, field, lo, hi, log2_b, log2_t):
    o, base, la, st, sk = _dbfv_setup(po, field, lo, hi, 32)
    t = 1 << log2_t
    digits = po.select_digits(len(base), len(base))
    rk = o.gen_rk(st, sk, digits, la)
    a, b = 5 + (1 << (log2_t // 2)), 7 + (1 << (log2_t // 3))
    c1 = o.crt_to_pb(o.dbfv_enc(st, log2_b, log2_t, base, o.encode_scalar(a), sk, la), base)
    c2 = o.crt_to_pb(o.dbfv_enc(st, log2_b, log2_t, base, o.encode_scalar(b), sk, la), base)
    res = o.dbfv_hom_mul(log2_b, log2_t, c1, c2, base, rk, digits)
    dec = o.dbfv_decrypt(res, base, sk, log2_b, log2_t)
    assert o.decode_scalar(t, dec) == cmod(a * b, t)
