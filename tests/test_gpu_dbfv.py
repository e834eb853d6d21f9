"""The dBFV reduction path (split_overflow / dbfv_reduce / dbfv_enc / dbfv_hom_mul,
src/dbfv.rs:661-1143) on the GPU, bit-exact against the oracle, plus decryption of the product."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [("field_192", 200, 220, 4, 8), ("field_18", 400, 420, 16, 64), ("field_18", 520, 540, 32, 96),
         ("field_36864", 600, 630, 8, 24)]


@pytest.fixture(scope="module")
def rings(po, be):
    import ringcuda

    cache = {}

    def get(f, lo, hi):
        if (f, lo, hi) not in cache:
            cache[(f, lo, hi)] = (po.Ring(f, lo, hi, 4), ringcuda.RingContext(f, lo, hi, 4, backend=be))
        return cache[(f, lo, hi)]

    return get


@pytest.mark.parametrize("field,lo,hi,log2_b,log2_t", CASES)
def test_dbfv_enc_reduce_mul_match_oracle(po, rings, field, lo, hi, log2_b, log2_t):
    import ringcuda

    o, d = rings(field, lo, hi)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    t = 1 << log2_t
    st_o, st_d = [77], [77]
    sk = o.gen_sk(st_o)
    dsk = d.gen_sk(st_d)
    assert (dsk.to_numpy() == sk).all()
    a, b = 3 + (1 << (log2_t // 2)), 11 + (1 << (log2_t // 3))
    enc_o = [o.dbfv_enc(st_o, log2_b, log2_t, base, o.encode_scalar(v), sk, la) for v in (a, b)]
    enc_d = [ringcuda.dbfv_enc(d, st_d, log2_b, log2_t, base, o.encode_scalar(v), dsk, la) for v in (a, b)]
    for x, y in zip(enc_o, enc_d):
        assert (y.to_numpy() == x).all()
    pb = [o.crt_to_pb(x, base) for x in enc_o]
    # reduction of an unreduced sum (bound 2)
    s = pb[0] + pb[1]
    exp = o.dbfv_reduce(log2_b, log2_t, s, base, bound=2)
    got = ringcuda.dbfv_reduce(d, log2_b, log2_t, d.tensor(s), base, bound=2).to_numpy()
    assert (got == exp).all()
    digits = po.select_digits(min(3, len(base)), len(base))
    rk = o.gen_rk(st_o, sk, digits, la)
    for period in (False, True):
        exp = o.dbfv_hom_mul(log2_b, log2_t, pb[0], pb[1], base, rk, digits, period_output=period)
        got = ringcuda.dbfv_hom_mul(d, log2_b, log2_t, d.tensor(pb[0]), d.tensor(pb[1]), base,
                                    d.tensor(rk.reshape((-1,) + rk.shape[2:])), digits, period_output=period).to_numpy()
        assert got.shape == exp.shape and (got == exp).all(), period
    dec = o.dbfv_decrypt(got_crt(o, got, base, True), base, sk, log2_b, log2_t)
    assert o.decode_scalar(t, dec) == po.cmod(a * b, t)


def got_crt(o, x, base, period):
    return o.pb_to_crt(x, base) if period else x
