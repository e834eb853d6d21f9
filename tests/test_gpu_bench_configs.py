"""Bit-exact parity at the sizes the benchmark runs, against the oracle:

* batched CRT transforms (configuration 3): both large fields and every RNS length 4..24, three
  elements each (126 elements, 1764 (element, factor) slabs in one persistent launch), forward
  transform, Montgomery product with a per-element operand, inverse transform, autotuned and
  replayed from a CUDA graph; every element is compared (src/ring.rs:1118-1161);
* the homomorphic CRT step (configuration 4) exactly as benched: field_49152, r = 23, t = 2^24 in
  three digits of 2^8, the order-64 generator (13 baby x 5 giant steps), 13 Galois keys of six
  gadget digits, an HBM budget of 8 keys with the other 5 streamed (src/bootstrap/homcrt.rs:365-429);
* BFV ciphertext multiplication at field_36864 with r = 12 and r = 20 initial factors, t = 256,
  ceil(r / 4) gadget digits, with decryption (src/bfv.rs:747-775).

The oracle runs single-threaded; these cases take tens of seconds of CPU each.
"""
import math

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

CRT_FIELDS = (("field_36864", 900, 930, 8), ("field_49152", 1280, 1310, 2))


def test_crt_batch_every_rns_length(po, be):
    import halcuda
    import ringcuda

    g = np.random.default_rng(2026)
    items, checks = [], []
    for f, lo, hi, tb in CRT_FIELDS:
        o = po.Ring(f, lo, hi, tb)
        d = ringcuda.RingContext(f, lo, hi, tb, backend=be)
        assert d.primes == o.primes
        for r in range(4, 25):
            base = list(range(r))
            # residues uniform in [-2^56, 2^56) as the benchmark draws them (input bound 2)
            x = g.integers(-(1 << 56), 1 << 56, size=o.shape(3, r), dtype=np.int64)
            op = g.integers(-(1 << 56), 1 << 56, size=o.shape(3, r), dtype=np.int64)
            dx, dop = d.tensor(x), d.tensor(op)
            items.append((d, dx, dop, base))
            y = o.pb_to_crt(x, base)
            y = np.ascontiguousarray(y).copy()
            po.mul_mont64(y, np.ascontiguousarray(op), [o.primes[i] for i in base])
            checks.append((dx, o.crt_to_pb(y, base), f, r))
    batch = ringcuda.CrtBatch(items, ringcuda.CRT_FORWARD | ringcuda.CRT_MUL | ringcuda.CRT_INVERSE, backend=be)
    assert batch.num_slabs == 3 * 2 * sum(range(4, 25))
    batch.tune(reps=1)  # on scratch copies: the inputs are untouched
    graph = halcuda.Graph(be, batch.run)
    graph.launch()
    be.synchronize()
    bad = [(f, r) for dx, exp, f, r in checks if not (dx.to_numpy() == exp).all()]
    assert not bad, bad


def _bsgs(length):
    baby = min(range(1, length + 1), key=lambda c: (c + 3 * ((length - 1) // c + 1), c))
    return baby, (length - 1) // baby + 1


def test_homcrt_benched_configuration(po, be):
    import ringcuda

    o = po.Ring("field_49152", 1280, 1310, 2)
    d = ringcuda.RingContext("field_49152", 1280, 1310, 2, backend=be)
    base = o.initial_base()
    r = len(base)
    assert r == 23
    log2_b, log2_t, gen, length = 8, 24, 20965738, 64
    digits = po.select_digits(math.ceil(r / 4), r)
    assert len(digits) == 6
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [99]
    sk = o.gen_sk(st)
    m = o.info["m"]
    baby, giant = _bsgs(length)
    assert (baby, giant) == (13, 5)
    gs = sorted(set([pow(gen, j, m) for j in range(1, baby)] + [pow(gen, baby, m)]))
    keys = {gg: o.gen_gk(st, sk, gg, digits, la) for gg in gs}
    t = 1 << log2_t
    rng = np.random.default_rng(5)
    ct = np.zeros(o.shape(6, r), dtype=np.int64)
    ct[0:2] = o.enc(st, base, t, [int(v) for v in rng.integers(0, t, size=o.n)], sk, la)
    for dd in (1, 2):
        ct[2 * dd:2 * dd + 2] = o.enc(st, base, t, [0] * o.n, sk, la)
    coeffs = [[int(v) for v in rng.integers(-t // 2, t // 2, size=o.dl)] for _ in range(length)]
    exp = o.dbfv_hom_cyclic_transform(log2_b, log2_t, gen, coeffs, ct, base, keys, digits)
    key_bytes = 2 * len(digits) * r * o.n * 8
    ks = ringcuda.Keyset(d, digits, r, 8 * key_bytes)
    for gg in gs:
        ks.add(gg, d.tensor(keys[gg].reshape((-1,) + keys[gg].shape[2:])))
    dct = d.tensor(ct)
    for rep in range(2):  # the second run streams the over-budget keys again into reused slots
        got = ringcuda.dbfv_hom_cyclic_transform(d, log2_b, log2_t, gen, coeffs, dct, base, ks).to_numpy()
        assert got.shape == exp.shape
        assert (got == exp).all(), "run %d" % rep
    s = ks.stats()
    assert s["resident"] == 8 and s["streamed"] == 5 and s["streamed_copies"] > 0
    ks.close()


@pytest.mark.parametrize("lo,hi,r", [(660, 690, 12), (1120, 1150, 20)])
def test_hom_mul_config2_rns_lengths(po, be, lo, hi, r):
    import ringcuda

    o = po.Ring("field_36864", lo, hi, 8)
    d = ringcuda.RingContext("field_36864", lo, hi, 8, backend=be)
    base = o.initial_base()
    assert len(base) == r
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [r]
    sk = o.gen_sk(st)
    digits = po.select_digits(math.ceil(r / 4), r)
    rk = o.gen_rk(st, sk, digits, la)
    t = 256
    rng = np.random.default_rng(r)
    m1 = [int(v) for v in rng.integers(0, 3, size=o.n)]
    ct1 = o.enc(st, base, t, m1, sk, la)
    ct2 = o.enc(st, base, t, o.encode_scalar(7), sk, la)
    exp = o.hom_mul(t, ct1, ct2, base, rk, digits)
    rk_d = d.tensor(rk.reshape((-1,) + rk.shape[2:]))
    got = d.hom_mul(t, d.tensor(ct1), d.tensor(ct2), base, rk_d, digits).to_numpy()
    assert (got == exp).all()
    assert o.decrypt(got, base, sk, t) == [po.cmod(7 * v, t) for v in m1]


def test_uniform_ternary_secret_key(po, be):
    """The benchmark's secret key (hc_bfv_gen_sk_uniform_ternary, no reference counterpart):
    coefficient j is (splitmix64 draw j mod 3) - 1, returned in CRT basis over the initial base; a
    field_36864 r = 16 ct-mult of encryptions under it equals the oracle's and decrypts to the
    product."""
    import ringcuda

    R = ringcuda.RingContext("field_36864", 120, 140, 8, backend=be)
    o = po.Ring("field_36864", 120, 140, 8)
    base = R.initial_base()
    st, st2 = [77], [77]
    sk = R.gen_sk_uniform_ternary(st)
    exp = [po.splitmix64(st2) % 3 - 1 for _ in range(R.n)]
    assert st[0] == st2[0]
    pb = R.allocate(1, len(base))
    be.hal_assign(pb, sk)
    R.crt_to_pb(pb, base)
    lifts, _ = o.element_lifts(pb.to_numpy(), base)
    assert lifts == exp
    assert all(abs(exp.count(v) - R.n / 3) < 0.02 * R.n for v in (-1, 0, 1))
    R.close()

    R = ringcuda.RingContext("field_36864", 900, 930, 8, backend=be)
    o = po.Ring("field_36864", 900, 930, 8)
    base = R.initial_base()
    st = [2026]
    sk = R.gen_sk_uniform_ternary(st)
    digits = po.select_digits(math.ceil(len(base) / 4), len(base))
    la = R.log2_alpha_for_sigma(base, 3.2)
    rk = R.gen_rk(st, sk, digits, la)
    g = np.random.default_rng(12)
    m1 = [int(v) for v in g.integers(0, 256, size=R.n)]
    ct1, ct2 = R.enc(st, base, 256, m1, sk, la), R.enc(st, base, 256, o.encode_scalar(5), sk, la)
    got = R.hom_mul(256, ct1, ct2, base, rk, digits).to_numpy()
    rk_o = rk.to_numpy().reshape(len(digits), 2, len(base), R.dl, R.dk)
    assert (got == o.hom_mul(256, ct1.to_numpy(), ct2.to_numpy(), base, rk_o, digits)).all()
    assert o.decrypt(got, base, sk.to_numpy(), 256) == [po.cmod(5 * v, 256) for v in m1]
    R.close()
