"""Bit-exact parity of the fused GPU ring and BFV operations against the oracle's restatement of
the reference's ring.rs / bfv.rs over hal::cpu, plus decryption of the results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RING_CASES = {
    "field_18": ("field_18", 300, 320, 4),
    "field_192": ("field_192", 100, 120, 8),
    "field_36864": ("field_36864", 900, 930, 8),
    "field_49152": ("field_49152", 1280, 1310, 2),
}


@pytest.fixture(scope="module")
def rings(po, be):
    import ringcuda

    cache = {}

    def get(name):
        if name not in cache:
            f, lo, hi, tb = RING_CASES[name]
            cache[name] = (po.Ring(f, lo, hi, tb), ringcuda.RingContext(f, lo, hi, tb, backend=be))
        return cache[name]

    return get


def residues(g, shape, primes, bound=1):
    out = np.empty(shape, dtype=np.int64)
    for j in range(shape[1]):
        p = primes[j]
        out[:, j] = g.integers(-bound * p, bound * p, size=(shape[0],) + tuple(shape[2:]), endpoint=True)
    return out


@pytest.mark.parametrize("name", list(RING_CASES))
def test_primes_and_crt_kernels(rings, name):
    o, d = rings(name)
    assert d.primes == o.primes and d.initial_len == o.initial_len
    assert d.extension_base(d.initial_base()) == o.extension_base(o.initial_base())
    for idx in sorted({0, len(o.primes) // 2, len(o.primes) - 1}):
        for a, b in zip(o.kernels(idx), d.crt_kernels(idx)):
            assert (a == b).all()


@pytest.mark.parametrize("name", list(RING_CASES))
def test_transforms(rings, name):
    o, d = rings(name)
    g = np.random.default_rng(11)
    base = o.initial_base()
    count = 2 if name in ("field_36864", "field_49152") else 3
    x = residues(g, o.shape(count, len(base)), [o.primes[i] for i in base], bound=2)
    t = d.tensor(x)
    d.pb_to_crt(t, base)
    exp = o.pb_to_crt(x, base)
    assert (t.to_numpy() == exp).all()
    d.crt_to_pb(t, base)
    assert (t.to_numpy() == o.crt_to_pb(exp, base)).all()


def test_bconv_known_answer_primes(po, be):
    import ringcuda

    from test_oracle_ring_bfv import BCONV_PRIMES, trunc_mod

    rf = BCONV_PRIMES
    o = po.Ring("field_2", raw_primes=rf)
    d = ringcuda.RingContext("field_2", raw_primes=rf, backend=be)
    d2 = [1 << 64, 3 << 100, -7 << 100, 9 << 120, -1 << 120, 5 << 120, 0, 7 << 120]
    src = np.zeros((2, 7, 8, 1), dtype=np.int64)
    for i in range(7):
        for j in range(8):
            src[0, i, j, 0] = po.montgomery_repr(j, rf[i])
            src[1, i, j, 0] = po.montgomery_repr(trunc_mod(d2[j], rf[i]), rf[i])
    exp = o.bconv(src, list(range(7)), list(range(7, 13)))
    out = be.hal_allocate_i64((2, 6, 8, 1))
    s = be.tensor(src)
    d.bconv(out, list(range(7, 13)), s, list(range(7)))
    assert (out.to_numpy() == exp).all()
    assert (s.to_numpy() == src).all()  # the source is not destroyed
    g = np.random.default_rng(3)
    x = residues(g, (1, 7, 16, 1), rf[:7])
    digits = [(0, 3), (3, 5), (5, 7)]
    got = be.hal_allocate_i64((3, 7, 16, 1))
    d.bconv_gadget(got, be.tensor(x), list(range(7)), digits)
    assert (got.to_numpy() == o.bconv_gadget(x, list(range(7)), digits)).all()


@pytest.mark.parametrize("name", ["field_36864", "field_49152", "field_192"])
def test_bconv_full_size(rings, name):
    o, d = rings(name)
    g = np.random.default_rng(12)
    base = o.initial_base()
    ext = o.extension_base(base)
    x = residues(g, o.shape(3, len(base)), [o.primes[i] for i in base], bound=1)
    out = d.allocate(3, len(ext))
    d.bconv(out, ext, d.tensor(x), base)
    assert (out.to_numpy() == o.bconv(x, base, ext)).all()
    y = residues(g, o.shape(2, len(ext)), [o.primes[i] for i in ext], bound=1)
    out2 = d.allocate(2, len(base))
    d.bconv(out2, base, d.tensor(y), ext)
    assert (out2.to_numpy() == o.bconv(y, ext, base)).all()
    for nd in sorted({1, min(3, len(base)), len(base)}):
        digits = [tuple(v) for v in __import__("ringcuda").select_digits(nd, len(base))]
        z = residues(g, o.shape(1, len(base)), [o.primes[i] for i in base])
        got = d.allocate(nd, len(base))
        d.bconv_gadget(got, d.tensor(z), base, digits)
        assert (got.to_numpy() == o.bconv_gadget(z, base, digits)).all(), nd


@pytest.mark.parametrize("name", ["field_18", "field_36864", "field_49152"])
def test_apply_galois(rings, name):
    o, d = rings(name)
    g = np.random.default_rng(13)
    base = o.initial_base()[:3]
    x = residues(g, o.shape(2, len(base)), [o.primes[i] for i in base])
    m = o.info["m"]
    gens = list(o.info["gens"]) + [g_ * h % m for g_, h in zip(o.info["gens"], o.info["gens"][1:])]
    for gg in gens:
        out = d.allocate(2, len(base))
        d.apply_galois(out, d.tensor(x), base, gg)
        assert (out.to_numpy() == o.apply_galois(x, base, gg)).all(), gg


def _keys_np(o, keys):
    return keys.reshape((-1, 2) + keys.shape[1:]) if keys.ndim == 4 else keys


@pytest.mark.parametrize("name", ["field_192", "field_18"])
def test_keygen_and_encryption_match(rings, name):
    o, d = rings(name)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    assert d.log2_alpha_for_sigma(base, 3.2) == la
    so, sd = [77], [77]
    sk_o, sk_d = o.gen_sk(so), d.gen_sk(sd)
    assert so == sd and (sk_d.to_numpy() == sk_o).all()
    m = [(i % 255) - 127 for i in range(o.n)]
    ct_o = o.enc(so, base, 256, m, sk_o, la)
    ct_d = d.enc(sd, base, 256, m, sk_d, la)
    assert so == sd and (ct_d.to_numpy() == ct_o).all()
    digits = po_digits(len(base), len(base))
    rk_o = o.gen_rk(so, sk_o, digits, la)
    rk_d = d.gen_rk(sd, sk_d, digits, la)
    assert (rk_d.to_numpy().reshape(rk_o.shape) == rk_o).all()
    g = o.info["gens"][-1]
    gk_o = o.gen_gk(so, sk_o, g, digits, la)
    gk_d = d.gen_gk(sd, sk_d, g, digits, la)
    assert (gk_d.to_numpy().reshape(gk_o.shape) == gk_o).all()
    noisy = d.noisy_plaintext(ct_d, base, sk_d).to_numpy()
    assert (noisy == o.noisy_plaintext(ct_o, base, sk_o)).all()
    assert o.decode_scaled(noisy, base, 256) == m


def po_digits(nd, r):
    import ringcuda

    return [tuple(x) for x in ringcuda.select_digits(nd, r)]


def test_key_switch_lift_rescale_modswitch(rings):
    o, d = rings("field_18")
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [5]
    sk1 = o.gen_sk(st)
    sk2 = o.gen_sk(st)
    m = [(i % 15) - 7 for i in range(o.n)]
    ct = o.enc(st, base, 16, m, sk1, la)
    digits = po_digits(len(base), len(base))
    ksk = o.gen_ksk(st, base, sk1, sk2, digits, la)
    c1 = o.crt_to_pb(ct[1:2], base)
    exp = o.key_switch(ct[0:1], c1, base, ksk, digits)
    got = d.key_switch(d.tensor(ct[0:1]), d.tensor(c1), base, d.tensor(ksk.reshape((-1,) + ksk.shape[2:])), digits)
    assert (got.to_numpy() == exp).all()
    assert o.decrypt(exp, base, sk2, 16) == m
    ct_pb = o.crt_to_pb(ct, base)
    for crt in (None, ct):
        exp_l = o.lift_to_extended(ct_pb, base, crt)
        got_l = d.lift_to_extended(d.tensor(ct_pb), base, d.tensor(crt) if crt is not None else None)
        assert (got_l.to_numpy() == exp_l).all()
    lifted = base + o.extension_base(base)
    g = np.random.default_rng(14)
    x = residues(g, o.shape(3, len(lifted)), [o.primes[i] for i in lifted])
    exp_r = o.rescale_to_base(x, lifted, len(base), 16)
    got_r = d.rescale_to_base(d.tensor(x), lifted, len(base), 16)
    assert (got_r.to_numpy() == exp_r).all()
    for new_len in (1, len(base) - 2, len(base)):
        exp_m = o.mod_switch_down(ct_pb, base, new_len)
        got_m = d.mod_switch_down(d.tensor(ct_pb), base, new_len)
        assert (got_m.to_numpy() == exp_m).all(), new_len


HOM_MUL_CASES = [("field_192", 100, 120, 8, 256, 1.0), ("field_18", 300, 320, 16, 1 << 16, 1.0),
                 ("field_192", 200, 220, 64, 1 << 64, 0.5), ("field_36864", 900, 930, 8, 256, 0.25),
                 ("field_49152", 600, 630, 2, 4, 0.5)]


@pytest.mark.parametrize("case", HOM_MUL_CASES, ids=lambda c: "%s-t%d" % (c[0], c[4].bit_length() - 1))
def test_hom_mul(po, be, case):
    import ringcuda

    field, lo, hi, tb, t, dfrac = case
    o = po.Ring(field, lo, hi, tb)
    d = ringcuda.RingContext(field, lo, hi, tb, backend=be)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [31]
    sk = o.gen_sk(st)
    digits = po_digits(max(1, int(np.ceil(len(base) * dfrac))), len(base))
    rk = o.gen_rk(st, sk, digits, la)
    a, b = (3 << 20, 5 << 19) if t > (1 << 32) else (5, 7)
    ct1 = o.enc(st, base, t, o.encode_scalar(a), sk, la)
    ct2 = o.enc(st, base, t, o.encode_scalar(b), sk, la)
    rk_d = d.tensor(rk.reshape((-1,) + rk.shape[2:]))
    for period in (False, True):
        exp = o.hom_mul(t, ct1, ct2, base, rk, digits, period_output=period)
        got = d.hom_mul(t, d.tensor(ct1), d.tensor(ct2), base, rk_d, digits, period_output=period).to_numpy()
        assert (got == exp).all(), period
        if not period:
            assert o.decode_scalar(t, o.decrypt(got, base, sk, t)) == po.cmod(a * b, t)


@pytest.mark.parametrize("name", ["field_18", "field_36864"])
def test_hom_gal(rings, name, po):
    o, d = rings(name)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [6]
    sk = o.gen_sk(st)
    # one prime per digit where the base is small (src/bfv.rs:1130), four per digit at full size
    digits = po_digits(len(base) if len(base) < 8 else len(base) // 4, len(base))
    gens = list(o.info["gens"])[:3]
    gks = np.stack([o.gen_gk(st, sk, g, digits, la) for g in gens])
    ptxt = [int(i % 3 == 0) for i in range(o.n)]
    ct = o.enc(st, base, 16, ptxt, sk, la)
    exp = o.hom_gal(ct, base, gens, gks, digits)
    got = d.hom_gal(d.tensor(ct), base, gens, d.tensor(gks.reshape((-1,) + gks.shape[3:])), digits).to_numpy()
    assert (got.reshape(exp.shape) == exp).all()
    for gi, g in enumerate(gens):
        dec = o.decrypt(got.reshape(exp.shape)[gi], base, sk, 16)
        # decrypting the rotated ciphertext gives the plaintext permuted by g (src/ring.rs:1183-1222)
        perm = o.apply_galois(np.arange(o.n, dtype=np.int64).reshape(1, 1, o.dl, o.dk), [0], g).reshape(-1)
        assert dec == [ptxt[int(perm[i])] for i in range(o.n)]


@pytest.mark.parametrize("name", ["field_18", "field_36864"])
def test_hom_gal_batch_matches_oracle(rings, name, po):
    """B ciphertexts under one automorphism in one call: each equals the oracle's hom_gal."""
    o, d = rings(name)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [8]
    sk = o.gen_sk(st)
    digits = po_digits(len(base) if len(base) < 8 else len(base) // 4, len(base))
    g = list(o.info["gens"])[0]
    gk = o.gen_gk(st, sk, g, digits, la)
    B = 3
    cts = [o.enc(st, base, 16, [(i * (b + 2)) % 16 for i in range(o.n)], sk, la) for b in range(B)]
    got = d.hom_gal_batch(d.tensor(np.concatenate(cts)), base, g, d.tensor(gk.reshape((-1,) + gk.shape[2:])),
                          digits).to_numpy()
    for b in range(B):
        exp = o.hom_gal(cts[b], base, [g], gk[None], digits)[0]
        assert (got[2 * b:2 * b + 2] == exp).all(), b


def test_hom_mul_batched_matches_single(po, be):
    """B ciphertext pairs stacked along dimension 0 in one call give the per-pair results."""
    import ringcuda

    o = po.Ring("field_192", 100, 120, 8)
    d = ringcuda.RingContext("field_192", 100, 120, 8, backend=be)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [17]
    sk = o.gen_sk(st)
    digits = po_digits(len(base), len(base))
    rk = d.tensor(o.gen_rk(st, sk, digits, la).reshape((-1,) + (len(base), o.dl, o.dk)))
    B = 3
    c1 = np.concatenate([o.enc(st, base, 256, [(i * (b + 1)) % 256 for i in range(o.n)], sk, la) for b in range(B)])
    c2 = np.concatenate([o.enc(st, base, 256, [(i + b) % 256 for i in range(o.n)], sk, la) for b in range(B)])
    for period in (False, True):
        got = d.hom_mul(256, d.tensor(c1), d.tensor(c2), base, rk, digits, period_output=period).to_numpy()
        for b in range(B):
            one = d.hom_mul(256, d.tensor(c1[2 * b:2 * b + 2]), d.tensor(c2[2 * b:2 * b + 2]), base, rk, digits,
                            period_output=period).to_numpy()
            assert (got[2 * b:2 * b + 2] == one).all(), (b, period)


def test_hom_mul_batched_full_size_matches_oracle(po, be):
    """Two field_36864 r = 16 ciphertext pairs in one call (the batched form of the benchmark,
    with its parallel branches) equal the oracle's per-pair hom_mul."""
    import ringcuda

    o = po.Ring("field_36864", 900, 930, 8)
    d = ringcuda.RingContext("field_36864", 900, 930, 8, backend=be)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [19]
    sk = o.gen_sk(st)
    digits = po_digits(4, len(base))
    rk = o.gen_rk(st, sk, digits, la)
    rk_d = d.tensor(rk.reshape((-1,) + rk.shape[2:]))
    B = 2
    c1 = [o.enc(st, base, 256, [(i * (b + 3)) % 256 for i in range(o.n)], sk, la) for b in range(B)]
    c2 = [o.enc(st, base, 256, [(5 * i + b) % 256 for i in range(o.n)], sk, la) for b in range(B)]
    got = d.hom_mul(256, d.tensor(np.concatenate(c1)), d.tensor(np.concatenate(c2)), base, rk_d, digits).to_numpy()
    for b in range(B):
        exp = o.hom_mul(256, c1[b], c2[b], base, rk, digits)
        assert (got[2 * b:2 * b + 2] == exp).all(), b


def word_offset(be, arr):
    """`arr` in a view whose rows start one word into a wider buffer: 8-byte aligned only, with an
    odd dimension-2 stride, so no 16-byte access fits it."""
    n0, n1, n2, n3 = arr.shape
    buf = be.hal_allocate_i64((n0, n1, n2, n3 + 1))
    return buf.slice(None, None, None, (1, n3 + 1)).copy_from(arr)


@pytest.mark.parametrize("name", ["field_18", "field_36864"])
def test_unaligned_views_match_oracle(rings, name, po, be):
    """Operands and keys in views that admit no 16-byte access (the one-position forms of the key
    switch and the tensor product) give the oracle's hom_mul, key switch and hom_gal."""
    o, d = rings(name)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [29]
    sk, sk2 = o.gen_sk(st), o.gen_sk(st)
    digits = po_digits(len(base) if len(base) < 8 else len(base) // 4, len(base))
    ct1 = o.enc(st, base, 16, [i % 16 for i in range(o.n)], sk, la)
    ct2 = o.enc(st, base, 16, [(3 * i + 1) % 16 for i in range(o.n)], sk, la)
    rk = o.gen_rk(st, sk, digits, la)
    exp = o.hom_mul(16, ct1, ct2, base, rk, digits)
    got = d.hom_mul(16, word_offset(be, ct1), word_offset(be, ct2), base,
                    word_offset(be, rk.reshape((-1,) + rk.shape[2:])), digits).to_numpy()
    assert (got == exp).all()
    ksk = o.gen_ksk(st, base, sk, sk2, digits, la)
    c1 = o.crt_to_pb(ct1[1:2], base)
    exp_k = o.key_switch(ct1[0:1], c1, base, ksk, digits)
    got_k = d.key_switch(d.tensor(ct1[0:1]), d.tensor(c1), base, word_offset(be, ksk.reshape((-1,) + ksk.shape[2:])),
                         digits).to_numpy()
    assert (got_k == exp_k).all()
    g = list(o.info["gens"])[0]
    gk = o.gen_gk(st, sk, g, digits, la)
    exp_g = o.hom_gal(ct2, base, [g], gk[None], digits)[0]
    got_g = d.hom_gal_batch(d.tensor(ct2), base, g, word_offset(be, gk.reshape((-1,) + gk.shape[2:])),
                            digits).to_numpy()
    assert (got_g == exp_g).all()


def test_graph_replay_matches(po, be):
    """A captured hom_mul replayed from a CUDA graph reproduces the direct result."""
    import halcuda
    import ringcuda

    d = ringcuda.RingContext("field_192", 100, 120, 8, backend=be)
    o = po.Ring("field_192", 100, 120, 8)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [23]
    sk = o.gen_sk(st)
    digits = po_digits(len(base), len(base))
    rk = d.tensor(o.gen_rk(st, sk, digits, la).reshape((-1,) + (len(base), o.dl, o.dk)))
    c1 = d.tensor(o.enc(st, base, 256, [5] * o.n, sk, la))
    c2 = d.tensor(o.enc(st, base, 256, [7] * o.n, sk, la))
    out = d.allocate(2, len(base))
    d.hom_mul(256, c1, c2, base, rk, digits, out=out)
    direct = out.to_numpy()
    be.hal_assign(out, d.allocate(2, len(base)))
    g = halcuda.Graph(be, lambda: d.hom_mul(256, c1, c2, base, rk, digits, out=out))
    g.launch()
    g.launch()
    assert (out.to_numpy() == direct).all()
