"""The homomorphic CRT transform step (hom_cyclic_transform_dbfv, src/bootstrap/homcrt.rs:369-429)
and hom_gal with Galois keysets on the GPU, bit-exact against the oracle, with the keys resident
in HBM, streamed from pinned host memory, or split between both."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    "field_18": (("field_18", 300, 320, 4), 932),
    "field_49152": (("field_49152", 200, 230, 2), 20965738),
}


def pow_mod(g, e, m):
    r = 1
    for _ in range(e):
        r = r * g % m
    return r


def bsgs_split(n):
    best = min(range(1, n + 1), key=lambda c: (c + 3 * ((n - 1) // c + 1), c))
    return best, (n - 1) // best + 1


@pytest.fixture(scope="module")
def setups(po, be):
    import ringcuda

    cache = {}

    def get(name):
        if name not in cache:
            (f, lo, hi, tb), g = CASES[name]
            o = po.Ring(f, lo, hi, tb)
            d = ringcuda.RingContext(f, lo, hi, tb, backend=be)
            base = o.initial_base()
            la = o.log2_alpha_for_sigma(base, 3.2)
            st = [77]
            sk = o.gen_sk(st)
            digits = po.select_digits(min(3, len(base)), len(base))
            cache[name] = dict(o=o, d=d, base=base, la=la, st=st, sk=sk, g=g, digits=digits, keys={})
        return cache[name]

    return get


def keys_for(S, gs):
    o = S["o"]
    for gg in gs:
        if gg not in S["keys"]:
            S["keys"][gg] = o.gen_gk(S["st"], S["sk"], gg, S["digits"], S["la"])
    return {gg: S["keys"][gg] for gg in gs}


def make_keyset(S, gks, budget_keys):
    import ringcuda

    d, digits = S["d"], S["digits"]
    o = S["o"]
    key_bytes = 2 * len(digits) * o.initial_len * o.n * 8
    ks = ringcuda.Keyset(d, digits, o.initial_len, budget_keys * key_bytes)
    for gg, k in sorted(gks.items()):
        ks.add(gg, d.tensor(k.reshape((-1,) + k.shape[2:])))
    return ks


def residues(g, shape, primes):
    out = np.empty(shape, dtype=np.int64)
    for j in range(shape[1]):
        p = primes[j]
        out[:, j] = g.integers(-p, p, size=(shape[0],) + tuple(shape[2:]), endpoint=True)
    return out


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("budget", [100, 0, 2])
def test_hom_gal_keyset(setups, name, budget):
    import ringcuda

    S = setups(name)
    o, d, base = S["o"], S["d"], S["base"]
    m = o.info["m"]
    gs = [pow_mod(S["g"], j, m) for j in (1, 2, 3)]
    gks = keys_for(S, gs)
    ks = make_keyset(S, gks, budget)
    rng = np.random.default_rng(3)
    ct = residues(rng, o.shape(2, len(base)), [o.primes[i] for i in base])
    exp = o.hom_gal(ct, base, gs, np.stack([gks[gg] for gg in gs]), S["digits"])
    got = ringcuda.hom_gal_keyset(d, d.tensor(ct), base, gs, ks).to_numpy()
    assert (got == exp.reshape(got.shape)).all()
    st = ks.stats()
    assert st["resident"] + st["streamed"] == 3 and st["resident"] == min(budget, 3)
    assert st["streamed_copies"] == st["streamed"]


@pytest.mark.parametrize("name,length,log2_b,log2_t,dct,budget", [
    ("field_18", 8, 4, 8, 2, 100), ("field_18", 8, 4, 8, 2, 0), ("field_18", 1, 4, 8, 2, 0),
    ("field_18", 3, 3, 9, 1, 1), ("field_49152", 20, 6, 18, 3, 2), ("field_49152", 5, 8, 16, 2, 100),
    # six output digits: the giant-step kernel runs in two launches of up to four digits
    ("field_18", 8, 2, 12, 4, 100), ("field_18", 6, 2, 12, 6, 1),
])
def test_hom_cyclic_transform(setups, name, length, log2_b, log2_t, dct, budget):
    import ringcuda

    S = setups(name)
    o, d, base = S["o"], S["d"], S["base"]
    m = o.info["m"]
    baby, giant = bsgs_split(length)
    gs = sorted(set([pow_mod(S["g"], j, m) for j in range(1, baby)] + ([pow_mod(S["g"], baby, m)] if giant > 1 else [])))
    gks = keys_for(S, gs)
    ks = make_keyset(S, gks, budget)
    rng = np.random.default_rng(length + dct)
    ct = residues(rng, o.shape(2 * dct, len(base)), [o.primes[i] for i in base])
    t = 1 << log2_t
    coeffs = [[int(v) for v in rng.integers(-t, t, size=o.dl)] for _ in range(length)]
    exp = o.dbfv_hom_cyclic_transform(log2_b, log2_t, S["g"], coeffs, ct, base, gks, S["digits"])
    got = ringcuda.dbfv_hom_cyclic_transform(d, log2_b, log2_t, S["g"], coeffs, d.tensor(ct), base, ks).to_numpy()
    assert got.shape == exp.shape
    assert (got == exp).all()


@pytest.mark.parametrize("budget", [100, 1])
def test_hom_cyclic_transform_back_to_back(setups, be, budget):
    """Several transforms issued back to back with different coefficients and no synchronisation
    between them: each call's coefficient digits travel through the ring's pinned staging buffer
    without blocking the host, so a later call must not overwrite an upload still in flight; every
    result equals the oracle's."""
    import ringcuda

    S = setups("field_49152")
    o, d, base = S["o"], S["d"], S["base"]
    m = o.info["m"]
    length, log2_b, log2_t, dct = 12, 6, 18, 3
    baby, giant = bsgs_split(length)
    gs = sorted(set([pow_mod(S["g"], j, m) for j in range(1, baby)] + [pow_mod(S["g"], baby, m)]))
    gks = keys_for(S, gs)
    ks = make_keyset(S, gks, budget)
    rng = np.random.default_rng(91)
    ct = residues(rng, o.shape(2 * dct, len(base)), [o.primes[i] for i in base])
    dct_t = d.tensor(ct)
    t = 1 << log2_t
    sets = [[[int(v) for v in rng.integers(-t, t, size=o.dl)] for _ in range(length)] for _ in range(4)]
    outs = [ringcuda.dbfv_hom_cyclic_transform(d, log2_b, log2_t, S["g"], c, dct_t, base, ks) for c in sets]
    be.synchronize()
    for c, got in zip(sets, outs):
        exp = o.dbfv_hom_cyclic_transform(log2_b, log2_t, S["g"], c, ct, base, gks, S["digits"])
        assert (got.to_numpy() == exp).all()
