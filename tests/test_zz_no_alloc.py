"""hc_bfv_key_switch_noalloc against hc_bfv_key_switch and against the oracle.

The no-allocation key switch serves callers that cannot allocate device memory themselves or
through the library - a host that hands out HBM from its own arena or fixed budget, or a code path
where cudaMalloc / cudaFree are not allowed or would synchronise the device. It keeps its gadget
digits in a static device array shared by all calls, so each test makes two calls in a row on
different ciphertexts: the second must not see anything left over from the first. Results are
compared bit-exactly (the tolerance of every integer test here) with the allocating entry point and
with the oracle's key_switch, and the library's allocation counter and the device pool's high-water
mark must not move across a call. This file is named to run last, so that it also runs after the
rest of the suite has used the device; it creates its own context and ring and passes when run
alone as well.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELD = ("field_36864", 900, 930, 8)


def _digits(r, d):
    per, large, cur, out = r // d, r % d, 0, []
    for i in range(d):
        ln = per + 1 if i < large else per
        out.append((cur, cur + ln))
        cur += ln
    return out


@pytest.fixture(scope="module")
def setup(po):
    import halcuda
    import ringcuda

    be = halcuda.CudaBackend(0)
    ring = ringcuda.RingContext(*FIELD, backend=be)
    oracle = po.Ring(*FIELD)
    yield halcuda, be, ring, oracle
    ring.close()
    be.close()


def _ciphertext_parts(ring, st, base, sk, la, seed):
    g = np.random.default_rng(seed)
    m = [int(v) for v in g.integers(0, 256, size=ring.n)]
    ct = ring.enc(st, base, 256, m, sk, la)
    c0 = ring.allocate(1, len(base))
    c0.copy_from(ct.to_numpy()[0:1])
    c1 = ring.allocate(1, len(base))
    c1.copy_from(ct.to_numpy()[1:2])
    ring.crt_to_pb(c1, base)
    return c0, c1


@pytest.mark.parametrize("ndigits", [4, 1])
def test_noalloc_key_switch_matches_key_switch_and_oracle(setup, ndigits):
    halcuda, be, ring, oracle = setup
    base = ring.initial_base()
    la = ring.log2_alpha_for_sigma(base, 3.2)
    st = [2027 + ndigits]
    sk1, sk2 = ring.gen_sk(st), ring.gen_sk(st)
    digits = _digits(len(base), ndigits)
    ksk = ring.gen_ksk(st, base, sk1, sk2, digits, la)
    ksk_host = ksk.to_numpy().reshape(len(digits), 2, len(base), ring.dl, ring.dk)  # the oracle's key layout
    out = ring.allocate(2, len(base))
    for call, seed in enumerate((1, 2)):
        c0, c1 = _ciphertext_parts(ring, st, base, sk1, la, 10 * ndigits + seed)
        exp = ring.key_switch(c0, c1, base, ksk, digits).to_numpy()
        be.synchronize()
        calls0, used0, _ = halcuda.memory_stats(be, reset_high=True)
        ring.key_switch_noalloc(c0, c1, base, ksk, digits, out)
        be.synchronize()
        calls1, used1, high1 = halcuda.memory_stats(be)
        assert calls1 == calls0, "call %d made %d allocation calls" % (call, calls1 - calls0)
        assert high1 == used0 and used1 == used0, "call %d drew on the device memory pool" % call
        got = out.to_numpy()
        assert (got == exp).all(), "call %d differs from hc_bfv_key_switch" % call
        ref = oracle.key_switch(c0.to_numpy(), c1.to_numpy(), base, ksk_host, digits)
        assert (got == np.asarray(ref).reshape(got.shape)).all(), "call %d differs from the oracle" % call


def test_noalloc_key_switch_rejects_what_it_cannot_do(setup):
    halcuda, be, ring, oracle = setup
    base = ring.initial_base()
    # tables for this digit split were never built: refused, nothing is allocated for them
    c0, c1, out = ring.allocate(1, len(base)), ring.allocate(1, len(base)), ring.allocate(2, len(base))
    keys = ring.allocate(2 * 3, len(base))
    with pytest.raises(halcuda.HalError, match="no tables"):
        ring.key_switch_noalloc(c0, c1, base, keys, _digits(len(base), 3), out)
    # 4 digits x 30 RNS factors x 36864 residues is above the 2^22-word scratch array
    wide = list(range(30))
    c0w, c1w, outw = ring.allocate(1, 30), ring.allocate(1, 30), ring.allocate(2, 30)
    keysw = ring.allocate(8, 30)
    with pytest.raises(halcuda.HalError, match="exceeds the scratch array"):
        ring.key_switch_noalloc(c0w, c1w, wide, keysw, _digits(30, 4), outw)
    # a c0 with fewer RNS rows than the base, or a key tensor of another ring shape: HC_ERR_SHAPE
    keys4 = ring.allocate(2 * 4, len(base))
    short_c0 = ring.allocate(1, len(base) - 1)
    with pytest.raises(halcuda.HalError, match="error 1: key switch c0"):
        ring.key_switch_noalloc(short_c0, c1, base, keys4, _digits(len(base), 4), out)
    bad_keys = be.hal_allocate_i64((8, len(base), ring.dl, ring.dk // 2))
    with pytest.raises(halcuda.HalError, match="error 1: key tensor"):
        ring.key_switch_noalloc(c0, c1, base, bad_keys, _digits(len(base), 4), out)
