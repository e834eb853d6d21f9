"""The reference crate's bfv_hom_mul call sequence issued through the hal::Backend trait entry
points only (trait_ring.py, the path an unchanged crate takes above a hal::cuda backend): its
results are bit-identical to the oracle's hom_mul and to the fused ring-level hc_bfv_hom_mul, at
the benchmarked field_36864 r = 16 parameters, on a key over a longer base than the ciphertext
(the crate restricts the key as a view), and at field_49152 (src/bfv.rs:747-775)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("field,lo,hi,level", [("field_36864", 900, 930, None), ("field_36864", 900, 930, 12),
                                               ("field_49152", 280, 300, None)])
def test_trait_hom_mul_equals_oracle_and_fused(po, be, field, lo, hi, level):
    import ringcuda
    import trait_ring

    o = po.Ring(field, lo, hi, 8)
    R = ringcuda.RingContext(field, lo, hi, 8, backend=be)
    full = o.initial_base()
    base = full if level is None else full[:level]
    la = o.log2_alpha_for_sigma(full, 3.2)
    st = [31]
    sk = o.gen_sk(st)
    digits = po.select_digits(math.ceil(len(full) / 4), len(full))
    rk = o.gen_rk(st, sk, digits, la)
    g = np.random.default_rng(4)
    m1 = [int(v) for v in g.integers(0, 256, size=o.n)]
    la_b = o.log2_alpha_for_sigma(base, 3.2)
    ct1 = o.enc(st, base, 256, m1, sk, la_b)
    ct2 = o.enc(st, base, 256, o.encode_scalar(3), sk, la_b)
    exp = o.hom_mul(256, ct1, ct2, base, rk, digits)
    d1, d2 = R.tensor(ct1), R.tensor(ct2)
    rk_d = R.tensor(rk.reshape((-1,) + rk.shape[2:]))
    bfv = trait_ring.TraitBfv(trait_ring.TraitRing(R))
    l0 = be.launch_count()
    got = bfv.hom_mul(256, d1, d2, base, rk_d, digits).to_numpy()
    assert be.launch_count() - l0 > 40  # the crate's sequence: dozens of trait calls
    assert (got == exp).all()
    fused = R.hom_mul(256, d1, d2, base, rk_d, digits).to_numpy()
    assert (got == fused).all()
    assert o.decrypt(got, base, sk, 256) == [po.cmod(3 * v, 256) for v in m1]
    R.close()
