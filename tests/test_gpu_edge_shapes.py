"""Edge shapes through the ring layer and the batched transforms: elements counts of zero (a
no-op, no launch, the reference's loops over an empty batch), a batch whose items include an
empty one, and the largest RNS length of the large fields' initial bases in one call, each
bit-exact against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RINGS = {
    "field_36864": ("field_36864", 900, 930, 8),
    "field_49152": ("field_49152", 1280, 1310, 2),
}


@pytest.fixture(scope="module")
def rings(po, be):
    import ringcuda

    cache = {}

    def get(name):
        if name not in cache:
            f, lo, hi, tb = RINGS[name]
            cache[name] = (po.Ring(f, lo, hi, tb), ringcuda.RingContext(f, lo, hi, tb, backend=be))
        return cache[name]

    yield get
    for _, d in cache.values():
        d.close()


def residues(g, shape, primes, bound=1):
    out = np.empty(shape, dtype=np.int64)
    for j in range(shape[1]):
        p = primes[j]
        out[:, j] = g.integers(-bound * p, bound * p, size=(shape[0],) + tuple(shape[2:]), endpoint=True)
    return out


@pytest.mark.parametrize("name", list(RINGS))
def test_transform_of_zero_elements_is_a_no_op(be, rings, name):
    o, d = rings(name)
    base = [0, 1, 2]
    one = d.allocate(1, len(base))
    d.pb_to_crt(one, base)  # builds the base's tables (their construction launches kernels)
    be.synchronize()
    x = d.allocate(0, len(base))
    l0 = be.launch_count()
    d.pb_to_crt(x, base)
    d.crt_to_pb(x, base)
    be.synchronize()
    assert be.launch_count() == l0
    assert tuple(x.shape) == (0, 3, o.shape(1, 1)[2], o.shape(1, 1)[3])


def test_batch_with_an_empty_item(po, be, rings):
    import ringcuda

    g = np.random.default_rng(41)
    items, checks = [], []
    for name, count, base in (("field_36864", 0, [0, 1]), ("field_49152", 2, [0, 1, 2]), ("field_36864", 1, [2])):
        o, d = rings(name)
        primes = [o.primes[i] for i in base]
        x = residues(g, o.shape(count, len(base)), primes, 2)
        op = residues(g, o.shape(max(count, 1), len(base)), primes, 1)
        dx = d.tensor(x)
        items.append((d, dx, d.tensor(op), base))
        if count:
            y = o.pb_to_crt(x, base)
            y = np.ascontiguousarray(y).copy()
            po.mul_mont64(y, np.ascontiguousarray(op), primes)
            checks.append((dx, o.crt_to_pb(y, base)))
    batch = ringcuda.CrtBatch(items, ringcuda.CRT_FORWARD | ringcuda.CRT_MUL | ringcuda.CRT_INVERSE)
    assert batch.num_slabs == 2 * 3 + 1
    batch.run()
    for dx, exp in checks:
        assert (dx.to_numpy() == exp).all()
    batch.close()


@pytest.mark.parametrize("name", list(RINGS))
def test_transform_over_the_whole_initial_base(po, rings, name):
    """One call over every factor of the initial base (34 for field_36864 at 900-930 bits, 48 for
    field_49152 at 1280-1310), both directions."""
    o, d = rings(name)
    base = list(range(len(o.initial_base())))
    primes = [o.primes[i] for i in base]
    g = np.random.default_rng(43)
    x = residues(g, o.shape(1, len(base)), primes, 2)
    exp = o.pb_to_crt(x, base)
    dx = d.tensor(x)
    d.pb_to_crt(dx, base)
    got = dx.to_numpy()
    assert (got == exp).all()
    back = o.crt_to_pb(exp, base)
    d.crt_to_pb(dx, base)
    assert (dx.to_numpy() == back).all()
