"""Batched CRT transforms (one persistent launch over elements of several fields and RNS lengths)
against the oracle's pb_to_crt / mul_mont64 / crt_to_pb, element by element, bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RINGS = {
    "field_36864": ("field_36864", 900, 930, 8),
    "field_49152": ("field_49152", 1280, 1310, 2),
    "field_18": ("field_18", 300, 320, 4),
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

    return get


def residues(g, shape, primes, bound):
    out = np.empty(shape, dtype=np.int64)
    for j in range(shape[1]):
        p = primes[j]
        out[:, j] = g.integers(-bound * p, bound * p, size=(shape[0],) + tuple(shape[2:]), endpoint=True)
    return out


def expected(po, o, x, op, base, ops):
    primes = [o.primes[i] for i in base]
    y = x
    if ops & 1:
        y = o.pb_to_crt(y, base)
    if ops & 2:
        y = np.ascontiguousarray(y).copy()
        po.mul_mont64(y, np.ascontiguousarray(op), primes)
    if ops & 4:
        y = o.crt_to_pb(y, base)
    return y


# (ring, count, base, operand count)
ITEMS = [("field_36864", 2, [0, 1], 2), ("field_49152", 1, [0, 2], 1), ("field_18", 3, [0, 1, 2], 1),
         ("field_36864", 1, [3, 5, 7], 1), ("field_18", 1, [4], 1)]


def build(po, rings, seed, ops, items=ITEMS):
    import ringcuda

    g = np.random.default_rng(seed)
    batch_items, checks = [], []
    for name, count, base, opc in items:
        o, d = rings(name)
        primes = [o.primes[i] for i in base]
        x = residues(g, o.shape(count, len(base)), primes, 2)
        op = residues(g, o.shape(opc, len(base)), primes, 1)
        dx = d.tensor(x)
        dop = d.tensor(op) if ops & 2 else None
        batch_items.append((d, dx, dop, base))
        checks.append((dx, expected(po, o, x, op, base, ops)))
    return ringcuda.CrtBatch(batch_items, ops), checks


@pytest.mark.parametrize("ops", [7, 1, 4, 2, 5, 3, 6])
def test_crt_batch_matches_oracle(po, be, rings, ops):
    batch, checks = build(po, rings, 100 + ops, ops)
    batch.run()
    for i, (dx, exp) in enumerate(checks):
        assert (dx.to_numpy() == exp).all(), "item %d" % i
    batch.close()


@pytest.mark.parametrize("shape", [(128, 1, 4), (256, 3, 6), (64, 2, 0), (256, 1, 5), (96, 4, 3)])
def test_crt_batch_launch_shapes(po, be, rings, shape):
    batch, checks = build(po, rings, 7, 7)
    batch.launch = shape
    assert batch.launch == shape
    batch.run()
    for i, (dx, exp) in enumerate(checks):
        assert (dx.to_numpy() == exp).all(), "item %d" % i


def test_crt_batch_tuned_and_graph_replay(po, be, rings):
    import halcuda

    batch, checks = build(po, rings, 11, 7)
    shape = batch.tune(reps=1)
    assert batch.launch == shape and shape[0] in (128, 256)
    # the tuner ran on scratch memory: the data is untouched until the batch runs
    graph = halcuda.Graph(be, batch.run)
    graph.launch()
    be.synchronize()
    for i, (dx, exp) in enumerate(checks):
        assert (dx.to_numpy() == exp).all(), "item %d" % i


def test_crt_batch_one_launch_per_shape_class(po, be, rings):
    """The batch runs one persistent kernel per shape class of its slabs: field_36864's and
    field_49152's specialised shapes and the generic tile programme (field_18) are three."""
    batch, checks = build(po, rings, 23, 7)
    l0 = be.launch_count()
    batch.run()
    be.synchronize()
    assert be.launch_count() - l0 == 3
    for i, (dx, exp) in enumerate(checks):
        assert (dx.to_numpy() == exp).all(), "item %d" % i
    single, checks1 = build(po, rings, 24, 7, items=[("field_49152", 2, [0, 1, 2], 1)])
    l0 = be.launch_count()
    single.run()
    be.synchronize()
    assert be.launch_count() - l0 == 1
    for dx, exp in checks1:
        assert (dx.to_numpy() == exp).all()


@pytest.mark.parametrize("items", [ITEMS, [("field_36864", 2, [0, 1, 2], 1), ("field_49152", 2, [0, 1], 2)]],
                         ids=["with-generic", "both-specialised"])
def test_crt_batch_one_launch_option(po, be, rings, items):
    """HC_CRT_ONE_LAUNCH: every slab in one persistent launch (the kernel carrying both specialised
    classes, or the generic programme), bit-exact like the per-class form."""
    import ringcuda

    batch, checks = build(po, rings, 29, 7 | ringcuda.CRT_ONE_LAUNCH, items=items)
    shape = batch.tune(reps=1)
    assert batch.launch == shape
    l0 = be.launch_count()
    batch.run()
    be.synchronize()
    assert be.launch_count() - l0 == 1
    for i, (dx, exp) in enumerate(checks):
        assert (dx.to_numpy() == exp).all(), "item %d" % i
