"""Host-side failure paths of the runtime and of the key-switch entry points, with no GPU fault:
a bounded event wait that gives up while the GPU is still busy (HC_ERR_TIMEOUT, the context stays
usable), and key switches refused on the host for operands of the wrong shape (HC_ERR_SHAPE)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ring(be):
    import ringcuda

    R = ringcuda.RingContext("field_36864", 900, 930, 8, backend=be)
    yield R
    R.close()


def test_bounded_event_wait_times_out_and_the_context_stays_usable(be, ring):
    import halcuda

    base = ring.initial_base()
    plans = [be.hal_create_ntt_plan(ring.modulus(i), [2, 3, 8, 64]) for i in base]
    t = ring.allocate(32, len(base))
    ev0, ev1 = halcuda.Event(), halcuda.Event()
    be.synchronize()
    ev0.record(be)
    # 400 inverse NTT passes over 151 MB: the GPU needs several times longer for them than the host
    # takes to issue them, so work is still queued when the bounded wait below starts
    for _ in range(400):
        be.hal_intt_mont64_dim(t, plans, halcuda.DIM3)
    ev1.record(be)
    with pytest.raises(halcuda.HalError, match="error 5: event wait timed out"):
        ev0.elapsed_ms(ev1, timeout_ms=1.0)
    ms = ev0.elapsed_ms(ev1, timeout_ms=0)  # unbounded: the work finishes normally
    assert ms > 1.0
    a = np.arange(24, dtype=np.int64).reshape(1, 2, 3, 4)
    da, db = be.tensor(a), be.tensor(2 * a)
    be.hal_add_i64(da, db)
    assert (da.to_numpy() == 3 * a).all()


def test_key_switch_refuses_wrong_shapes(be, ring):
    import halcuda

    base = ring.initial_base()
    r = len(base)
    digits = [(0, 4), (4, 8), (8, 12), (12, 16)]
    c0, c1 = ring.allocate(1, r), ring.allocate(1, r)
    keys = ring.allocate(8, r)
    with pytest.raises(halcuda.HalError, match="error 1: key switch c0"):
        ring.key_switch(ring.allocate(1, r - 1), c1, base, keys, digits)
    with pytest.raises(halcuda.HalError, match="error 1: key switch c0"):
        ring.key_switch(ring.allocate(2, r), c1, base, keys, digits)
    with pytest.raises(halcuda.HalError, match="error 1: key switch c1"):
        ring.key_switch(c0, ring.allocate(1, r - 2), base, keys, digits)
    with pytest.raises(halcuda.HalError, match="error 1: key tensor"):
        ring.key_switch(c0, c1, base, be.hal_allocate_i64((8, r, ring.dl, ring.dk // 2)), digits)
    with pytest.raises(halcuda.HalError, match="error 1: key tensor too small"):
        ring.key_switch(c0, c1, base, ring.allocate(6, r), digits)
    # the refused calls left the context usable: a valid key switch runs
    out = ring.key_switch(c0, c1, base, keys, digits)
    assert out.shape == (2, r, ring.dl, ring.dk)
