"""Host-side logic of the serving engine (no GPU): the seeded Poisson request stream."""
import numpy as np
import pytest


def test_stream_is_seeded_poisson_with_the_requested_mix():
    serving = pytest.importorskip("serving")
    a = serving.make_stream(20000, 2000.0, [0.5, 0.35, 0.15], ["field_36864", "field_49152"], (4, 20), 3, seed=5)
    b = serving.make_stream(20000, 2000.0, [0.5, 0.35, 0.15], ["field_36864", "field_49152"], (4, 20), 3, seed=5)
    assert [(q.op, q.field, q.level, q.arrival) for q in a] == [(q.op, q.field, q.level, q.arrival) for q in b]
    arr = np.array([q.arrival for q in a])
    assert arr[0] == 0.0 and (np.diff(arr) >= 0).all()
    rate = (len(a) - 1) / arr[-1]
    assert abs(rate - 2000.0) / 2000.0 < 0.03
    ops = [q.op for q in a]
    for op, p in (("mul", 0.5), ("rot", 0.35), ("crt", 0.15)):
        assert abs(ops.count(op) / len(a) - p) < 0.02
    levels = [q.level for q in a]
    assert min(levels) == 4 and max(levels) == 20
    assert abs(sum(q.field == "field_49152" for q in a) / len(a) - 0.5) < 0.02
