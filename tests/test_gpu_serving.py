"""The serving engine: every request's result is the same whether it runs alone or inside the
mixed, continuously batched stream (bit-exact, the tolerance of all integer work here), also when
the HBM budget lets only one request in flight at a time."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fields(be):
    import serving

    return {
        "field_36864": serving.FieldState(be, "field_36864", (280, 300), 256, [4, 5], 2, 3283177, seed=1),
        "field_49152": serving.FieldState(be, "field_49152", (280, 300), 256, [4, 5], 2, 20965738, seed=2),
    }


def run_and_check(be, fields, budget, batched):
    import serving

    reqs = serving.make_stream(40, 2000.0, [0.5, 0.35, 0.15], sorted(fields), (4, 5), 2, seed=9)
    eng = serving.Engine(be, fields, budget, max_batch=8)
    stats = eng.run(reqs, batched=batched, keep_outputs=True)
    assert stats["requests"] == 40 and all(q.t_done >= q.arrival for q in reqs)
    mixed = {q.rid: q.out.to_numpy() for q in reqs}
    for q in reqs:
        alone = serving.Request(q.rid, q.op, q.field, q.level, 0.0, q.slot)
        eng.submit([alone])
        assert (alone.out.to_numpy() == mixed[q.rid]).all(), (q.op, q.field, q.level)
    return stats


def test_results_alone_equal_results_in_the_mix(be, fields):
    stats = run_and_check(be, fields, 8 << 30, batched=True)
    assert stats["batches"] <= 40


def test_results_equal_under_a_one_request_budget(be, fields):
    run_and_check(be, fields, 1, batched=True)


def test_plain_form_equal(be, fields):
    stats = run_and_check(be, fields, 8 << 30, batched=False)
    assert stats["batches"] == 40
