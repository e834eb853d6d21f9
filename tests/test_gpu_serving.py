"""The serving engine: every request's result is the same whether it runs alone or inside the
mixed, continuously batched stream (bit-exact, the tolerance of all integer work here), also when
the HBM budget lets only one request in flight at a time."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fields(be):
    import serving

    out = {
        "field_36864": serving.FieldState(be, "field_36864", (280, 300), 256, [4, 5], 2, 3283177, seed=1),
        "field_49152": serving.FieldState(be, "field_49152", (280, 300), 256, [4, 5], 2, 20965738, seed=2),
    }
    yield out
    for F in out.values():
        F.close()


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


GENERATORS = {"field_36864": 3283177, "field_49152": 20965738}
SEEDS = {"field_36864": 3, "field_49152": 4}


@pytest.fixture(scope="module")
def streamed_fields(be, po):
    """Both fields with three Galois elements each (g, g^2, g^3) and an HBM key budget of no key:
    every Galois key is streamed from pinned host memory into a device slot per rotation."""
    import serving

    out = {}
    for name, gen in GENERATORS.items():
        m = po.field_info(name)["m"]
        gs = [pow(gen, k, m) for k in (1, 2, 3)]
        out[name] = serving.FieldState(be, name, (280, 300), 256, [4, 5], 2, gs, seed=SEEDS[name], resident_keys=0)
    yield out
    for F in out.values():
        F.close()


def _oracle_result(po, F, q):
    """The request's result from the oracle, with keys drawn from the same seeded generator in the
    same order as FieldState draws them (secret key, relinearisation key, the Galois keys)."""
    import math

    o = po.Ring(F.name, 280, 300, 8)
    full = o.initial_base()
    digits = po.select_digits(math.ceil(len(full) / 4), len(full))
    la = o.log2_alpha_for_sigma(full, 3.2)
    st = [SEEDS[F.name]]
    sk = o.gen_sk(st)
    rk = o.gen_rk(st, sk, digits, la)
    gks = {g: o.gen_gk(st, sk, g, digits, la) for g in F.gs}
    base = list(range(q.level))
    c1, c2 = (x.to_numpy() for x in F.pool[q.level][q.slot])
    if q.op == "mul":
        return o.hom_mul(F.t, c1, c2, base, rk, digits)
    if q.op == "rot":
        g = q.g or F.gs[q.gi]
        return o.hom_gal(c1, base, [g], gks[g][None], digits)[0]
    return o.pb_to_crt(c1[0:1], base)


def test_streamed_galois_keys_alone_mix_and_oracle(be, po, streamed_fields):
    """Rotations by three automorphisms per field with every Galois key streamed in from pinned
    host memory: each result equals the request run alone, and the first request of every
    (operation, field) pair equals the oracle's bfv_hom_mul / bfv_hom_gal / pb_to_crt with the
    same seeded keys."""
    import serving

    fields = streamed_fields
    reqs = serving.make_stream(48, 2000.0, [0.3, 0.55, 0.15], sorted(fields), (4, 5), 2, seed=21, n_galois=3)
    copies0 = {n: F.keys.stats()["streamed_copies"] for n, F in fields.items()}
    eng = serving.Engine(be, fields, 8 << 30, max_batch=8)
    stats = eng.run(reqs, batched=True, keep_outputs=True)
    assert stats["requests"] == 48 and stats["failed"] == stats["refused"] == stats["cancelled"] == 0
    for n, F in fields.items():
        s = F.keys.stats()
        assert s["resident"] == 0 and s["streamed"] == 3 and s["streamed_copies"] > copies0[n]
    mixed = {q.rid: q.out.to_numpy() for q in reqs}
    for q in reqs:
        alone = serving.Request(q.rid, q.op, q.field, q.level, 0.0, q.slot, q.gi)
        eng.submit([alone])
        assert (alone.out.to_numpy() == mixed[q.rid]).all(), (q.op, q.field, q.level, q.gi)
    checked = set()
    for q in reqs:
        key = (q.op, q.field)
        if key in checked:
            continue
        checked.add(key)
        exp = np.asarray(_oracle_result(po, fields[q.field], q))
        assert (mixed[q.rid] == exp.reshape(mixed[q.rid].shape)).all(), key
    assert len(checked) == 6


def test_host_side_failures_do_not_stop_the_stream(be, fields, po):
    """Failures made on the host, with no GPU fault: requests above the per-request HBM limit are
    refused at admission, a rotation by an automorphism that has no key fails when the library
    refuses its batch, and cancelled requests are dropped before admission. Every other request
    completes with the same result as alone."""
    import serving

    reqs = serving.make_stream(40, 2000.0, [0.5, 0.35, 0.15], sorted(fields), (4, 5), 2, seed=9)
    limit = max(F.bytes_of("rot", 5) for F in fields.values())
    too_big = {q.rid for q in reqs if fields[q.field].bytes_of(q.op, q.level) > limit}
    assert too_big and len(too_big) < len(reqs)
    rots = [q for q in reqs if q.op == "rot" and q.rid not in too_big]
    m = po.field_info(rots[0].field)["m"]
    rots[0].g = pow(GENERATORS[rots[0].field], 7, m)  # no key for sigma_g^7
    keyless = {rots[0].rid}
    cancel = {q.rid for q in reqs[10:14] if q.rid not in too_big | keyless}
    eng = serving.Engine(be, fields, 8 << 30, max_batch=8, max_request_bytes=limit)
    for rid in cancel:
        eng.cancel(rid)
    stats = eng.run(reqs, batched=True, keep_outputs=True)
    assert stats["refused"] == len(too_big) and stats["cancelled"] == len(cancel)
    assert stats["failed"] == 1  # the keyless rotation was alone in its (op, field, level, g) group
    for q in reqs:
        if q.rid in too_big:
            assert q.error.startswith("refused") and q.out is None
        elif q.rid in cancel:
            assert q.cancelled and q.error == "cancelled" and q.out is None
        elif q.rid in keyless:
            assert q.error.startswith("failed") and "no Galois key" in q.error
        else:
            assert not q.error
            alone = serving.Request(q.rid, q.op, q.field, q.level, 0.0, q.slot)
            eng.submit([alone])
            assert (alone.out.to_numpy() == q.out.to_numpy()).all(), (q.op, q.field, q.level)


@pytest.mark.slow
def test_benchmark_parameters_against_the_oracle(be, po):
    """Serving at the benchmark's parameters (log2 q in 1100..1140, t = 256) at its largest level,
    20 factors, on both fields: one multiplication, one rotation and one transform each, served
    together in one stream, every result equal to the oracle's with the same seeded keys."""
    import math

    import serving

    fields, seeds = {}, {"field_36864": 31, "field_49152": 32}
    for name, gen in GENERATORS.items():
        fields[name] = serving.FieldState(be, name, (1100, 1140), 256, [20], 1, gen, seed=seeds[name])
    reqs = [serving.Request(k, op, name, 20, 0.0, 0) for k, (op, name) in
            enumerate((op, name) for name in sorted(fields) for op in serving.OPS)]
    stats = serving.Engine(be, fields, 16 << 30, max_batch=8).run(reqs, batched=True, keep_outputs=True)
    assert stats["requests"] == 6 and stats["failed"] == 0
    for q in reqs:
        F = fields[q.field]
        o = po.Ring(q.field, 1100, 1140, 8)
        full = o.initial_base()
        digits = po.select_digits(math.ceil(len(full) / 4), len(full))
        la = o.log2_alpha_for_sigma(full, 3.2)
        st = [seeds[q.field]]
        sk = o.gen_sk(st)
        rk = o.gen_rk(st, sk, digits, la)
        gk = o.gen_gk(st, sk, F.g, digits, la)
        base = list(range(20))
        c1, c2 = (x.to_numpy() for x in F.pool[20][0])
        if q.op == "mul":
            exp = o.hom_mul(F.t, c1, c2, base, rk, digits)
        elif q.op == "rot":
            exp = o.hom_gal(c1, base, [F.g], gk[None], digits)[0]
        else:
            exp = o.pb_to_crt(c1[0:1], base)
        got = q.out.to_numpy()
        assert (got == np.asarray(exp).reshape(got.shape)).all(), (q.op, q.field)
    for F in fields.values():
        F.close()
