"""Benchmark of the GB300 ring-arithmetic backend.

Workload (BFV ciphertext multiplication at full size): field_36864 (n = 36864 = 12 x 3072), an
initial RNS base of r = 16 primes of 57 bits (log2 q in 900..930), plaintext modulus t = 256,
secret key sparse ternary, error sigma = 3.2, relinearisation key with ceil(r/4) = 4 gadget digits.
The plain GPU form: one step is one ciphertext multiplication per launch (bfv_hom_mul incl.
lifting, tensoring, rescaling and relinearisation, replayed from a CUDA graph of the call), the
steps cycling over B = 8 seeded synthetic ciphertext pairs (larger than L2 together) on two
streams. The batched form (all B pairs in one call) is reported beside it.

Prints one JSON line. `value` is ct-mults/s with the operands resident in HBM; `e2e` is the same
metric through the C ABI with each step's operands copied from pinned host memory and its result
copied back inside the timed region. `--impl reference` times the oracle, the CPU restatement of
the reference's hal::cpu path (the Rust crate cannot be built here), on all host cores.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cyclosubfield-dbfv_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "CRT transforms/s & ct-mults/s, batched vs plain on 1 GB300, bit-exact; p99 ms"
FIELD, LOG2_Q, T_BITS, T = "field_36864", (900, 930), 8, 256
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=8, help="ciphertext pairs (cycled one per step; all in one "
                                                            "call in the batched form)")
    ap.add_argument("--streams", type=int, default=2, help="streams the one-ct-mult launches alternate on")
    ap.add_argument("--e2e-slots", type=int, default=4, help="operand slots (and streams) of the e2e pipeline "
                                                              "(a divisor of --batch)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-crt-batch", action="store_true", help="skip the batched CRT-transform workload")
    ap.add_argument("--no-homcrt", action="store_true", help="skip the homomorphic CRT transform workload")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving workload")
    ap.add_argument("--only", choices=["crt_batch", "homcrt", "serving"],
                    help="run just this workload and print its result (for profiling it alone)")
    ap.add_argument("--roofline-only", action="store_true",
                    help="time only the dominant NTT kernel (the launches a profile of it captures)")
    ap.add_argument("--transform-only", action="store_true",
                    help="time only the fused CRT transform passes (the launches a profile of them captures)")
    return ap.parse_args()


# ------------------------------------------------------------------------------ distributed
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())


# ------------------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clocks and throttle reasons during the timed region."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.begin = self.end = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.1)  # the sampler's first query precedes the timed region

    def mark(self, begin):
        """Host wall-clock bounds of the timed region (the samples inside them are the ones reported)."""
        import datetime

        if begin:
            self.begin = datetime.datetime.now()
        else:
            self.end = datetime.datetime.now()

    def stop(self):
        import datetime

        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.05)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        rows = []
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f")
                rows.append((ts, float(f[2]), float(f[3]), f[6:10]))
            except ValueError:
                continue
        inside = [r for r in rows if self.begin and self.end and self.begin <= r[0] <= self.end]
        use = inside or rows  # a region shorter than the sampling period: the samples around it
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in use:
            for name, val in zip(names, r[3]):
                if val.lower() == "active":
                    reasons.add(name)
        sm = [r[1] for r in use]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": use[-1][2] if use else None,
                "samples": len(use), "samples_in_timed_region": len(inside), "reasons": sorted(reasons)}


# ------------------------------------------------------------------------------ workload
class Workload:
    def __init__(self, be, batch, seed=2026):
        import halcuda
        import ringcuda

        self.be = be
        self.ring = ringcuda.RingContext(FIELD, LOG2_Q[0], LOG2_Q[1], T_BITS, backend=be)
        R = self.ring
        self.base = R.initial_base()
        self.r = len(self.base)
        self.digits = ringcuda.select_digits(math.ceil(self.r / 4), self.r)
        la = R.log2_alpha_for_sigma(self.base, 3.2)
        st = [seed]
        self.sk = R.gen_sk(st)
        self.rk = R.gen_rk(st, self.sk, self.digits, la)
        self.batch = batch
        # B ciphertext pairs stacked along dimension 0: rows 2b, 2b + 1 hold pair b
        self.ct1, self.ct2 = R.allocate(2 * batch, self.r), R.allocate(2 * batch, self.r)
        for b in range(batch):
            m1 = [((i * 7 + b) % 255) - 127 for i in range(R.n)]
            m2 = [((i * 13 + 3 * b) % 255) - 127 for i in range(R.n)]
            be.hal_assign(self.ct1.rows(2 * b, 2 * b + 2), R.enc(st, self.base, T, m1, self.sk, la))
            be.hal_assign(self.ct2.rows(2 * b, 2 * b + 2), R.enc(st, self.base, T, m2, self.sk, la))
        self.out = R.allocate(2 * batch, self.r)
        self.ct_bytes = 2 * self.r * R.n * 8
        self.step()  # first use builds the ring's caches (host synchronising); then capture
        be.synchronize()
        self.graph = halcuda.Graph(be, self.step)
        # one graph per pair: one ct-mult per launch
        self.single = [halcuda.Graph(be, lambda b=b: self.plain(b)) for b in range(batch)]

    def step(self):
        """All B ct-mults in one call: every stage launches once over the whole batch."""
        self.ring.hom_mul(T, self.ct1, self.ct2, self.base, self.rk, self.digits, out=self.out)

    def slots(self, n=2):
        """`n` one-pair operand slots for multi-buffering: pair 0 with its one-ct-mult graph, and
        n - 1 more sets with copies of pair 0's operands and their own captured calls."""
        import halcuda
        import types

        R = self.ring
        out = [types.SimpleNamespace(ct1=self.ct1.rows(0, 2), ct2=self.ct2.rows(0, 2), out=self.out.rows(0, 2),
                                     graph=self.single[0])]
        for _ in range(n - 1):
            b = types.SimpleNamespace(ct1=R.allocate(2, self.r), ct2=R.allocate(2, self.r), out=R.allocate(2, self.r))
            self.be.hal_assign(b.ct1, self.ct1.rows(0, 2))
            self.be.hal_assign(b.ct2, self.ct2.rows(0, 2))
            self.be.synchronize()
            b.graph = halcuda.Graph(self.be, lambda b=b: R.hom_mul(T, b.ct1, b.ct2, self.base, self.rk, self.digits,
                                                                   out=b.out))
            b.graph.launch()  # the first replay uploads the graph; keep it out of the timed region
            self.be.synchronize()
            out.append(b)
        return out

    def plain(self, b):
        """One ct-mult per call, the reference's calling pattern."""
        self.ring.hom_mul(T, self.ct1.rows(2 * b, 2 * b + 2), self.ct2.rows(2 * b, 2 * b + 2), self.base, self.rk,
                          self.digits, out=self.out.rows(2 * b, 2 * b + 2))


class CrtWorkload:
    """Batched CRT transforms: `elements` ring elements, the field drawn uniformly from
    {field_36864, field_49152} and the RNS length uniformly from 4..24 (seeded); each element goes
    period basis -> CRT basis, Montgomery product with a seeded operand, CRT basis -> period
    basis. Residues are uniform in [-2^56, 2^56), below every 57-bit factor. Elements of the same
    field and length share one tensor; the batch runs them all in one persistent launch."""

    FIELDS = (("field_36864", 900, 930, 8), ("field_49152", 1280, 1310, 2))

    def __init__(self, be, elements=512, seed=3):
        import numpy as np

        import ringcuda

        self.be = be
        self.rings = [ringcuda.RingContext(f, lo, hi, tb, backend=be) for f, lo, hi, tb in self.FIELDS]
        g = np.random.default_rng(seed)
        fields = g.integers(0, 2, size=elements)
        lens = g.integers(4, 25, size=elements)
        groups = {}
        for f, r in zip(fields.tolist(), lens.tolist()):
            groups[(f, r)] = groups.get((f, r), 0) + 1
        block = g.integers(-(1 << 56), 1 << 56, size=1 << 22, dtype=np.int64)
        self.items, self.elements, self.residues = [], elements, 0
        for (f, r), c in sorted(groups.items()):
            R = self.rings[f]
            shape = R.shape(c, r)
            size = c * r * R.dl * R.dk
            reps = -(-size // block.size)
            x = be.tensor(np.tile(block, reps)[:size].reshape(shape))
            op = be.tensor(np.tile(block[::-1], reps)[:size].reshape(shape))
            self.items.append((R, x, op, list(range(r))))
            self.residues += size
        self.batch = ringcuda.CrtBatch(self.items, ringcuda.CRT_FORWARD | ringcuda.CRT_MUL | ringcuda.CRT_INVERSE,
                                       backend=be)
        self.launch = self.batch.tune(reps=2)
        self.batch.run()
        be.synchronize()
        import halcuda

        self.graph = halcuda.Graph(be, self.batch.run)

    def plain_element(self, R, x, op, base, mods, i):
        """One element with the HAL/ring calls of the reference, one launch per pass."""
        xi, oi = x.rows(i, i + 1), op.rows(i, i + 1)
        R.pb_to_crt(xi, base)
        self.be.hal_mul_mont64(xi, oi, mods)
        R.crt_to_pb(xi, base)


def crt_batch_bench(be, steps, warmup):
    """CRT transforms/s (2 per element: forward and inverse) batched (graph replay of the persistent
    launch) and plain (one element at a time); inputs ~2.5 GB, larger than L2."""
    import halcuda

    w = CrtWorkload(be)
    ev0, ev1 = halcuda.Event(), halcuda.Event()
    for _ in range(warmup):
        w.graph.launch()
    be.synchronize()
    l0 = be.launch_count()
    ev0.record(be)
    for _ in range(steps):
        w.graph.launch()
    ev1.record(be)
    ms = ev0.elapsed_ms(ev1) / steps
    launches = (be.launch_count() - l0) // steps
    # host-side modulus lists are built outside the timed region
    plain_items = [(R, x, op, base, R.mods_for(base)) for R, x, op, base in w.items]
    w.plain_element(*plain_items[0], 0)
    be.synchronize()
    ev0.record(be)
    for R, x, op, base, mods in plain_items:
        for i in range(x.shape[0]):
            w.plain_element(R, x, op, base, mods, i)
    ev1.record(be)
    plain_ms = ev0.elapsed_ms(ev1)
    n = w.elements
    return {"workload": "%d elements, field uniform in {field_36864, field_49152}, RNS length uniform in 4..24; "
                        "each pb->crt, mul_mont64 by an operand, crt->pb" % n,
            "elements": n, "slabs": w.batch.num_slabs, "residues": w.residues,
            "crt_transforms_per_s": round(2 * n / (ms * 1e-3), 1),
            "plain_crt_transforms_per_s": round(2 * n / (plain_ms * 1e-3), 1),
            "ms_per_batch": round(ms, 4), "plain_ms_per_batch": round(plain_ms, 4),
            "launches_per_batch": launches, "plain_launches_per_batch": 9 * n,
            "launch_shape": {"threads": w.launch[0], "ctas_per_sm": w.launch[1], "dim2_columns": 1 << w.launch[2]},
            "autotuned": True, "l2": "inputs 2 x %.1f GB, larger than L2" % (w.residues * 8 / 1e9)}


def homcrt_bench(be, reps=3):
    """Homomorphic CRT transform step (hom_cyclic_transform_dbfv) on field_49152, r = 23 factors
    (log2 q in 1280..1310), dBFV modulus t = 2^24 in 3 digits of 8 bits: sum_{i < 64} c_i sigma^i(ct)
    for the descriptor's order-64 generator, 13 baby steps and 5 giant steps, 13 Galois keys with
    6 gadget digits (108 MB each). Timed with every key resident in HBM, and with an HBM key budget
    of 8 keys, the other 5 streamed from pinned host memory for every use."""
    import numpy as np

    import halcuda
    import ringcuda

    R = ringcuda.RingContext("field_49152", 1280, 1310, 2, backend=be)
    base = R.initial_base()
    r = len(base)
    log2_b, log2_t, g, length = 8, 24, 20965738, 64
    digits = ringcuda.select_digits(math.ceil(r / 4), r)
    la = R.log2_alpha_for_sigma(base, 3.2)
    st = [99]
    sk = R.gen_sk(st)
    m = 35297665
    baby = min(range(1, length + 1), key=lambda c: (c + 3 * ((length - 1) // c + 1), c))
    giant = (length - 1) // baby + 1
    gs = sorted(set([pow(g, j, m) for j in range(1, baby)] + [pow(g, baby, m)]))
    keys = {gg: R.gen_gk(st, sk, gg, digits, la) for gg in gs}
    t = 1 << log2_t
    rng = np.random.default_rng(5)
    ct = R.allocate(6, r)
    be.hal_assign(ct.rows(0, 2), R.enc(st, base, t, [int(v) for v in rng.integers(0, t, size=R.n)], sk, la))
    for dd in (1, 2):
        be.hal_assign(ct.rows(2 * dd, 2 * dd + 2), R.enc(st, base, t, [0] * R.n, sk, la))
    coeffs = [[int(v) for v in rng.integers(-t // 2, t // 2, size=R.dl)] for _ in range(length)]
    key_bytes = 2 * len(digits) * r * R.n * 8
    out = {"workload": "hom_cyclic_transform_dbfv field_49152 r=%d, t=2^%d (b=2^%d, 3 digits), len %d "
                       "(%d baby x %d giant steps), %d Galois keys of %d gadget digits"
                       % (r, log2_t, log2_b, length, baby, giant, len(gs), len(digits)),
           "key_MB": round(key_bytes / 1e6, 1), "keys": len(gs)}
    ev0, ev1 = halcuda.Event(), halcuda.Event()
    for label, budget in (("resident", len(gs)), ("streamed", 8)):
        ks = ringcuda.Keyset(R, digits, r, budget * key_bytes)
        for gg in gs:
            ks.add(gg, keys[gg])
        ringcuda.dbfv_hom_cyclic_transform(R, log2_b, log2_t, g, coeffs, ct, base, ks)  # warm-up (tables)
        be.synchronize()
        s0 = ks.stats()
        ev0.record(be)
        for _ in range(reps):
            ringcuda.dbfv_hom_cyclic_transform(R, log2_b, log2_t, g, coeffs, ct, base, ks)
        ev1.record(be)
        ms = ev0.elapsed_ms(ev1) / reps
        s1 = ks.stats()
        out[label] = {"ms_per_transform": round(ms, 3), "resident_keys": s1["resident"], "streamed_keys": s1["streamed"],
                      "streamed_GB_per_transform": round((s1["streamed_bytes"] - s0["streamed_bytes"]) / reps / 1e9, 3)}
        ks.close()
    out["key_switches_per_transform"] = 3 * (baby - 1) + 3 * (giant - 1)
    R.close()
    return out


def serving_bench(be, n=4000, rate=2000.0):
    """Serving: a seeded Poisson stream of `n` requests at `rate` per second - ciphertext
    multiplications 50 %, automorphisms 35 %, standalone CRT transforms 15 % - over field_36864
    and field_49152 (log2 q in 1100..1140, t = 256) at RNS levels uniform in 4..20, keys resident
    in HBM, admission by an HBM budget of 16 GB; continuously batched and plain (one request per
    call) through the same engine."""
    import serving

    fields = {
        "field_36864": serving.FieldState(be, "field_36864", (1100, 1140), 256, range(4, 21), 2, 3283177, seed=11),
        "field_49152": serving.FieldState(be, "field_49152", (1100, 1140), 256, range(4, 21), 2, 20965738, seed=12),
    }
    out = {"workload": "%d requests, Poisson %.0f/s, mix mul/rot/crt 50/35/15, fields field_36864 + field_49152, "
                       "levels 4..20, keys in HBM, HBM admission budget 16 GB" % (n, rate)}
    serving.Engine(be, fields, 16 << 30).warm()  # builds the rings' tables
    for label, batched in (("batched", True), ("plain", False)):
        reqs = serving.make_stream(n, rate, [0.5, 0.35, 0.15], sorted(fields), (4, 20), 2, seed=7)
        out[label] = serving.Engine(be, fields, 16 << 30).run(reqs, batched=batched)
    # capacity: the same requests all arriving at once (the engine's saturated throughput)
    reqs = serving.make_stream(n, 1e9, [0.5, 0.35, 0.15], sorted(fields), (4, 20), 2, seed=7)
    out["capacity_batched"] = serving.Engine(be, fields, 16 << 30).run(reqs, batched=True)
    for f in fields.values():
        f.ring.close()
    return out


def flush_l2(be, scratch):
    import halcuda

    halcuda.memset_async(be, scratch.ptr, 0, scratch.numel() * 8)


def timed_steps(be, work, steps, scratch):
    """Sum of CUDA-event times of `steps` graph replays (L2 flushed before each, outside the events)."""
    import halcuda

    ev0, ev1 = halcuda.Event(), halcuda.Event()
    total = 0.0
    for _ in range(steps):
        flush_l2(be, scratch)
        ev0.record(be)
        work.graph.launch()
        ev1.record(be)
        total += ev0.elapsed_ms(ev1)
    return total


def single_steps(be, work, steps, streams, start=0):
    """`steps` ct-mults, one per launch: step k replays the one-pair graph of pair (start + k) mod B
    on stream k mod 2 (a graph stays on one stream), back to back. The pairs' operands and results
    (B = 8: 226 MB) exceed L2, so a step's inputs are not cached from its previous use. Returns the
    CUDA-event time from before the first to after the last step."""
    import halcuda

    ev0, ev1 = halcuda.Event(), halcuda.Event()
    ends = [halcuda.Event() for _ in streams]
    ev0.record(be)
    for st in streams:
        with be.on(st):
            ev0.wait(be)
    for k in range(steps):
        b = (start + k) % work.batch
        with be.on(streams[b % len(streams)]):
            work.single[b].launch()
    for e, st in zip(ends, streams):
        with be.on(st):
            e.record(be)
        e.wait(be)
    ev1.record(be)
    return ev0.elapsed_ms(ev1)


def plain_calls(be, work, rounds, scratch):
    """Per-call event times of the plain form (one ct-mult per call, no graph)."""
    import halcuda

    ev0, ev1 = halcuda.Event(), halcuda.Event()
    per = []
    for _ in range(rounds):
        flush_l2(be, scratch)
        for b in range(work.batch):
            ev0.record(be)
            work.plain(b)
            ev1.record(be)
            per.append(ev0.elapsed_ms(ev1))
    return per


def e2e_steps(be, work, steps, nslots=4):
    """One ct-mult per step through the C ABI with host buffers: step k copies pair k mod B's
    operands from pinned host memory into device slot k mod nslots, replays the slot's one-pair
    call and copies the result back to pinned host memory, all inside the timed region. The slots
    take turns on their own streams, so some slots' copies overlap the others' compute. Every
    copied-back result is checked against the resident run's."""
    import halcuda
    import numpy as np

    R = work.ring
    full = (2 * work.batch, work.r, R.dl, R.dk)
    slots = work.slots(nslots)
    h1, h2, hout = halcuda.PinnedBuffer(full), halcuda.PinnedBuffer(full), halcuda.PinnedBuffer(full)
    h1.array[...] = work.ct1.to_numpy()
    h2.array[...] = work.ct2.to_numpy()
    hout.array[...] = 0
    streams = [halcuda.Stream() for _ in slots]
    nbytes = work.ct_bytes  # one ciphertext pair's operand (or result) bytes
    ev0, ev1 = halcuda.Event(), halcuda.Event()
    ends = [halcuda.Event() for _ in slots]
    be.synchronize()
    expect = work.out.to_numpy()
    ev0.record(be)
    for st in streams:
        with be.on(st):
            ev0.wait(be)
    for step in range(steps):
        k, b = step % len(slots), step % work.batch
        sl, off = slots[k], b * nbytes
        with be.on(streams[k]):
            halcuda.memcpy_async(be, sl.ct1.ptr, h1.ptr + off, nbytes, halcuda.H2D)
            halcuda.memcpy_async(be, sl.ct2.ptr, h2.ptr + off, nbytes, halcuda.H2D)
            sl.graph.launch()
            halcuda.memcpy_async(be, hout.ptr + off, sl.out.ptr, nbytes, halcuda.D2H)
    for k, st in enumerate(streams):
        with be.on(st):
            ends[k].record(be)
        ends[k].wait(be)
    ev1.record(be)
    ms = ev0.elapsed_ms(ev1)
    be.synchronize()
    for b in range(min(steps, work.batch)):
        if not np.array_equal(hout.array[2 * b:2 * b + 2], expect[2 * b:2 * b + 2]):
            raise RuntimeError("e2e: the result of pair %d copied back differs from the resident run" % b)
    for st in streams:
        st.close()
    return ms, 2 * nbytes, nbytes, hout


# DRAM bytes (read + written) of one launch of that kernel on the [24, 34, 12, 3072] tensor, and
# the busy fraction of the integer multiply (fmaheavy, IMAD family) pipe over its elapsed cycles,
# from one ncu capture of `python bench.py --roofline-only` (None: not captured for this build).
NCU_TRAFFIC_BYTES = 240784640 + 179246592
NCU_IMAD_PIPE_FRAC = 0.811
ROOF_ROWS = 24  # ciphertext rows of the roofline tensor: 240 MB, larger than L2


def kernel_roofline(be, R, base, reps, peaks):
    """Dominant kernel: the dimension-3 lazy NTT of the transforms (one HAL launch of the
    specialised [2, 3, 8, 64] line kernel), timed alone on a [24, r + e, 12, 3072] tensor of
    lifted products (eight ct-mults' worth, 240 MB: larger than L2, so every launch reads and
    writes HBM). Algorithmic bytes per launch: one read and one write of every i64 residue
    (16 B per residue)."""
    import halcuda

    lifted = base + R.extension_base(base)
    t = R.allocate(ROOF_ROWS, len(lifted))
    plans = [R_plan for R_plan in _k_plans(R, lifted)]
    ev0, ev1 = halcuda.Event(), halcuda.Event()
    for _ in range(3):
        be.hal_intt_mont64_dim(t, plans, halcuda.DIM3)
    be.synchronize()
    ev0.record(be)
    for _ in range(reps):
        be.hal_intt_mont64_dim(t, plans, halcuda.DIM3)
    ev1.record(be)
    ms = ev0.elapsed_ms(ev1) / reps
    bytes_alg = 16 * ROOF_ROWS * len(lifted) * R.n
    achieved = bytes_alg / (ms * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs")
    # the binding roof: Barrett products. The pass's algorithmic count is 7 per residue (ten radix-2
    # stages at 1/2 and one radix-3 stage at 2, the reference's formula), against the GPU's
    # measured rate of the same product in a register-only kernel
    products = 7 * ROOF_ROWS * len(lifted) * R.n
    bpeak = halcuda.barrett_peak(be)
    int_roof = {"bound": "int (exact 64-bit Barrett products)", "achieved": round(products / (ms * 1e-3) / 1e9, 1),
                "peak": round(bpeak / 1e9, 1), "unit": "G products/s",
                "frac": round(products / (ms * 1e-3) / bpeak, 4), "products_per_launch": products,
                "peak_source": "measured here: register-only kernel of the same product (hc_barrett_peak)"}
    return {"kernel": "ntt_line_kernel (inverse, dim 3, lines [2, 3, 8, 64], tensor [%d, %d, 12, 3072])"
                      % (ROOF_ROWS, len(lifted)),
            "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4) if peak else None,
            "traffic": NCU_TRAFFIC_BYTES if len(lifted) == 34 else None,
            "bytes_per_launch": bytes_alg, "launch_ms": round(ms, 5),
            "l2": "tensor of %d MB, larger than L2" % (bytes_alg // 2 // 2**20),
            "peak_source": "measured" if not peaks.get("fallback") else "fallback",
            "int_pipe": {"pipe": "fmaheavy (IMAD)", "busy_frac_of_elapsed": NCU_IMAD_PIPE_FRAC,
                         "source": "ncu capture of the same launch (--roofline-only)"},
            "int_roofline": int_roof,
            "note": "bit-exact lazy Barrett NTT: bound by the 32-bit integer multiply pipe, not by HBM; the binding "
                    "roof is int_roofline (%.2f of the measured Barrett-product rate)" % int_roof["frac"]}


# Exact 64-bit products per residue of one CRT transform (pb_to_crt or crt_to_pb, the reference's
# formula: F = sum over NTT stages of 1/2 per radix-2 and 2 per radix-3 stage, forward and inverse,
# plus the two kernel products): field_36864 rows [4, 3] and lines [2, 3, 8, 64]: F = 3 + 7 per
# direction, 22 per transform; field_49152 rows [4] and lines [3, 64, 64]: F = 1 + 8, 20.
TRANSFORM_PRODUCTS = {"field_36864": 22, "field_49152": 20}


def transform_roofline(be, R, base, reps, peaks, rows=ROOF_ROWS):
    """The fused CRT transform passes (csrc/crt_fused.cu): pb_to_crt of a [rows, r + e, 12, 3072]
    tensor of lifted products (240 MB, larger than L2) in its two cluster launches, timed with
    CUDA events on the library's stream. Algorithmic bytes: one read and one write of every
    residue per launch (32 B per residue per transform); algorithmic products: 22 per residue."""
    import halcuda

    lifted = base + R.extension_base(base)
    t = R.allocate(rows, len(lifted))
    ev0, ev1 = halcuda.Event(), halcuda.Event()
    for _ in range(3):
        R.pb_to_crt(t, lifted)
    be.synchronize()
    l0 = be.launch_count()
    ev0.record(be)
    for _ in range(reps):
        R.pb_to_crt(t, lifted)
    ev1.record(be)
    ms = ev0.elapsed_ms(ev1) / reps
    launches = (be.launch_count() - l0) // reps
    # the same transform as the reference's four HAL calls, one launch per dimension and direction
    import numpy as np

    ker = [R.crt_kernels(i) for i in lifted]
    kl = be.tensor(np.stack([k[0] for k in ker]).reshape(1, len(lifted), R.dl, 1))
    kk = be.tensor(np.stack([k[1] for k in ker]).reshape(1, len(lifted), 1, R.dk))
    p2 = [be.hal_create_ntt_plan(R.modulus(i), [4, 3]) for i in lifted]
    p3 = _k_plans(R, lifted)
    mods = R.mods_for(lifted)

    def four_calls():
        be.hal_ntt_mul_mont64_dim(t, p2, halcuda.DIM2, kl, mods)
        be.hal_ntt_mul_mont64_dim(t, p3, halcuda.DIM3, kk, mods)
        be.hal_intt_mont64_dim(t, p2, halcuda.DIM2)
        be.hal_intt_mont64_dim(t, p3, halcuda.DIM3)

    four_calls()
    be.synchronize()
    ev0.record(be)
    for _ in range(reps):
        four_calls()
    ev1.record(be)
    ms4 = ev0.elapsed_ms(ev1) / reps
    residues = rows * len(lifted) * R.n
    bytes_alg = 16 * launches * residues
    products = TRANSFORM_PRODUCTS[FIELD] * residues
    bpeak = halcuda.barrett_peak(be)
    peak = peaks.get("hbm_gbs")
    achieved = bytes_alg / (ms * 1e-3) / 1e9
    return {"kernel": "crt_slab3072_kernel (fused CRT passes, pb_to_crt of [%d, %d, 12, 3072])" % (rows, len(lifted)),
            "launches_per_transform": launches, "ms_per_transform": round(ms, 5),
            "four_hal_calls_ms_per_transform": round(ms4, 5),
            "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4) if peak else None, "bytes_per_transform": bytes_alg,
            "int_roofline": {"achieved": round(products / (ms * 1e-3) / 1e9, 1), "peak": round(bpeak / 1e9, 1),
                             "unit": "G products/s", "frac": round(products / (ms * 1e-3) / bpeak, 4),
                             "products_per_transform": products}}


_PLAN_CACHE = {}


def _k_plans(R, base):
    key = (id(R), tuple(base))
    if key not in _PLAN_CACHE:
        be = R.backend
        _PLAN_CACHE[key] = [be.hal_create_ntt_plan(R.modulus(i), [2, 3, 8, 64]) for i in base]
    return _PLAN_CACHE[key]


def cpu_baseline(seconds_budget=12.0):
    """The oracle (single thread, restating the reference's hal::cpu path) on one ct-mult."""
    from oracle import pyoracle as po

    o = po.Ring(FIELD, LOG2_Q[0], LOG2_Q[1], T_BITS)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [7]
    sk = o.gen_sk(st)
    digits = po.select_digits(math.ceil(len(base) / 4), len(base))
    rk = o.gen_rk(st, sk, digits, la)
    c1 = o.enc(st, base, T, [1] * o.n, sk, la)
    c2 = o.enc(st, base, T, [2] * o.n, sk, la)
    n, t0 = 0, time.perf_counter()
    while True:
        o.hom_mul(T, c1, c2, base, rk, digits)
        n += 1
        el = time.perf_counter() - t0
        if el > seconds_budget:
            break
    return {"value": round(n / el, 4), "unit": "ct-mults/s", "cores": 1, "kind": "port",
            "sample": "%d bfv_hom_mul on %s r=%d (oracle C++ restatement of hal::cpu, g++ -O3 without CPU "
                      "tuning, 1 thread, %.1f s)"
                      % (n, FIELD, len(base), el)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


# ------------------------------------------------------------------------------ reference arm
_REF_STATE = {}


def _ref_init():
    from oracle import pyoracle as po

    o = po.Ring(FIELD, LOG2_Q[0], LOG2_Q[1], T_BITS)
    base = o.initial_base()
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [11 + os.getpid()]
    sk = o.gen_sk(st)
    digits = po.select_digits(math.ceil(len(base) / 4), len(base))
    rk = o.gen_rk(st, sk, digits, la)
    _REF_STATE.update(o=o, base=base, rk=rk, digits=digits, c1=o.enc(st, base, T, [1] * o.n, sk, la),
                      c2=o.enc(st, base, T, [3] * o.n, sk, la))


def _ref_task(_):
    s = _REF_STATE
    s["o"].hom_mul(T, s["c1"], s["c2"], s["base"], s["rk"], s["digits"])
    return 1


def reference_arm(args, dist):
    if dist.rank != 0:
        return
    import multiprocessing as mp

    from oracle import build as oracle_build

    oracle_build.build()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_ref_init) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_task, range(cores))
        t0 = time.perf_counter()
        done = 0
        for _ in range(args.steps):
            done += sum(pool.map(_ref_task, range(cores)))
        el = time.perf_counter() - t0
    value = done / el
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "ct-mults/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * el / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": {"workload": "bfv_hom_mul %s r=16 t=256, %d ct-mults per step (one per host core)"
                                   % (FIELD, cores), "field": FIELD, "rns_len": 16},
            "cpu_baseline": {"value": round(value, 4), "unit": "ct-mults/s", "cores": cores, "kind": "port",
                             "sample": "%d ct-mults per step on %d processes; oracle C++ restatement of the "
                                       "reference's hal::cpu path, g++ -O3 without CPU tuning (the Rust crate is not "
                                       "buildable here)"
                                       % (cores, cores)},
            "e2e": {"value": round(value, 4), "unit": "ct-mults/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------ main
def main():
    args = parse()
    dist = Dist()
    if args.impl == "reference":
        reference_arm(args, dist)
        return
    import halcuda

    halcuda.lib()
    be = halcuda.CudaBackend(dist.local_rank)
    if args.only:
        fn = {"crt_batch": lambda: crt_batch_bench(be, max(3, args.steps // 2), args.warmup),
              "homcrt": lambda: homcrt_bench(be, reps=max(1, args.steps // 3)),
              "serving": lambda: serving_bench(be)}[args.only]
        print(json.dumps({args.only: fn()}), flush=True)
        return
    if args.transform_only:
        import ringcuda

        ring = ringcuda.RingContext(FIELD, LOG2_Q[0], LOG2_Q[1], T_BITS, backend=be)
        print(json.dumps(transform_roofline(be, ring, ring.initial_base(), max(1, args.steps), load_peaks())),
              flush=True)
        return
    if args.roofline_only:
        import ringcuda

        ring = ringcuda.RingContext(FIELD, LOG2_Q[0], LOG2_Q[1], T_BITS, backend=be)
        print(json.dumps(kernel_roofline(be, ring, ring.initial_base(), max(1, args.steps), load_peaks())), flush=True)
        return
    work = Workload(be, args.batch)
    scratch = be.hal_allocate_i64((1, 1, 1, 2 * L2_BYTES // 8))
    peaks = load_peaks()

    streams = [halcuda.Stream() for _ in range(args.streams)]
    for g in work.single:  # first replays upload the graphs
        g.launch()
    single_steps(be, work, args.warmup, streams)
    be.synchronize()

    clocks = ClockSampler(dist.local_rank)
    dist.barrier()
    be.synchronize()
    clocks.start()
    launches0 = be.launch_count()
    clocks.mark(True)
    total_ms = single_steps(be, work, args.steps, streams, start=args.warmup)
    be.synchronize()
    clocks.mark(False)
    launches = be.launch_count() - launches0
    clk = clocks.stop()
    dist.barrier()
    total_ms = dist.max(total_ms)
    value = dist.world * args.steps / (total_ms * 1e-3)

    # the batched form: all B pairs in one call (one graph), L2 flushed before every step
    for _ in range(args.warmup):
        timed_steps(be, work, 1, scratch)
    nb = min(args.steps, 40)
    batched_ms = timed_steps(be, work, nb, scratch)
    batched = {"ct_mults_per_s": round(work.batch * nb / (batched_ms * 1e-3), 3), "batch": work.batch,
               "ms_per_step": round(batched_ms / nb, 4), "steps": nb,
               "l2": "flushed before every step (512 MB memset, untimed)"}

    # plain form (one ct-mult per timed call) and its latency distribution
    per = plain_calls(be, work, min(20, max(2, args.steps // 2)), scratch)
    per.sort()
    plain = 1e3 / statistics.mean(per)
    p50, p99 = per[len(per) // 2], per[min(len(per) - 1, int(math.ceil(0.99 * len(per))) - 1)]

    e2e_n = max(args.steps, 40)  # at least 40 steps, so that the pipeline's fill and drain stay small
    e2e_ms, h2d, d2h, _ = e2e_steps(be, work, e2e_n, args.e2e_slots)
    e2e_val = dist.world * e2e_n / (e2e_ms * 1e-3)
    roof = kernel_roofline(be, work.ring, work.base, 20, peaks)
    crt = None if args.no_crt_batch else crt_batch_bench(be, min(20, max(3, args.steps // 2)), args.warmup)
    hcrt = None if args.no_homcrt else homcrt_bench(be)
    srv = None if args.no_serving else serving_bench(be)

    if dist.rank != 0:
        return
    cpu = None if args.no_cpu_baseline else cpu_baseline()
    line = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "ct-mults/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int64",
        "data": "synthetic (seeded encryptions of the reference's parameter shapes)",
        "config": {"workload": "plain GPU form: one bfv_hom_mul per launch (one CUDA-graph replay of the call) "
                               "at %s r=%d t=%d d=%d" % (FIELD, work.r, T, len(work.digits)),
                   "field": FIELD, "rns_len": work.r,
                   "extension_len": len(work.ring.extension_base(work.base)), "gadget_digits": len(work.digits),
                   "ct_mults_per_step": 1, "streams": len(streams),
                   "l2": "steps cycle over %d ciphertext pairs (%d MB of operands and results, larger than L2); "
                         "no flush" % (work.batch, 3 * work.ct_bytes * work.batch // 2**20)},
        "batched": batched,
        "plain_ct_mults_per_s": round(plain, 3),
        "latency_ms": {"p50": round(p50, 4), "p99": round(p99, 4), "samples": len(per)},
        "e2e": {"value": round(e2e_val, 3), "unit": "ct-mults/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": roof,
        "clocks": clk,
    }
    if crt:
        line["crt_batch"] = crt
    if hcrt:
        line["homcrt"] = hcrt
    if srv:
        line["serving"] = srv
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
