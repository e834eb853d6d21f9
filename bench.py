"""Benchmark of the GB300 ring-arithmetic backend.

Workload (BFV ciphertext multiplication at full size): field_36864 (n = 36864 = 12 x 3072), an
initial RNS base of r = 16 primes of 57 bits (log2 q in 900..930), plaintext modulus t = 256,
secret key uniform ternary (every coefficient uniform in {-1, 0, 1}; the parity tests use the
reference's sparse generator as well), error sigma = 3.2, relinearisation key with ceil(r/4) = 4
gadget digits.
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
    ap.add_argument("--no-trait-path", action="store_true", help="skip the trait-level ct-mult")
    ap.add_argument("--no-rns-lengths", action="store_true", help="skip the ct-mult at r = 12 and r = 20")
    ap.add_argument("--crt-elements", type=int, default=512,
                    help="elements of the batched CRT workload with --only crt_batch (512: the configuration's)")
    ap.add_argument("--only", choices=["crt_batch", "homcrt", "serving", "trait_path"],
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
class _Nvml:
    """Read-only NVML queries through ctypes (libnvidia-ml.so.1): the SM clock, its maximum and
    the clock-event (throttle) reasons of one GPU."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, ordinal):
        """`ordinal`: the CUDA device ordinal; its PCI bus id (from the CUDA driver, which applies
        CUDA_VISIBLE_DEVICES) selects the NVML device."""
        import ctypes

        cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        bus = ctypes.create_string_buffer(32)
        if cu.cuInit(0) != 0 or cu.cuDeviceGet(ctypes.byref(dev), ctypes.c_int(ordinal)) != 0 or \
                cu.cuDeviceGetPCIBusId(bus, ctypes.c_int(32), dev) != 0:
            raise OSError("no CUDA device")
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus, ctypes.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self._u = ctypes.c_uint()
        self._r = ctypes.c_ulonglong()
        self.ctypes = ctypes

    def sample(self):
        """(SM MHz, max SM MHz, reason bits)"""
        c = self.ctypes
        self.lib.nvmlDeviceGetClockInfo(self.h, c.c_int(1), c.byref(self._u))  # NVML_CLOCK_SM
        sm = self._u.value
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, c.c_int(1), c.byref(self._u))
        mx = self._u.value
        self.reasons_fn(self.h, c.byref(self._r))
        return sm, mx, self._r.value


class ClockSampler:
    """SM clocks and throttle reasons sampled during the timed region: NVML every millisecond from a
    host thread where the library loads (so that even a region of a few milliseconds holds
    samples), else nvidia-smi every 20 ms."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.nvml = None
        self.thread = None
        self.rows = []  # NVML: (perf_counter, sm, max, reason bits)
        self.running = False
        self.begin = self.end = None
        self.begin_pc = self.end_pc = None

    def start(self):
        import threading

        try:
            self.nvml = _Nvml(self.gpu)
            self.nvml.sample()
        except Exception:
            self.nvml = None
        if self.nvml:
            self.running = True

            def loop():
                while self.running:
                    try:
                        self.rows.append((time.perf_counter(),) + self.nvml.sample())
                    except Exception:
                        pass
                    time.sleep(0.001)

            self.thread = threading.Thread(target=loop, daemon=True)
            self.thread.start()
            time.sleep(0.02)
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.1)  # the sampler's first query precedes the timed region

    def mark(self, begin):
        """Host bounds of the timed region (the samples inside them are the ones reported)."""
        import datetime

        if begin:
            self.begin, self.begin_pc = datetime.datetime.now(), time.perf_counter()
        else:
            self.end, self.end_pc = datetime.datetime.now(), time.perf_counter()

    def _summary(self, use, inside, reasons, source):
        sm = [r[0] for r in use]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": use[-1][1] if use else None,
                "samples": len(use), "samples_in_timed_region": len(inside), "reasons": sorted(reasons),
                "source": source}

    def stop(self):
        import datetime

        if self.nvml:
            time.sleep(0.005)
            self.running = False
            self.thread.join(timeout=1)
            rows = [(r[1], r[2], r[3]) for r in self.rows]
            inside = [(r[1], r[2], r[3]) for r in self.rows
                      if self.begin_pc is not None and self.begin_pc <= r[0] <= self.end_pc]
            use = inside or rows
            reasons = {name for r in use for bit, name in _Nvml.REASONS.items() if r[2] & bit}
            return self._summary(use, inside, reasons, "NVML, 1 ms")
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
        return self._summary([(r[1], r[2]) for r in use], inside, reasons, "nvidia-smi, 20 ms")


# ------------------------------------------------------------------------------ workload
class Workload:
    def __init__(self, be, batch, seed=2026, log2_q=LOG2_Q):
        import halcuda
        import ringcuda

        self.be = be
        self.ring = ringcuda.RingContext(FIELD, log2_q[0], log2_q[1], T_BITS, backend=be)
        R = self.ring
        self.base = R.initial_base()
        self.r = len(self.base)
        self.digits = ringcuda.select_digits(math.ceil(self.r / 4), self.r)
        la = R.log2_alpha_for_sigma(self.base, 3.2)
        st = [seed]
        self.sk = R.gen_sk_uniform_ternary(st)  # the configuration's key: coefficients uniform in {-1, 0, 1}
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
    field and length share one tensor; the batch runs them in one persistent launch per field (each
    field's slabs with their own kernel build and tuned shape), and a second batch over the same
    items runs all of them in one persistent launch with one shape."""

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
        ops = ringcuda.CRT_FORWARD | ringcuda.CRT_MUL | ringcuda.CRT_INVERSE
        self.batch = ringcuda.CrtBatch(self.items, ops, backend=be)
        self.launch = self.batch.tune(reps=2)
        self.batch.run()
        # the same items as one persistent launch over both fields, one launch shape
        self.batch1 = ringcuda.CrtBatch(self.items, ops | ringcuda.CRT_ONE_LAUNCH, backend=be)
        self.launch1 = self.batch1.tune(reps=2)
        self.batch1.run()
        be.synchronize()
        import halcuda

        self.graph = halcuda.Graph(be, self.batch.run)
        self.graph1 = halcuda.Graph(be, self.batch1.run)

    def plain_element(self, R, x, op, base, mods, i):
        """One element with the HAL/ring calls of the reference, one launch per pass."""
        xi, oi = x.rows(i, i + 1), op.rows(i, i + 1)
        R.pb_to_crt(xi, base)
        self.be.hal_mul_mont64(xi, oi, mods)
        R.crt_to_pb(xi, base)


def crt_batch_bench(be, steps, warmup, bpeak=None, peaks=None, elements=512):
    """CRT transforms/s (2 per element: forward and inverse) batched (graph replay of the persistent
    launch) and plain (one element at a time); inputs ~2.5 GB, larger than L2. After the timing a
    seeded sample of elements is run once more through the batch and compared with the plain form
    (per-element ring and HAL calls, each bit-exact against the oracle in the tests)."""
    import numpy as np

    import halcuda

    w = CrtWorkload(be, elements)
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
    # the one-launch form of the same batch
    for _ in range(warmup):
        w.graph1.launch()
    be.synchronize()
    ev0.record(be)
    for _ in range(steps):
        w.graph1.launch()
    ev1.record(be)
    ms1 = ev0.elapsed_ms(ev1) / steps
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
    # sample check: 8 seeded (item, element) pairs, the batch's result vs the plain form on a copy
    rng = np.random.default_rng(17)
    picks = [(int(k), int(rng.integers(0, w.items[int(k)][1].shape[0])))
             for k in rng.integers(0, len(w.items), size=8)]
    for graph, form in ((w.graph, "per-class"), (w.graph1, "one-launch")):
        before = [w.items[k][1].rows(i, i + 1).to_numpy() for k, i in picks]
        graph.launch()
        be.synchronize()
        for (k, i), x0 in zip(picks, before):
            R, x, op, base = w.items[k]
            y = be.tensor(x0)
            R.pb_to_crt(y, base)
            be.hal_mul_mont64(y, op.rows(i, i + 1), R.mods_for(base))
            R.crt_to_pb(y, base)
            if not np.array_equal(y.to_numpy(), x.rows(i, i + 1).to_numpy()):
                raise RuntimeError("crt_batch (%s): element %d of item %d differs from the plain form" % (form, i, k))
    # roofline: exact 64-bit products (two transforms and the operand product per residue) and
    # algorithmic bytes (read x and the operand, write x: 24 B per residue)
    products = sum(x.shape[0] * len(base) * R.n * (2 * TRANSFORM_PRODUCTS["field_%d" % R.n] + 1)
                   for R, x, op, base in w.items)
    roof = None
    if bpeak:
        hbm = (peaks or {}).get("hbm_gbs")
        ach = products / (ms * 1e-3)
        roof = {"int_roofline": {"achieved": round(ach / 1e9, 1), "peak": round(bpeak / 1e9, 1), "unit": "G products/s",
                                 "frac": round(ach / bpeak, 4),
                                 "plain_frac": round(products / (plain_ms * 1e-3) / bpeak, 4),
                                 "products_per_batch": products},
                "hbm": {"achieved": round(24 * w.residues / (ms * 1e-3) / 1e9, 1), "peak": hbm, "unit": "GB/s",
                        "frac": round(24 * w.residues / (ms * 1e-3) / 1e9 / hbm, 4) if hbm else None}}
    return {"workload": "%d elements, field uniform in {field_36864, field_49152}, RNS length uniform in 4..24; "
                        "each pb->crt, mul_mont64 by an operand, crt->pb" % n,
            "elements": n, "slabs": w.batch.num_slabs, "residues": w.residues, "roofline": roof,
            "checked": "8 seeded elements re-run after the timing, in both forms: equal to the plain form",
            "crt_transforms_per_s": round(2 * n / (ms * 1e-3), 1),
            "plain_crt_transforms_per_s": round(2 * n / (plain_ms * 1e-3), 1),
            "ms_per_batch": round(ms, 4), "plain_ms_per_batch": round(plain_ms, 4),
            "launches_per_batch": launches, "plain_launches_per_batch": 9 * n,
            "launch_shape": {"threads": w.launch[0], "ctas_per_sm": w.launch[1], "dim2_columns": 1 << w.launch[2],
                             "of": "the shape class with the most residues; each class has its own"},
            "one_launch": {"crt_transforms_per_s": round(2 * n / (ms1 * 1e-3), 1), "ms_per_batch": round(ms1, 4),
                           "launches_per_batch": 1,
                           "int_roofline_frac": round(products / (ms1 * 1e-3) / bpeak, 4) if bpeak else None,
                           "launch_shape": {"threads": w.launch1[0], "ctas_per_sm": w.launch1[1],
                                            "dim2_columns": 1 << w.launch1[2]},
                           "note": "every slab of both fields in one persistent launch with one shape "
                                   "(HC_CRT_ONE_LAUNCH); the main figure runs one launch per field"},
            "autotuned": True, "l2": "inputs 2 x %.1f GB, larger than L2" % (w.residues * 8 / 1e9)}


def homcrt_bench(be, reps=5):
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
    for label, budget in (("resident", len(gs)), ("streamed", 8)):
        ks = ringcuda.Keyset(R, digits, r, budget * key_bytes)
        for gg in gs:
            ks.add(gg, keys[gg])
        ringcuda.dbfv_hom_cyclic_transform(R, log2_b, log2_t, g, coeffs, ct, base, ks)  # warm-up (tables)
        be.synchronize()
        s0 = ks.stats()
        # back-to-back transforms with an event between each two; the median of the per-transform
        # times is reported, so that one step delayed by the shared host does not set the figure
        evs = [halcuda.Event() for _ in range(reps + 1)]
        evs[0].record(be)
        for q in range(reps):
            ringcuda.dbfv_hom_cyclic_transform(R, log2_b, log2_t, g, coeffs, ct, base, ks)
            evs[q + 1].record(be)
        times = [evs[q].elapsed_ms(evs[q + 1]) for q in range(reps)]
        s1 = ks.stats()
        out[label] = {"ms_per_transform": round(statistics.median(times), 3),
                      "ms_min_max": [round(min(times), 3), round(max(times), 3)], "transforms": reps,
                      "resident_keys": s1["resident"], "streamed_keys": s1["streamed"],
                      "streamed_GB_per_transform": round((s1["streamed_bytes"] - s0["streamed_bytes"]) / reps / 1e9, 3)}
        ks.close()
    out["key_switches_per_transform"] = 3 * (baby - 1) + 3 * (giant - 1)
    # every baby-step key is read once per step for all three digits (one key-switch launch), the
    # giant-step key once per giant rotation (one launch for all output digits)
    kb = (baby - 1 + giant - 1) * key_bytes
    out["key_GB_read_per_transform"] = round(kb / 1e9, 3)
    out["key_read_GBps_resident"] = round(kb / (out["resident"]["ms_per_transform"] * 1e-3) / 1e9, 1)
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
        f.close()
    # over-budget keys: rotations by four automorphisms per field (g, g^2, g^3, g^4) with an HBM
    # key budget of two keys per field, so that half of the Galois keys are streamed in from
    # pinned host memory by the rotations that need them
    gens = {"field_36864": (3283177, 8536255), "field_49152": (20965738, 35297665)}
    fields = {}
    for seed, (name, (g, m)) in enumerate(sorted(gens.items()), start=11):
        fields[name] = serving.FieldState(be, name, (1100, 1140), 256, range(4, 21), 2,
                                          [pow(g, k, m) for k in range(1, 5)], seed=seed, resident_keys=2)
    serving.Engine(be, fields, 16 << 30).warm()
    s0 = {n_: f.keys.stats() for n_, f in fields.items()}
    reqs = serving.make_stream(n, rate, [0.5, 0.35, 0.15], sorted(fields), (4, 20), 2, seed=7, n_galois=4)
    res = serving.Engine(be, fields, 16 << 30).run(reqs, batched=True)
    s1 = {n_: f.keys.stats() for n_, f in fields.items()}
    res["keys"] = {n_: {"resident": s1[n_]["resident"], "streamed": s1[n_]["streamed"],
                        "key_MB": round(fields[n_].key_bytes / 1e6, 1),
                        "streamed_copies": s1[n_]["streamed_copies"] - s0[n_]["streamed_copies"],
                        "streamed_GB": round((s1[n_]["streamed_bytes"] - s0[n_]["streamed_bytes"]) / 1e9, 2)}
                   for n_ in fields}
    out["batched_streamed_keys"] = res
    for f in fields.values():
        f.close()
    return out


def ct_mult_int_work(work, ms_per_ct_mult, bpeak):
    """The exact integer work of one ct-mult: the CRT transforms' Barrett products (TRANSFORM_PRODUCTS
    per residue of every transformed (row, prime) slab: both operands' crt_to_pb, the lifted
    extension rows' pb_to_crt, the product's crt_to_pb over the lifted base, the relinearised
    (c0, c1) rows' pb_to_crt and the gadget digits' pb_to_crt) and the base conversions' terms
    (source x destination products plus the correction row: both lifts, rescale's two conversions,
    the gadget decomposition). `ntt_time_frac` is the time those products would take at the
    measured Barrett rate, as a fraction of the measured time per ct-mult."""
    R, r, d = work.ring, work.r, len(work.digits)
    e = len(R.extension_base(work.base))
    slabs = 2 * 2 * r + 2 * 2 * e + 3 * (r + e) + 2 * r + d * r
    products = slabs * R.n * TRANSFORM_PRODUCTS[FIELD]
    per_digit = -(-r // d)
    terms = (2 * 2 * (r * e + r) + 3 * (r * e + r) + 3 * (e * r + e) + d * (r * per_digit + per_digit)) * R.n
    return {"transformed_slabs": slabs, "barrett_products": products, "conversion_terms": terms,
            "ntt_time_frac": round(products / bpeak / (ms_per_ct_mult * 1e-3), 4),
            "note": "the transforms' products at the measured Barrett rate take this fraction of a batched ct-mult; "
                    "the conversions (29-bit limb products on the same pipe) and the key switch take most of the rest"}


def trait_path_bench(be, work, reps=20):
    """The reference crate's own bfv_hom_mul call sequence issued through the hal::Backend trait
    entry points only (trait_ring.py: what the unchanged crate runs above a hal::cuda backend), on
    the headline workload's first ciphertext pair: direct calls (one ctypes call per trait method,
    host-issued like the crate's) and a CUDA-graph replay of the same sequence. Its result is
    compared with the fused path's (hc_bfv_hom_mul), which the tests pin to the oracle."""
    import numpy as np

    import halcuda
    import trait_ring

    R = work.ring
    bfv = trait_ring.TraitBfv(trait_ring.TraitRing(R))
    c1, c2 = work.ct1.rows(0, 2), work.ct2.rows(0, 2)
    out = R.allocate(2, work.r)

    def call():
        bfv.hom_mul(T, c1, c2, work.base, work.rk, work.digits, out=out)

    call()  # builds the crate-side caches (imports of its constant tensors)
    be.synchronize()
    exp = R.hom_mul(T, c1, c2, work.base, work.rk, work.digits).to_numpy()
    if not np.array_equal(out.to_numpy(), exp):
        raise RuntimeError("trait path: result differs from hc_bfv_hom_mul")
    ev0, ev1 = halcuda.Event(), halcuda.Event()
    l0 = be.launch_count()
    call()
    launches = be.launch_count() - l0
    be.synchronize()
    t0 = time.perf_counter()
    ev0.record(be)
    for _ in range(reps):
        call()
    ev1.record(be)
    direct_ms = ev0.elapsed_ms(ev1) / reps
    host_ms = 1e3 * (time.perf_counter() - t0) / reps
    graph = halcuda.Graph(be, call)
    graph.launch()
    be.synchronize()
    ev0.record(be)
    for _ in range(reps):
        graph.launch()
    ev1.record(be)
    graph_ms = ev0.elapsed_ms(ev1) / reps
    be.synchronize()
    if not np.array_equal(out.to_numpy(), exp):
        raise RuntimeError("trait path: graph replay differs from hc_bfv_hom_mul")
    return {"workload": "bfv_hom_mul %s r=%d t=%d d=%d through the trait entry points only, in the crate's call "
                        "order (src/bfv.rs:747-775, src/ring.rs)" % (FIELD, work.r, T, len(work.digits)),
            "launches_per_ct_mult": launches, "checked": "equal to hc_bfv_hom_mul (bit-exact)",
            "direct": {"ct_mults_per_s": round(1e3 / direct_ms, 1), "ms_per_ct_mult": round(direct_ms, 4),
                       "host_ms_per_ct_mult": round(host_ms, 4)},
            "graph": {"ct_mults_per_s": round(1e3 / graph_ms, 1), "ms_per_ct_mult": round(graph_ms, 4)}}


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


def rns_length_bench(be, streams, scratch, steps=100):
    """The ct-mult at the other ends of the configuration's RNS range, r = 12 and r = 20 (log2 q in
    660..690 and 1120..1150): one per launch (graph replays on the streams, as the headline) and
    8 per call; the same seeded workload construction as r = 16."""
    out = {}
    for lo, hi in ((660, 690), (1120, 1150)):
        w = Workload(be, 8, log2_q=(lo, hi))
        for g in w.single:
            g.launch()
        single_steps(be, w, 8, streams)
        be.synchronize()
        ms = single_steps(be, w, steps, streams)
        timed_steps(be, w, 2, scratch)
        nb = 20
        bms = timed_steps(be, w, nb, scratch)
        be.synchronize()
        out["r%d" % w.r] = {"log2_q": [lo, hi], "rns_len": w.r, "gadget_digits": len(w.digits),
                            "ct_mults_per_s": round(steps / (ms * 1e-3), 1),
                            "batched_ct_mults_per_s": round(w.batch * nb / (bms * 1e-3), 1)}
        w.single, w.graph = [], None
        w.ring.close()
    return out


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
# from one ncu capture of `python bench.py --roofline-only` (None: not captured for the current kernels).
NCU_TRAFFIC_BYTES = 240779264 + 183514624
NCU_IMAD_PIPE_FRAC = 0.782
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


# (field, log2 q range, t bits, rows of the timed tensor): lifted bases of 34 and 48 factors; 241 MB
# and 151 MB tensors, larger than L2
TRANSFORM_CASES = (("field_36864", (900, 930), 8, 24), ("field_49152", (1280, 1310), 2, 8))


def transform_roofline(be, R, field, rows, reps, bpeak, peaks):
    """CRT transforms as the ring runs them: pb_to_crt of a [rows, r + e, deg_L', deg_K] tensor of
    lifted residues (larger than L2), timed with CUDA events on the library's stream, beside the
    same transform as the reference's four HAL calls (one launch per dimension and direction).
    field_49152 runs as two fused cluster launches (csrc/crt_fused.cu), field_36864 as the four
    column / line launches. Algorithmic bytes: one read and one write of every residue per
    launch; algorithmic products: TRANSFORM_PRODUCTS per residue."""
    import numpy as np

    import halcuda

    base = R.initial_base()
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
    ker = [R.crt_kernels(i) for i in lifted]
    kl = be.tensor(np.stack([k[0] for k in ker]).reshape(1, len(lifted), R.dl, 1))
    kk = be.tensor(np.stack([k[1] for k in ker]).reshape(1, len(lifted), 1, R.dk))
    shape2, shape3 = ([4, 3], [2, 3, 8, 64]) if field == "field_36864" else ([4], [3, 64, 64])
    p2 = [be.hal_create_ntt_plan(R.modulus(i), shape2) for i in lifted]
    p3 = [be.hal_create_ntt_plan(R.modulus(i), shape3) for i in lifted]
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
    products = TRANSFORM_PRODUCTS[field] * residues
    peak = peaks.get("hbm_gbs")
    achieved = bytes_alg / (ms * 1e-3) / 1e9
    return {"workload": "pb_to_crt of [%d, %d, %d, %d] (%d MB)" % (rows, len(lifted), R.dl, R.dk, residues * 8 >> 20),
            "launches_per_transform": launches, "ms_per_transform": round(ms, 5),
            "four_hal_calls_ms_per_transform": round(ms4, 5),
            "hbm": {"achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4) if peak else None, "bytes_per_transform": bytes_alg},
            "int_roofline": {"achieved": round(products / (ms * 1e-3) / 1e9, 1), "peak": round(bpeak / 1e9, 1),
                             "unit": "G products/s", "frac": round(products / (ms * 1e-3) / bpeak, 4),
                             "products_per_transform": products,
                             "four_hal_calls_frac": round(products / (ms4 * 1e-3) / bpeak, 4)}}


def transform_rooflines(be, reps, peaks):
    import halcuda
    import ringcuda

    bpeak = halcuda.barrett_peak(be)
    out = {}
    for field, (lo, hi), tb, rows in TRANSFORM_CASES:
        R = ringcuda.RingContext(field, lo, hi, tb, backend=be)
        out[field] = transform_roofline(be, R, field, rows, reps, bpeak, peaks)
        R.close()
    return out


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


# ------------------------------------------------------------------------------ CPU baselines
# The oracle (single-threaded C++ restatement of the reference's hal::cpu path, test
# infrastructure) timed on bounded samples of configurations 3, 4 and 5 after the GPU
# measurements: one host core each (spawned processes, one per sample), then every host core at
# once.

def cpu_crt_batch_sample():
    """Configuration 3 on one core: six elements of the batch's mix (both fields, RNS lengths 4, 14
    and 24), each pb->crt, Montgomery product with an operand, crt->pb, for about 8 s."""
    import numpy as np

    from oracle import pyoracle as po

    g = np.random.default_rng(3)
    rings = {f: po.Ring(f, lo, hi, tb) for f, lo, hi, tb in CrtWorkload.FIELDS}
    work = []
    for f, o in rings.items():
        for r in (4, 14, 24):
            x = g.integers(-(1 << 56), 1 << 56, size=o.shape(1, r), dtype=np.int64)
            op = g.integers(-(1 << 56), 1 << 56, size=o.shape(1, r), dtype=np.int64)
            work.append((o, list(range(r)), x, op))

    def run(o, base, x, op):
        y = np.ascontiguousarray(o.pb_to_crt(x, base)).copy()
        po.mul_mont64(y, op, [o.primes[i] for i in base])
        return o.crt_to_pb(y, base)

    for item in work:  # first use builds each prime's CRT kernels: outside the timing
        run(*item)
    done, t0 = 0, time.perf_counter()
    while True:
        for item in work:
            run(*item)
        done += len(work)
        el = time.perf_counter() - t0
        if el > 8.0:
            break
    return {"value": round(2 * done / el, 2), "unit": "CRT transforms/s", "cores": 1, "kind": "port",
            "sample": "%d elements cycling over field_36864 and field_49152 at RNS lengths 4, 14, 24, pb->crt, "
                      "product, crt->pb, %.1f s on one core" % (done, el)}


def cpu_homcrt_sample():
    """Configuration 4 on one core: one full homomorphic CRT step at field_49152 r = 23, len 64,
    with the benchmark's keys and seeds (key generation untimed)."""
    import numpy as np

    from oracle import pyoracle as po

    o = po.Ring("field_49152", 1280, 1310, 2)
    base = o.initial_base()
    r = len(base)
    digits = po.select_digits(math.ceil(r / 4), r)
    la = o.log2_alpha_for_sigma(base, 3.2)
    st = [99]
    sk = o.gen_sk(st)
    m, gen, length = o.info["m"], 20965738, 64
    baby = min(range(1, length + 1), key=lambda c: (c + 3 * ((length - 1) // c + 1), c))
    gs = sorted(set([pow(gen, j, m) for j in range(1, baby)] + [pow(gen, baby, m)]))
    keys = {gg: o.gen_gk(st, sk, gg, digits, la) for gg in gs}
    t = 1 << 24
    rng = np.random.default_rng(5)
    ct = np.zeros(o.shape(6, r), dtype=np.int64)
    ct[0:2] = o.enc(st, base, t, [int(v) for v in rng.integers(0, t, size=o.n)], sk, la)
    for dd in (1, 2):
        ct[2 * dd:2 * dd + 2] = o.enc(st, base, t, [0] * o.n, sk, la)
    coeffs = [[int(v) for v in rng.integers(-t // 2, t // 2, size=o.dl)] for _ in range(length)]
    t0 = time.perf_counter()
    o.dbfv_hom_cyclic_transform(8, 24, gen, coeffs, ct, base, keys, digits)
    el = time.perf_counter() - t0
    return {"value": round(1e3 * el, 1), "unit": "ms per transform step", "higher_is_better": False, "cores": 1,
            "kind": "port", "sample": "one full step (13 baby x 5 giant steps, 48 key switches) on one core"}


def cpu_serving_sample(n=24):
    """Configuration 5 on one core: the first n requests of the benchmark's stream served one after
    another by the oracle (multiplications, rotations, transforms at their fields and levels)."""
    import numpy as np

    import serving
    from oracle import pyoracle as po

    g = np.random.default_rng(11)
    fields = {}
    for name, gal in (("field_36864", 3283177), ("field_49152", 20965738)):
        o = po.Ring(name, 1100, 1140, 8)
        full = o.initial_base()
        digits = po.select_digits(math.ceil(len(full) / 4), len(full))
        la = o.log2_alpha_for_sigma(full, 3.2)
        st = [5]
        sk = o.gen_sk(st)
        fields[name] = (o, digits, o.gen_rk(st, sk, digits, la), o.gen_gk(st, sk, gal, digits, la)[None], gal)
    reqs = serving.make_stream(n, 2000.0, [0.5, 0.35, 0.15], sorted(fields), (4, 20), 2, seed=7)

    def residues(o, rows, lv):
        x = np.empty(o.shape(rows, lv), dtype=np.int64)
        for j in range(lv):
            x[:, j] = g.integers(0, o.primes[j], size=x[:, j].shape)
        return x

    inputs = [(q, residues(fields[q.field][0], 2, q.level), residues(fields[q.field][0], 2, q.level)) for q in reqs]
    for name, (o, *_rest) in fields.items():  # CRT kernels of every prime: outside the timing
        o.pb_to_crt(residues(o, 1, 20), list(range(20)))
    lat = []
    t0 = time.perf_counter()
    for q, a, b in inputs:
        o, digits, rk, gk, gal = fields[q.field]
        base = list(range(q.level))
        s0 = time.perf_counter()
        if q.op == "mul":
            o.hom_mul(256, a, b, base, rk, digits)
        elif q.op == "rot":
            o.hom_gal(a, base, [gal], gk, digits)
        else:
            o.pb_to_crt(a[0:1], base)
        lat.append(1e3 * (time.perf_counter() - s0))
    el = time.perf_counter() - t0
    lat.sort()
    return {"value": round(n / el, 2), "unit": "req/s", "cores": 1, "kind": "port",
            "p50_ms": round(lat[len(lat) // 2], 1), "p99_ms": round(lat[-1], 1),
            "sample": "the first %d requests of the stream, served one after another on one core (%.1f s)" % (n, el)}


CPU_SAMPLES = {"headline": cpu_baseline, "crt_batch": cpu_crt_batch_sample, "homcrt": cpu_homcrt_sample,
               "serving": cpu_serving_sample}


def cpu_model():
    """The host CPU's model name (lscpu), or the machine type."""
    import platform

    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.machine()


def _sample_task(name):
    return CPU_SAMPLES[name]()


def cpu_all_cores(name):
    """The one-core sample `name` run at the same time in one spawned process per host core; the
    throughputs add up (a homcrt step's time becomes steps per second)."""
    import multiprocessing as mp

    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_sample_task, [name] * cores)
    el = time.perf_counter() - t0
    if name == "homcrt":
        value, unit = sum(1e3 / r["value"] for r in res), "transform steps/s"
    else:
        value, unit = sum(r["value"] for r in res), res[0]["unit"]
    return {"value": round(value, 3), "unit": unit, "cores": cores, "kind": "port", "cpu": cpu_model(),
            "sample": "the one-core sample in %d concurrent processes (%.0f s wall)" % (cores, el)}


def start_cpu_baselines(names):
    """Starts the one-core oracle samples in a spawned process pool (one process per sample);
    returns (pool, {name: async result})."""
    import multiprocessing as mp

    from oracle import build as oracle_build

    oracle_build.build()
    pool = mp.get_context("spawn").Pool(len(names))
    return pool, {n: pool.apply_async(_sample_task, (n,)) for n in names}


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
                                   % (FIELD, cores), "field": FIELD, "rns_len": 16,
                       "secret_key": "the reference's sparse ternary generator (a ct-mult's work does not depend "
                                     "on the key)"},
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
        fn = {"crt_batch": lambda: crt_batch_bench(be, max(3, args.steps // 2), args.warmup,
                                                   halcuda.barrett_peak(be), load_peaks(), args.crt_elements),
              "homcrt": lambda: homcrt_bench(be, reps=max(1, args.steps // 3)),
              "serving": lambda: serving_bench(be),
              "trait_path": lambda: trait_path_bench(be, Workload(be, 1))}[args.only]
        print(json.dumps({args.only: fn()}), flush=True)
        return
    if args.transform_only:
        print(json.dumps(transform_rooflines(be, max(1, args.steps), load_peaks())), flush=True)
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
    batched["int_work"] = ct_mult_int_work(work, batched_ms / nb / work.batch, halcuda.barrett_peak(be))

    # plain form (one ct-mult per timed call) and its latency distribution
    per = plain_calls(be, work, min(20, max(2, args.steps // 2)), scratch)
    per.sort()
    plain = 1e3 / statistics.mean(per)
    p50, p99 = per[len(per) // 2], per[min(len(per) - 1, int(math.ceil(0.99 * len(per))) - 1)]

    e2e_n = max(args.steps, 40)  # at least 40 steps, so that the pipeline's fill and drain stay small
    e2e_ms, h2d, d2h, _ = e2e_steps(be, work, e2e_n, args.e2e_slots)
    e2e_val = dist.world * e2e_n / (e2e_ms * 1e-3)
    roof = kernel_roofline(be, work.ring, work.base, 20, peaks)
    trait = None if args.no_trait_path else trait_path_bench(be, work)
    rns = None if args.no_rns_lengths else rns_length_bench(be, streams, scratch)
    bpeak = halcuda.barrett_peak(be)
    int8 = halcuda.int8_mma_peak(be)
    transforms = transform_rooflines(be, 10, peaks)
    crt = None if args.no_crt_batch else crt_batch_bench(be, min(20, max(3, args.steps // 2)), args.warmup, bpeak,
                                                          peaks)
    hcrt = None if args.no_homcrt else homcrt_bench(be)
    srv = None if args.no_serving else serving_bench(be)

    if dist.rank != 0:
        return
    # the oracle's samples run after the GPU work (spawned processes), so that their host memory
    # traffic does not slow the GPU's copies from pinned host memory (the streamed keys)
    cpu, cpu_more = None, {}
    if not args.no_cpu_baseline:
        names = ["headline"] + [n for n, r_ in (("crt_batch", crt), ("homcrt", hcrt), ("serving", srv)) if r_]
        pool, jobs = start_cpu_baselines(names)
        for name, job in jobs.items():
            res = job.get(timeout=900)
            if name == "headline":
                cpu = dict(res, cpu=cpu_model())
            else:
                cpu_more[name] = dict(res, cpu=cpu_model())
        pool.close()
        pool.join()
    for name, res in (("crt_batch", crt), ("homcrt", hcrt), ("serving", srv)):
        if res and name in cpu_more:
            res["cpu_baseline"] = cpu_more[name]
            res["cpu_baseline_all_cores"] = cpu_all_cores(name)  # after the GPU work: no contention
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
                   "secret_key": "uniform ternary", "error_sigma": 3.2,
                   "l2": "steps cycle over %d ciphertext pairs (%d MB of operands and results, larger than L2); "
                         "no flush" % (work.batch, 3 * work.ct_bytes * work.batch // 2**20)},
        "batched": batched,
        "plain_ct_mults_per_s": round(plain, 3),
        "latency_ms": {"p50": round(p50, 4), "p99": round(p99, 4), "samples": len(per)},
        "e2e": {"value": round(e2e_val, 3), "unit": "ct-mults/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": roof,
        "transform_rooflines": transforms,
        "peaks_measured_here": {"barrett_products_per_s": round(bpeak, -6), "int8_mma_macs_per_s": round(int8, -9)},
        "clocks": clk,
    }
    if trait:
        line["trait_path"] = trait
    if rns:
        line["rns_lengths"] = rns
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
