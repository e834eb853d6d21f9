"""Serving of homomorphic requests on one GPU with continuous batching.

Requests are ciphertext multiplications (bfv_hom_mul, src/bfv.rs:747-775), automorphisms
(bfv_hom_gal with one Galois element, src/bfv.rs:783-841) and standalone period -> CRT transforms
(pb_to_crt, src/ring.rs:1118-1138) over several field descriptors and RNS levels (a level is the
length r of the prefix of the field's initial RNS base). Relinearisation keys stay resident in
HBM; each field's Galois keys live in a keyset that keeps them in HBM up to a byte budget and
streams the others from pinned host memory with asynchronous copies right before their key
switch (the GPU counterpart of the reference's on-disk key store, src/keystore.rs:87-119).

Failures are handled on the host and never stop the stream: a request larger than the engine's
per-request limit is refused at admission, a request whose batch the library rejects (for example
a rotation by an automorphism without a key) completes with its error, and a request cancelled
before admission is dropped; each such request carries its status in `error`.

The engine runs one host loop:
  * arrivals are admitted while the HBM bytes of the admitted, unfinished requests stay within the
    budget; the rest wait in arrival order;
  * admitted requests are grouped by (operation, field, level, Galois element) and each group is
    submitted as batched calls (the B ciphertext pairs of a group go through one hom_mul call, the
    B ciphertexts of a rotation group through one hom_gal call, the B elements of a transform
    group through one transform call); the loop never waits for the device: at most `max_rounds`
    submission rounds are queued on it at a time, and requests that arrive meanwhile gather on
    the host, to be admitted and submitted together as soon as a round finishes - the device
    queue stays full while batches grow with the load;
  * the batches of a round go round-robin to `streams` CUDA streams, so that independent batches
    (small levels fill only part of the GPU) run concurrently;
  * completion is detected by polling one event per batch; the latency of a request is the time
    from its arrival to the completion of its batch.
The plain form submits every request alone, in arrival order, on one stream, through the same
loop.
"""
import collections
import math
import time
from dataclasses import dataclass, field as dc_field

import numpy as np

import halcuda
import ringcuda

OPS = ("mul", "rot", "crt")


@dataclass
class Request:
    rid: int
    op: str
    field: str
    level: int
    arrival: float  # seconds after the start of the stream
    slot: int  # input index in the pool of its (field, level)
    gi: int = 0  # rotations: index of the Galois element in the field's list
    g: int = 0  # rotations: an explicit Galois element instead of the list's (0: use gi)
    t_done: float = -1.0
    out: object = dc_field(default=None, repr=False)
    error: str = ""  # why the request did not run ("" when it did)
    cancelled: bool = False


class FieldState:
    """A field descriptor's ring with a device-resident relinearisation key, Galois keys of the
    elements `galois` (one element or a list) in a keyset whose HBM budget holds `resident_keys`
    of them (None: all; the others are streamed from pinned host memory), and a pool of encrypted
    inputs per level."""

    def __init__(self, be, name, log2_q, t, levels, pool_size, galois, seed, resident_keys=None):
        self.name, self.t = name, t
        self.gs = list(galois) if isinstance(galois, (list, tuple)) else [galois]
        self.g = self.gs[0]
        self.ring = ringcuda.RingContext(name, log2_q[0], log2_q[1], int(math.log2(t)), backend=be)
        R = self.ring
        if R.initial_len < max(levels):
            raise ValueError("%s: the initial RNS base has %d factors, levels up to %d requested"
                             % (name, R.initial_len, max(levels)))
        full = R.initial_base()
        self.digits = ringcuda.select_digits(math.ceil(len(full) / 4), len(full))
        la = R.log2_alpha_for_sigma(full, 3.2)
        st = [seed]
        sk = R.gen_sk(st)
        self.rk = R.gen_rk(st, sk, self.digits, la)
        gks = [R.gen_gk(st, sk, g, self.digits, la) for g in self.gs]
        self.gk = gks[0]
        self.key_bytes = 2 * len(self.digits) * len(full) * R.n * 8
        nres = len(self.gs) if resident_keys is None else resident_keys
        self.keys = ringcuda.Keyset(R, self.digits, len(full), nres * self.key_bytes)
        for g, k in zip(self.gs, gks):
            self.keys.add(g, k)
        del gks  # the keyset holds its own copies (in HBM or pinned host memory)
        self.sk = sk
        rng = np.random.default_rng(seed)
        self.pool = {}
        for lv in levels:
            base = list(range(lv))
            la_l = R.log2_alpha_for_sigma(base, 3.2)
            items = []
            for _ in range(pool_size):
                m1 = [int(v) for v in rng.integers(0, t, size=R.n)]
                m2 = [int(v) for v in rng.integers(0, t, size=R.n)]
                items.append((R.enc(st, base, t, m1, sk, la_l), R.enc(st, base, t, m2, sk, la_l)))
            self.pool[lv] = items
        self.mods = {lv: R.mods_for(list(range(lv))) for lv in levels}

    def close(self):
        """Releases the keyset, then the ring."""
        self.keys.close()
        self.ring.close()

    def bytes_of(self, op, level):
        """HBM bytes a request holds while in flight (outputs, staging and temporaries)."""
        slab = level * self.ring.n * 8
        ext = len(self.ring.extension_base(list(range(level))))
        if op == "mul":
            return 8 * slab + 3 * (level + ext) * self.ring.n * 8 * 2
        if op == "rot":
            return 6 * slab + 2 * len(self.digits) * slab
        return 2 * slab


def make_stream(n, rate, mix, fields, levels, pool_size, seed, n_galois=1):
    """A seeded Poisson request stream: exponential inter-arrival times of mean 1/rate, operations
    drawn with probabilities `mix`, field and level uniform, and for rotations one of `n_galois`
    Galois elements, uniform (drawn from a second generator, so that the rest of the stream does
    not depend on n_galois)."""
    g = np.random.default_rng(seed)
    gaps = g.exponential(1.0 / rate, size=n)
    ops = g.choice(len(OPS), size=n, p=mix)
    fs = g.integers(0, len(fields), size=n)
    lv = g.integers(levels[0], levels[1] + 1, size=n)
    sl = g.integers(0, pool_size, size=n)
    gi = np.random.default_rng(seed + 1).integers(0, n_galois, size=n)
    t = np.cumsum(gaps) - gaps[0]
    return [Request(i, OPS[int(ops[i])], fields[int(fs[i])], int(lv[i]), float(t[i]), int(sl[i]),
                    int(gi[i]) if OPS[int(ops[i])] == "rot" else 0) for i in range(n)]


class Engine:
    def __init__(self, be, fields, hbm_budget_bytes, max_batch=64, max_rounds=2, streams=4, max_request_bytes=None):
        self.be = be
        self.fields = fields
        self.budget = int(hbm_budget_bytes)
        self.max_request_bytes = max_request_bytes
        self.max_batch = max_batch
        self.max_rounds = max_rounds
        self.streams = [halcuda.Stream() for _ in range(max(0, streams))]
        self.next_stream = 0
        self.cancelled = set()

    def cancel(self, rid):
        """Cancels request `rid`: if it has not been admitted yet it is dropped (status
        "cancelled"); a request already submitted completes normally."""
        self.cancelled.add(rid)

    def submit_on_stream(self, reqs, use_streams):
        """submit() on the next extra stream (round robin) or on the context's own stream; the
        batch's temporaries are released on the stream they were used on."""
        if not use_streams or not self.streams:
            return self.submit(reqs)
        s = self.streams[self.next_stream % len(self.streams)]
        self.next_stream += 1
        with self.be.on(s):
            return self.submit(reqs)

    def warm(self):
        """Runs one request of every (operation, field, level) once, so that the rings' tables
        (transform kernels, base conversions, permutations) exist before serving starts."""
        for name, F in self.fields.items():
            for lv in F.pool:
                for op in OPS:
                    for gi in range(len(F.gs) if op == "rot" else 1):
                        self.submit([Request(-1, op, name, lv, 0.0, 0, gi)])
        self.be.synchronize()

    # ---- submission (asynchronous on the context's stream) ----
    def submit(self, reqs):
        """Submits one group of same-(op, field, level, Galois element) requests as batched calls;
        returns an event recorded behind them."""
        F = self.fields[reqs[0].field]
        R, lv, op = F.ring, reqs[0].level, reqs[0].op
        base = list(range(lv))
        B = len(reqs)
        be = self.be
        if op == "mul":
            if B == 1:
                c1, c2 = F.pool[lv][reqs[0].slot]
                reqs[0].out = R.hom_mul(F.t, c1, c2, base, F.rk, F.digits)
            else:
                a, b = R.allocate(2 * B, lv), R.allocate(2 * B, lv)
                for i, q in enumerate(reqs):
                    c1, c2 = F.pool[lv][q.slot]
                    be.hal_assign(a.rows(2 * i, 2 * i + 2), c1)
                    be.hal_assign(b.rows(2 * i, 2 * i + 2), c2)
                out = R.hom_mul(F.t, a, b, base, F.rk, F.digits)
                for i, q in enumerate(reqs):
                    q.out = out.rows(2 * i, 2 * i + 2)
        elif op == "rot":
            g = reqs[0].g or F.gs[reqs[0].gi]
            if B == 1:
                reqs[0].out = ringcuda.hom_gal_batch_keyset(R, F.pool[lv][reqs[0].slot][0], base, g, F.keys)
            else:
                a = R.allocate(2 * B, lv)
                for i, q in enumerate(reqs):
                    be.hal_assign(a.rows(2 * i, 2 * i + 2), F.pool[lv][q.slot][0])
                out = ringcuda.hom_gal_batch_keyset(R, a, base, g, F.keys)
                for i, q in enumerate(reqs):
                    q.out = out.rows(2 * i, 2 * i + 2)
        else:
            x = R.allocate(B, lv)
            for i, q in enumerate(reqs):
                be.hal_assign(x.rows(i, i + 1), F.pool[lv][q.slot][0].rows(0, 1))
            R.pb_to_crt(x, base)
            for i, q in enumerate(reqs):
                q.out = x.rows(i, i + 1)
        ev = halcuda.Event()
        ev.record(be)
        return ev

    def run(self, reqs, batched=True, keep_outputs=False, timeout_s=120.0):
        """Serves the stream (arrival times relative to now); returns the stats dictionary."""
        be = self.be
        pending = collections.deque()
        inflight = []  # (event, requests, bytes, round)
        used, done, i, rnd = 0, 0, 0, 0
        launches0 = be.launch_count()
        batches = 0
        t0 = time.perf_counter()

        def finish(q, error):
            q.error, q.t_done, q.out = error, time.perf_counter() - t0, None

        while done < len(reqs):
            now = time.perf_counter() - t0
            if now > timeout_s:
                raise RuntimeError("serving did not finish within %.0f s" % timeout_s)
            while i < len(reqs) and reqs[i].arrival <= now:
                q = reqs[i]
                i += 1
                nb = self.fields[q.field].bytes_of(q.op, q.level)
                if self.max_request_bytes is not None and nb > self.max_request_bytes:
                    finish(q, "refused: needs %d bytes of HBM, the limit per request is %d"
                           % (nb, self.max_request_bytes))
                    done += 1
                    continue
                pending.append(q)
            if self.cancelled and pending:
                keep = collections.deque()
                for q in pending:
                    if q.rid in self.cancelled:
                        q.cancelled = True
                        finish(q, "cancelled")
                        done += 1
                    else:
                        keep.append(q)
                pending = keep
            progressed = False
            if inflight:
                keep = []
                for ev, group, nb, rd in inflight:
                    if ev.query():
                        td = time.perf_counter() - t0
                        for q in group:
                            q.t_done = td
                            if not keep_outputs:
                                q.out = None
                        done += len(group)
                        used -= nb
                        progressed = True
                    else:
                        keep.append((ev, group, nb, rd))
                inflight = keep
            if pending and len(set(x[3] for x in inflight)) < self.max_rounds:
                admitted = []
                while pending:
                    q = pending[0]
                    nb = self.fields[q.field].bytes_of(q.op, q.level)
                    if used + nb > self.budget and (used > 0 or admitted):
                        break
                    pending.popleft()
                    used += nb
                    admitted.append((q, nb))
                if admitted:
                    progressed = True
                    if batched:
                        groups = collections.OrderedDict()
                        for q, nb in admitted:
                            groups.setdefault((q.op, q.field, q.level, q.gi, q.g), []).append((q, nb))
                        units = []
                        for g in groups.values():
                            for s in range(0, len(g), self.max_batch):
                                units.append(g[s:s + self.max_batch])
                    else:
                        units = [[x] for x in admitted]
                    for u in units:
                        group, nb = [q for q, _ in u], sum(b for _, b in u)
                        try:
                            ev = self.submit_on_stream(group, batched)
                        except halcuda.HalError as e:  # refused by the library: the batch did not run
                            for q in group:
                                finish(q, "failed: %s" % e)
                            done += len(group)
                            used -= nb
                            continue
                        inflight.append((ev, group, nb, rnd))
                        batches += 1
                    rnd += 1
            if not progressed:
                time.sleep(20e-6)
        served = [q for q in reqs if not q.error]
        lat = np.array([q.t_done - q.arrival for q in served] or [0.0]) * 1e3
        span = max(q.t_done for q in reqs) - min(q.arrival for q in reqs)
        out = {"requests": len(reqs), "throughput_req_per_s": round(len(served) / span, 1) if span > 0 else 0.0,
               "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
               "mean_ms": round(float(lat.mean()), 3), "batches": batches,
               "gpu_launches": be.launch_count() - launches0, "span_s": round(span, 3)}
        for kind in ("refused", "failed", "cancelled"):
            out[kind] = sum(q.error.startswith(kind) for q in reqs)
        return out
