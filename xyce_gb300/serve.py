"""Continuous batching of transient requests on one GPU (the serving path).

Requests (.STEP / Monte-Carlo variants of a circuit, of uneven sizes) arrive
over time.  Two servers:

  * SlotServer: one slotted batch (xg_batch_create_slots) per size class,
    each on its own stream replaying its own CUDA graph.  A request is
    submitted into a free slot of its class's batch while that batch runs and
    starts at its next iteration; a finished request's slot is released as
    soon as its results are read, so neither a short request nor a newly
    arrived one waits for a batch's longest request.  Batches are created as
    classes first appear, and another one for a class whose slots are all
    taken, when the device's free memory (cudaMemGetInfo) minus a reserve
    holds its slots (plan_slots).  A request larger than its class's slot
    shape runs in a batch of its own, admitted by its measured footprint.
  * Server: requests grouped into fixed batches (xg_batch_create) as they
    arrive; a batch's requests leave as they finish, but new ones wait for a
    new batch.

Latency = completion - arrival, reported as p50 / p99 beside throughput.
"""
import collections
import gc
import time

import numpy as np

from . import abi, engine, netlists


class Request:
    __slots__ = ("netlist", "x0", "tstop", "out_idx", "arrival", "start", "done", "result")

    def __init__(self, netlist, x0, tstop, out_idx):
        self.netlist, self.x0, self.tstop, self.out_idx = netlist, x0, tstop, out_idx
        self.arrival = self.start = self.done = None
        self.result = None


def ring_mc_requests(n, seed=0, stages=(5, 501), tstop=5e-9):
    """n seeded Monte-Carlo ring oscillators: odd stage counts uniform in
    [stages[0], stages[1]], VTO and KP of every stage scaled by (1 + d),
    d ~ N(0, 0.1/3) truncated at +-10%; started from an alternating initial
    condition; recorded at the first node and mid-ring."""
    rng = np.random.default_rng(seed)
    lo, hi = (stages[0] - 1) // 2, (stages[1] - 1) // 2
    out = []
    for k in range(n):
        st = 2 * int(rng.integers(lo, hi + 1)) + 1
        nl = netlists.ring_oscillator(st, seed=int(rng.integers(1 << 30)))
        x0 = np.zeros(nl.n_nodes + nl.count(abi.DEV_VSRC))
        x0[:nl.n_nodes] = netlists.ring_oscillator_nodeset(st)
        out.append(Request(nl, x0, tstop, [1, st // 2 + 1]))
    return out


def poisson_arrivals(n, rate, seed=0):
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n))


class Server:
    """Continuous batching.  Queued requests are grouped by size class
    (unknowns within a factor of 2), so one batch's per-iteration time, set by
    its largest request, is not imposed on much smaller ones; the oldest
    waiting request picks the class admitted next.  Batches are set up on a
    helper thread (the set-up call releases the interpreter lock) while the
    running ones keep stepping."""

    def __init__(self, ctx, precision=abi.LU_FP64, n_refine=0, max_batch=512, max_concurrent=8,
                 memory_budget=64 << 30, chunk=64, tstep=1e-12, max_points=8192):
        self.ctx = ctx
        self.precision, self.n_refine = precision, n_refine
        self.max_batch, self.max_concurrent = max_batch, max_concurrent
        self.memory_budget, self.chunk, self.tstep = memory_budget, chunk, tstep
        self.max_points = max_points
        self.bytes_per_unknown = None

    @staticmethod
    def size_class(r):
        return int(np.log2(max(2, len(r.x0))))

    def close(self):
        """Nothing held between runs (each batch lives for its requests)."""

    def _footprint(self, reqs):
        unk = sum(len(r.x0) for r in reqs)
        return 0 if self.bytes_per_unknown is None else unk * self.bytes_per_unknown

    def _create(self, reqs):
        b = engine.Batch(self.ctx, [r.netlist for r in reqs], [r.x0 for r in reqs],
                         [r.tstop for r in reqs], [r.out_idx for r in reqs], tstep=self.tstep,
                         precision=self.precision, n_refine=self.n_refine,
                         max_points=self.max_points)
        b.run(self.chunk)
        return b

    def _take(self, queue):
        """Up to max_batch queued requests of the oldest request's size class."""
        cls = self.size_class(queue[0])
        take, keep = [], collections.deque()
        while queue:
            r = queue.popleft()
            if len(take) < self.max_batch and self.size_class(r) == cls:
                take.append(r)
            else:
                keep.append(r)
        queue.extend(keep)
        return take

    def run(self, requests, arrivals):
        """Serve requests arriving at the given times (s); returns a summary.
        No cyclic garbage collection runs meanwhile: a full collection over
        the requests' netlists would stall the loop that keeps the GPU fed."""
        was = gc.isenabled()
        gc.disable()
        try:
            return self._run(requests, arrivals)
        finally:
            if was:
                gc.enable()

    def _run(self, requests, arrivals):
        n = len(requests)
        for r, a in zip(requests, arrivals):
            r.arrival = float(a)
        import concurrent.futures as cf
        queue = collections.deque()
        active = []
        pending = None                 # (future, requests, footprint) being set up
        nxt = done = 0
        in_use = 0
        pool = cf.ThreadPoolExecutor(1)
        t0 = time.perf_counter()
        while done < n:
            now = time.perf_counter() - t0
            while nxt < n and requests[nxt].arrival <= now:
                queue.append(requests[nxt])
                nxt += 1
            busy = False
            if pending is not None and pending[0].done():
                b = pending[0].result()
                nb = b.device_bytes()
                self.bytes_per_unknown = nb / max(1, sum(len(r.x0) for r in pending[1]))
                in_use += nb - pending[2]
                active.append([b, pending[1], [False] * len(pending[1]), nb, 0])
                pending = None
                busy = True
            if pending is None and queue and len(active) < self.max_concurrent:
                take = self._take(queue)
                fp = self._footprint(take)
                if in_use + fp <= self.memory_budget:
                    for r in take:
                        r.start = now
                    pending = (pool.submit(self._create, take), take, fp)
                    in_use += fp
                    busy = True
                else:
                    queue.extendleft(reversed(take))
            for entry in list(active):
                b, reqs, fin, nb, seen = entry
                nd = b.poll(wait=False)
                if nd < 0:
                    continue
                busy = True
                t_now = time.perf_counter() - t0
                if nd > seen:
                    # some requests finished since the last look: find them
                    entry[4] = nd
                    for j, r in enumerate(reqs):
                        if not fin[j]:
                            st = b.stats(j)
                            if st["finished"]:
                                fin[j] = True
                                r.done = t_now
                                r.result = b.results(j)
                                done += 1
                if all(fin):
                    b.close()
                    in_use -= nb
                    active.remove(entry)
                else:
                    b.run(self.chunk)
            if not busy:
                time.sleep(0.0002)
        pool.shutdown()
        wall = time.perf_counter() - t0
        lat = np.array([r.done - r.arrival for r in requests])
        iters = sum(r.result[2]["newton_iters"] for r in requests)
        failed = sum(1 for r in requests if r.result[2]["status"] != 0)
        return {"requests": n, "wall_s": wall, "solves_per_s": n / wall,
                "newton_iters_per_s": iters / wall,
                "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3), "failed": failed}


def size_class(n_unknowns):
    """Requests with unknowns in [2^k, 2^(k+1)) share class k."""
    return int(np.log2(max(2, int(n_unknowns))))


def plan_slots(want, per_slot_bytes, free_bytes, reserve_bytes, in_use_bytes=0, cap_bytes=None):
    """How many slots of per_slot_bytes a new batch may take: at most `want`,
    within the device's free memory less the reserve, and within cap_bytes
    (if given) less what the server already holds.  0: admit nothing now."""
    room = free_bytes - reserve_bytes
    if cap_bytes is not None:
        room = min(room, cap_bytes - in_use_bytes)
    if room <= 0 or per_slot_bytes <= 0:
        return 0
    return int(max(0, min(want, room // per_slot_bytes)))


def merge_shapes(shapes, margin=1.25):
    """The smallest shape that holds every given one, its pivot-dependent
    sizes (L\\U and schedule) widened by `margin` (another request of the
    class may pivot differently)."""
    out = abi.XgSlotShape()
    out.max_unknowns = max(s.max_unknowns for s in shapes)
    for t in range(abi.NUM_DEV_TYPES):
        out.max_instances[t] = max(s.max_instances[t] for s in shapes)
    out.max_nnz = max(s.max_nnz for s in shapes)
    out.max_lu_nnz = int(max(s.max_lu_nnz for s in shapes) * margin) + 16
    out.max_schedule = int(max(s.max_schedule for s in shapes) * margin) + 64
    out.max_breakpoints = max(s.max_breakpoints for s in shapes) + 2
    return out


def ring_class_shapes(ctx, stages=(5, 501), tstop=5e-9, tstep=1e-12, seeds=(0, 1)):
    """Slot shapes for the Monte-Carlo ring stream: for each size class the
    needs of its largest ring (a few seeds), merged."""
    lo, hi = stages
    by_class = {}
    for st in range(lo, hi + 1, 2):
        by_class.setdefault(size_class(st + 2), []).append(st)
    shapes = {}
    for cls, sts in by_class.items():
        top = max(sts)
        needs = []
        for sd in seeds:
            nl = netlists.ring_oscillator(top, seed=sd)
            x0 = np.zeros(nl.n_nodes + nl.count(abi.DEV_VSRC))
            x0[:nl.n_nodes] = netlists.ring_oscillator_nodeset(top)
            needs.append(engine.slot_need(ctx, nl, x0, tstop, tstep))
        shapes[cls] = merge_shapes(needs)
    return shapes


class SlotServer:
    """Continuous batching at slot granularity (see the module docstring).
    shapes: {size class: XgSlotShape}; slots: slots per batch; reserve_bytes:
    device memory left free; memory_cap: at most this much held by the
    server's batches (None: no cap besides the device).  The batches live
    with the server, across calls of run(), as a long-running server keeps
    them; close() frees them."""

    def __init__(self, ctx, shapes, precision=abi.LU_FP64, n_refine=0, slots=512, chunk=32, tstep=1e-12,
                 max_points=8192, n_out=2, reserve_bytes=4 << 30, memory_cap=None, max_batches_per_class=8,
                 depth=1):
        self.ctx, self.shapes = ctx, dict(shapes)
        self.precision, self.n_refine = precision, n_refine
        self.slots, self.chunk, self.tstep = slots, chunk, tstep
        self.max_points, self.n_out = max_points, n_out
        self.reserve, self.cap = reserve_bytes, memory_cap
        self.max_batches_per_class = max_batches_per_class
        # chunks in flight per batch (at most 3: four snapshots).  Two keep
        # the device busy while the host harvests, but under load they hold
        # finished requests' slots a chunk longer and queue activations behind
        # two chunks: 20% fewer solves/s at 2,000 req/s than one.
        self.depth = depth
        self.opts = engine.batch_options(tstep, precision, n_refine, n_out, max_points)
        self.in_use = 0
        # class -> [entry]; entry: {"b": SlotBatch, "held": {slot: request}, "fut": submit future}
        self.pools = collections.defaultdict(list)

    def close(self):
        for entries in self.pools.values():
            for e in entries:
                self.in_use -= e["b"].device_bytes()
                e["b"].close()
        self.pools.clear()

    def _new_batch(self, cls):
        sh = self.shapes[cls]
        per = engine.slot_bytes(sh, self.opts)
        free, _ = engine.mem_info(self.ctx)
        n = plan_slots(self.slots, per, free, self.reserve, self.in_use, self.cap)
        if n <= 0:
            return None
        b = engine.SlotBatch(self.ctx, n, sh, self.n_out, tstep=self.tstep, precision=self.precision,
                             n_refine=self.n_refine, max_points=self.max_points)
        self.in_use += b.device_bytes()
        return b

    def run(self, requests, arrivals):
        """Serve requests arriving at the given times (s); returns a summary
        (no cyclic garbage collection meanwhile, as Server.run)."""
        was = gc.isenabled()
        gc.disable()
        try:
            return self._run(requests, arrivals)
        finally:
            if was:
                gc.enable()

    def _run(self, requests, arrivals):
        import concurrent.futures as cf
        n = len(requests)
        for r, a in zip(requests, arrivals):
            r.arrival = float(a)
        queues = collections.defaultdict(collections.deque)
        pools = self.pools
        solo = []                                 # (Batch, request, bytes): larger than the shape
        pool_ex = cf.ThreadPoolExecutor(2)
        nxt = done = 0
        t0 = time.perf_counter()
        oversize = 0

        def submit(entry, reqs):
            b = entry["b"]
            slots = b.submit([r.netlist for r in reqs], [r.x0 for r in reqs], [r.tstop for r in reqs],
                             [r.out_idx for r in reqs])
            return list(zip(reqs, slots))

        while done < n:
            now = time.perf_counter() - t0
            while nxt < n and requests[nxt].arrival <= now:
                r = requests[nxt]
                queues[size_class(len(r.x0))].append(r)
                nxt += 1
            busy = False
            # finished submits: the taken requests are now held by their slots
            for cls, entries in pools.items():
                for e in entries:
                    f = e["fut"]
                    if f is not None and f.done():
                        e["fut"] = None
                        busy = True
                        try:
                            placed = f.result()
                        except engine.XgError:
                            placed = None
                        if placed is None:
                            # a request of that group does not fit the shape:
                            # its whole group goes to batches of their own
                            for r in e.pop("pending"):
                                solo.append(self._solo(r, now))
                                oversize += 1
                            continue
                        e.pop("pending")
                        for r, sl in placed:
                            if sl >= 0:
                                e["held"][sl] = r
                            else:
                                queues[cls].appendleft(r)
            # admission: queued requests into free slots of their class
            for cls, q in queues.items():
                if not q:
                    continue
                if cls not in self.shapes:
                    while q:
                        solo.append(self._solo(q.popleft(), now))
                        oversize += 1
                    continue
                entries = pools[cls]
                target = None
                for e in entries:
                    if e["fut"] is None and e["b"].n - len(e["held"]) > 0:
                        target = e
                        break
                if target is None and all(e["fut"] is None for e in entries) and \
                        len(entries) < self.max_batches_per_class:
                    b = self._new_batch(cls)
                    if b is not None:
                        target = {"b": b, "held": {}, "fut": None}
                        entries.append(target)
                if target is None:
                    continue
                k = min(len(q), target["b"].n - len(target["held"]))
                take = [q.popleft() for _ in range(k)]
                for r in take:
                    r.start = now
                target["pending"] = take
                target["fut"] = pool_ex.submit(submit, target, take)
                busy = True
            # step and harvest: `depth` chunks in flight per batch; a poll
            # reads the snapshot of the newest finished one
            for cls, entries in pools.items():
                for e in entries:
                    b = e["b"]
                    if b.poll(wait=False) >= 0:
                        t_now = time.perf_counter() - t0
                        for sl in b.finished():
                            r = e["held"].pop(sl, None)
                            if r is None:
                                continue
                            r.result = b.results(sl)
                            r.done = t_now
                            b.release(sl)
                            done += 1
                            busy = True
                    if e["held"] or e["fut"] is not None:
                        while b.inflight() < self.depth:
                            b.run(self.chunk)
                            busy = True
            for item in list(solo):
                b, r, nb = item
                nd = b.poll(wait=False)
                if nd < 0:
                    continue
                if b.stats(0)["finished"]:
                    r.result = b.results(0)
                    r.done = time.perf_counter() - t0
                    b.close()
                    self.in_use -= nb
                    solo.remove(item)
                    done += 1
                else:
                    b.run(self.chunk)
                busy = True
            if not busy:
                time.sleep(0.0002)
        pool_ex.shutdown()
        wall = time.perf_counter() - t0
        lat = np.array([r.done - r.arrival for r in requests])
        iters = sum(r.result[2]["newton_iters"] for r in requests)
        failed = sum(1 for r in requests if r.result[2]["status"] != 0)
        return {"requests": n, "wall_s": wall, "solves_per_s": n / wall,
                "newton_iters_per_s": iters / wall,
                "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3), "failed": failed, "oversize": oversize,
                "batches": {int(c): len(v) for c, v in pools.items()}}

    def _solo(self, r, now):
        """A request larger than its class's shape: a batch of its own,
        admitted by its measured footprint (waits while memory is short)."""
        need = engine.slot_need(self.ctx, r.netlist, r.x0, r.tstop, self.tstep)
        nb = engine.slot_bytes(need, self.opts)
        while True:
            free, _ = engine.mem_info(self.ctx)
            if plan_slots(1, nb, free, self.reserve, self.in_use, self.cap) >= 1:
                break
            time.sleep(0.001)
        r.start = now
        b = engine.Batch(self.ctx, [r.netlist], [r.x0], [r.tstop], [r.out_idx], tstep=self.tstep,
                         precision=self.precision, n_refine=self.n_refine, max_points=self.max_points)
        nb = b.device_bytes()
        self.in_use += nb
        b.run(self.chunk)
        return (b, r, nb)


class Autotuner:
    """Picks the server's batch schedule (requests per batch, batch iterations
    per launch chunk, batches in flight) by measuring it: one parameter at a
    time, each candidate serving the same probe stream, keeping the value
    with the most solves/s.  `serve` is called as serve(params, requests,
    arrivals) and returns Server.run's summary; the probe's requests are
    rebuilt for every trial by `make_requests`.  Results can be kept in a
    JSON file keyed by the device and the workload, so a server starts from
    the last tuned schedule."""

    GRID = {"max_batch": (128, 256, 512, 1024), "chunk": (16, 64, 256), "max_concurrent": (2, 4, 8)}
    START = {"max_batch": 512, "chunk": 64, "max_concurrent": 8}

    def __init__(self, serve, make_requests, grid=None, start=None, cache_path=None, key=None):
        self.serve, self.make_requests = serve, make_requests
        self.grid = dict(grid or self.GRID)
        self.best = dict(start or self.START)
        self.cache_path, self.key = cache_path, key
        self.trials = []

    def _cached(self):
        import json
        import os
        if not self.cache_path or not self.key or not os.path.exists(self.cache_path):
            return None
        with open(self.cache_path) as f:
            return json.load(f).get(self.key)

    def _store(self):
        import json
        import os
        if not self.cache_path or not self.key:
            return
        data = {}
        if os.path.exists(self.cache_path):
            with open(self.cache_path) as f:
                data = json.load(f)
        data[self.key] = self.best
        with open(self.cache_path, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)

    def _score(self, params):
        key = tuple(sorted(params.items()))
        for p, sc in self.trials:
            if tuple(sorted(p.items())) == key:
                return sc
        reqs, arr = self.make_requests()
        res = self.serve(params, reqs, arr)
        self.trials.append((dict(params), res["solves_per_s"]))
        return res["solves_per_s"]

    def tune(self):
        hit = self._cached()
        if hit is not None:
            self.best = dict(hit)
            return self.best
        best_score = self._score(self.best)
        for name, values in self.grid.items():
            base = dict(self.best)
            for v in values:
                trial = dict(base, **{name: v})
                sc = self._score(trial)
                if sc > best_score:
                    best_score, self.best = sc, trial
        self._store()
        return self.best
