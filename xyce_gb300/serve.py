"""Continuous batching of transient requests on one GPU (the serving path).

Requests (.STEP / Monte-Carlo variants of a circuit, of uneven sizes) arrive
over time.  The server admits whatever has arrived into a new batch
(xg_batch_*) as soon as the concurrency limit and the device-memory budget
allow, so requests that arrive while others run start at once and their work
overlaps with the running batches on the device (each batch has its own
stream and replays its own CUDA graph).  Each batch is stepped in chunks of
batch iterations; between chunks the server harvests finished requests, so a
short request leaves as soon as it is done, not when its batch is.

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
