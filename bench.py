"""Benchmark of the Newton load: device loads per second on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl xg|reference]
                    [--workload single_load_mos1_1M] [--fma]

A step is one Newton load (Device::updateState + loadDAEVectors +
loadDAEMatrices for every instance) of the whole workload with inputs already
resident in HBM; value = device instances loaded per second.  e2e is the same
metric through the C ABI with host buffers: each step uploads the solution
vector from pinned host memory, loads, and reads F, Q, dFdxdVp, dQdxdVp, dF/dx
and dQ/dx back.  Inputs (parameter blocks alone are ~300 MB) exceed the
129 MB L2, so no flush is needed between steps.

--impl reference times the CPU restatement of the reference's load loops
(the oracle; the reference's own sources are not available where this runs)
on all host cores, on the same workload, one process per core over an equal
share of the instances.

Under torchrun (--gpus N > 1) every rank loads its own replica of the workload
(the load of independent circuits does not exchange data): weak scaling,
value = instances of all ranks / max rank time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from xyce_gb300 import abi, netlists  # noqa: E402

# Per-instance algorithmic bytes of one load, by device type: the parameter
# block and LIDs the kernel reads, plus state/store history read and written
# (MOSFET1: 14 doubles read, 13 written; diode: 2 read, 1 written; capacitor:
# 1 written).  Solution reads and output writes are counted once per node /
# non-zero in load_bytes().
# BSIM3: 5 store values of the previous iterate read, 5 store and 5 state
# values written, 20 members carried between loads read and written.
HIST_BYTES = {abi.DEV_MOS1: 27 * 8, abi.DEV_DIODE: 3 * 8, abi.DEV_CAP: 8, abi.DEV_RES: 0,
              abi.DEV_VSRC: 0, abi.DEV_BSIM3: 55 * 8}
NLID = {abi.DEV_RES: 2, abi.DEV_CAP: 2, abi.DEV_VSRC: 3, abi.DEV_DIODE: 3, abi.DEV_MOS1: 6,
        abi.DEV_BSIM3: 6}

WORKLOADS = {
    # Single Newton load of 1,000,000 BSIM3 instances (default level-9 model
    # cards, half NMOS / half PMOS, W~U[0.2,10]um, L~U[0.1,1]um) on a random
    # 250k-node netlist, node voltages U[0,1.8]V
    "single_load_bsim3_1M": dict(kind="random", n_dev=1_000_000, n_nodes=250_000,
                                 dev_type=abi.DEV_BSIM3),
    "single_load_bsim3_100k": dict(kind="random", n_dev=100_000, n_nodes=25_000,
                                   dev_type=abi.DEV_BSIM3),
    # the same at 300,000 instances: its terms and reduction lists (~220 MB)
    # exceed L2, its device memory (~1.2 GB) suits a profiler capture
    "single_load_bsim3_300k": dict(kind="random", n_dev=300_000, n_nodes=75_000,
                                   dev_type=abi.DEV_BSIM3),
    # the same shape (1,000,000 MOSFETs, half NMOS / half PMOS, W~U[0.2,10]um,
    # L~U[0.1,1]um, random 250k-node netlist, node voltages U[0,1.8]V) on the
    # level-1 model
    "single_load_mos1_1M": dict(kind="random", n_dev=1_000_000, n_nodes=250_000,
                                dev_type=abi.DEV_MOS1),
    "single_load_mos1_100k": dict(kind="random", n_dev=100_000, n_nodes=25_000,
                                  dev_type=abi.DEV_MOS1),
    "power_grid_200x200": dict(kind="grid"),
    # .TRAN 1ps 20ns of a 1,000-stage CMOS inverter chain (2,000 level-1
    # MOSFETs, 10 fF per stage, PULSE input 0->1.8 V, 100 ps edges, 2 ns
    # period); one step = one whole transient (DC point + time steps)
    "tran_inverter_chain_1000": dict(kind="tran", circuit="chain", stages=1000, tstop=20e-9,
                                     tstep=1e-12),
    # 200x200 resistive mesh (0.1 ohm, 1 fF per node) with 40,000 diode-
    # clamped level-1 sinks on seeded PULSE gates (delay U[0,5ns]), 120,002
    # unknowns; one step = .TRAN 1ps 3ps (the first breakpoint-dense window)
    "tran_power_grid_200x200": dict(kind="tran", circuit="grid", nx=200, sinks=40000, tstop=3e-12,
                                    tstep=1e-12),
    # 500,000 BSIM3 MOSFETs in seeded random 2-input NAND/NOR/INV logic
    # (fan-out 1-4, 5 fF wires, 200 PULSE inputs), ~250k nodes; one step =
    # .TRAN 2ps 10ps from the logic state (a bounded window of the 10 ns run)
    "tran_random_logic_500k": dict(kind="tran", circuit="logic", n_mos=500_000, tstop=10e-12,
                                   tstep=2e-12),
    # served batch: a Poisson stream (2,000 req/s) of 1,000 seeded Monte-Carlo
    # ring oscillators, 5-501 stages (VTO, KP +-10%), .TRAN 1ps 5ns each from an
    # initial condition; one step = serving the whole stream, FP32 factors with
    # one FP64 refinement step (the FP64 form is measured beside it)
    "serve_ring_mc": dict(kind="serve", n=1000, rate=2000.0, tstop=5e-9),
    # the same stream at its full length of 10,000 requests
    "serve_ring_mc_10k": dict(kind="serve", n=10000, rate=2000.0, tstop=5e-9),
    # one batch: 256 requests of the same Monte-Carlo ring stream, all at
    # once; one step = set up and run the batch to completion (FP32 factors
    # corrected by Newton; the batched kernels without the server's threads)
    "batch_ring_mc_256": dict(kind="batch", n=256, tstop=5e-9),
    # a 60x60 mesh with 1,200 sinks (6,002 unknowns), .TRAN 1ps 20ps: the
    # grid-wide LU path at a size a profiler captures quickly
    "tran_power_grid_60x60": dict(kind="tran", circuit="grid", nx=60, sinks=1200, tstop=20e-12,
                                  tstep=1e-12),
    # 101-stage ring oscillator (level-1, VTO/KP +-10% Monte-Carlo), from an
    # initial condition, .TRAN 1ps 5ns
    "tran_ring_oscillator_101": dict(kind="tran", circuit="ring", stages=101, tstop=5e-9,
                                     tstep=1e-12),
}
METRIC = "device-loads/sec"
TRAN_METRIC = "newton-iters/sec"


def _emit(line, emit):
    """Print the JSON line (emit) or hand it to the caller (a sub-record)."""
    if emit:
        print(json.dumps(line))
        return 0
    return line


def _mapped_libs():
    """This repository's shared libraries mapped into the calling process."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so")}
    except OSError:
        return []
    return sorted(os.path.relpath(q, HERE) for q in paths if q.startswith(HERE + os.sep))


def workload_config(name):
    """The `config` of a workload's line: what the workload is (both arms
    print the same dict); how an arm runs it goes in its `details`."""
    w = WORKLOADS[name]
    k = w["kind"]
    if k == "random":
        return {"workload": name, "instances": w["n_dev"], "nodes": w["n_nodes"],
                "l2": "inputs larger than L2 (parameter blocks alone exceed 129 MB)"}
    if k == "tran":
        return {"workload": name, "tstop": w["tstop"], "tstep": w["tstep"],
                "l2": "working set below L2; latency-bound"}
    if k in ("serve", "batch"):
        c = {"workload": name, "requests": w["n"], "stages": "5-501 odd", "tstop": w["tstop"],
             "l2": "per-request working sets below L2"}
        if k == "serve":
            c["rate_per_s"] = w["rate"]
        return c
    return {"workload": name}


def build_tran(name):
    """(netlist, starting guess over the node unknowns, tstop, tstep, uic, outputs)."""
    w = WORKLOADS[name]
    if w["circuit"] == "chain":
        k = w["stages"]
        nl = netlists.inverter_chain(k)
        return nl, netlists.inverter_chain_nodeset(k), w["tstop"], w["tstep"], False, [1, 2, k + 1]
    if w["circuit"] == "grid":
        nx, ns = w["nx"], w["sinks"]
        nl = netlists.power_grid(nx, nx, ns, seed=0 if nx == 200 else 1)
        return (nl, netlists.power_grid_nodeset(nx, nx, ns), w["tstop"], w["tstep"], False,
                [0, nx * nx // 2, nx * nx - 1])
    if w["circuit"] == "logic":
        nl = netlists.random_logic(w["n_mos"], seed=0)
        o = nl.logic["out"]
        # started from the logic state as an initial condition: the damped
        # Newton DC solve of this many BSIM3 junctions converges linearly
        # (one thermal voltage per iteration under pnjlim) within 200 steps
        return (nl, netlists.random_logic_nodeset(nl), w["tstop"], w["tstep"], True,
                [1, int(o[len(o) // 2]), int(o[-1])])
    k = w["stages"]
    nl = netlists.ring_oscillator(k, seed=3)
    return nl, netlists.ring_oscillator_nodeset(k), w["tstop"], w["tstep"], True, [1, k // 2, k]


def _x0(nl, guess):
    n = nl.n_nodes + nl.count(abi.DEV_VSRC)
    x0 = np.zeros(n)
    x0[:len(guess)] = guess
    return x0


def tran_cpu_baseline(name, seconds=20.0):
    """The oracle's transient driver on one core (the reference is single-
    threaded per rank) over the same window, or the leading part of it that
    fits the time budget."""
    from oracle.oracle import OracleCircuit, all_params, min_degree_order, transient
    nl, guess, tstop, tstep, uic, out = build_tran(name)
    opt = abi.device_options()
    oc = OracleCircuit(nl, all_params(nl, opt), opt)
    order = min_degree_order(oc.rowptr, oc.col)
    window = tstop / 16
    while True:
        t0 = time.perf_counter()
        _, _, st = transient(oc, window, tstep, out, col_order=order, x0=_x0(nl, guess), uic=uic)
        dt = time.perf_counter() - t0
        if dt >= 0.25 * seconds or window >= tstop:
            break
        window = min(tstop, window * max(2.0, 0.5 * seconds / max(dt, 1e-3)))
    oc.close()
    iters = st["newton_iters"] + st["dcop_iters"]
    return iters / dt, iters, window, st


def lu_shape(ctx, c):
    """The LU analysis of the circuit's pattern (sizes of the linear algebra
    per Newton iteration): analysed on the matrix dF/dx + dQ/dx/tstep of a
    load at zero, its diagonal kept away from zero."""
    from xyce_gb300 import engine
    c.set_state(*netlists.random_state(c.n_unknowns, c.n_state, c.n_store, seed=1))
    c.load(abi.load_flags(transient=1, newton_iter=1, pdt=1e12))
    vals = c.download(abi.VEC_DFDX) + 1e12 * c.download(abi.VEC_DQDX)
    rows = np.repeat(np.arange(c.n_unknowns), np.diff(c.rowptr))
    vals[rows == c.colidx] += 1.0
    lu = engine.LU(ctx, c.rowptr, c.colidx, vals)
    info = lu.info
    lu.close()
    return info


def run_tran(args, world, rank, local, dist, emit=True):
    import ctypes as C

    import torch

    from xyce_gb300 import engine
    torch.cuda.set_device(local)
    nl, guess, tstop, tstep, uic, out = build_tran(args.workload)
    prec = abi.LU_FP32 if args.fp32 else abi.LU_FP64
    nref = args.refine if args.fp32 else 0
    # the transient needs the load to the simulation's tolerance, not the
    # reference's rounding: the FMA build (long sums split over a block) unless
    # --exact-load
    ctx = engine.Context(local, abi.device_options(fma=0 if args.exact_load else 1))
    c = engine.Circuit(ctx, nl)
    x0 = _x0(nl, guess)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
    L = engine.lib()
    for _ in range(args.warmup):
        engine.transient(c, tstop, tstep, out, x0=x0, uic=uic, precision=prec, n_refine=nref)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    iters, dev_ms, launches = 0, 0.0, 0
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0 = L.xg_launch_count()
            e0.record(stream)
            tt, vv, st = engine.transient(c, tstop, tstep, out, x0=x0, uic=uic, precision=prec,
                                          n_refine=nref)
            e1.record(stream)
            torch.cuda.synchronize()
            launches += L.xg_launch_count() - l0
            dev_ms += e0.elapsed_time(e1)
            iters += st["newton_iters"] + st["dcop_iters"]
        wall = time.perf_counter() - t0
    step_s = dev_ms / 1e3 / args.steps
    if dist:
        tt_ = torch.tensor([step_s], device=f"cuda:{local}")
        dist.all_reduce(tt_, op=dist.ReduceOp.MAX)
        step_s = float(tt_.item())
    per_step_iters = iters / args.steps
    value = world * per_step_iters / step_s
    if rank != 0:
        c.close()
        return 0
    # the LU of this circuit (shape of the linear-algebra work per iteration)
    info = lu_shape(ctx, c)
    hbm, peak_kind = measured_peaks()
    n_types = sum(1 for t in range(abi.NUM_DEV_TYPES) if nl.count(t))
    params = {t: c.params(t) for t in range(abi.NUM_DEV_TYPES) if nl.count(t)}
    nparams = {t: p.shape[0] for t, p in params.items()}
    # algorithmic bytes of one Newton iteration: the load, the combine (two
    # matrices read, one written), refactor (L\U values and pattern read and
    # written) and solves (read)
    b_iter = (load_bytes(nl, c.n_unknowns, c.nnz, nparams) + 3 * 8 * c.nnz
              + 2 * 12 * info.nnz_lu + 12 * info.nnz_lu)
    ach = b_iter * per_step_iters / step_s / 1e9
    cpu_v, cpu_n, cpu_window, cpu_st = tran_cpu_baseline(args.workload, seconds=args.cpu_seconds)
    c.close()
    line = {
        "metric": TRAN_METRIC, "value": value, "unit": "newton-iters/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded netlist, the reference's benchmark circuit shape)",
        "config": workload_config(args.workload),
        "details": {"unknowns": c.n_unknowns, "nnz": c.nnz, "nnz_lu": info.nnz_lu, "lu_levels": info.levels,
                   "lu_chain_rows": info.solve_chain,
                   "lu_precision": f"fp32+{nref} fp64 refinement" if args.fp32 else "fp64",
                   "lu_order": "nested dissection" if info.ordering == 1 else "minimum degree",
                   "lu_analysis": "done by the first (warm-up) run of the circuit, reused by the "
                                  "timed runs (same first Newton matrix)",
                   "load_build": "exact (reference rounding)" if args.exact_load
                   else "fma, long sums split over a block",
                   "newton_iters_per_step": per_step_iters, "time_steps_per_step": st["steps"]},
        "roofline": {"kernel": "newton iteration", "bound": "hbm", "achieved": ach, "peak": hbm,
                     "unit": "GB/s", "frac": ach / hbm, "traffic": None, "peak_source": peak_kind,
                     "algorithmic_bytes_per_iter": b_iter},
        "e2e": {"value": value * (dev_ms / 1e3) / wall, "unit": "newton-iters/s",
                "h2d_bytes_per_step": 8 * len(x0),
                "d2h_bytes_per_step": int(8 * (1 + len(out)) * (st["steps"] + 1))},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "cpu_baseline": {"value": cpu_v, "unit": "newton-iters/s", "cores": 1, "kind": "port",
                         "sample": f".TRAN window {cpu_window:.3g} s: {cpu_n} Newton iterations on one core"},
        "wall_s": wall,
    }
    return _emit(line, emit)


SERVE_METRIC = "served solves/sec"
# the slot server's schedule grid: slots per batch and batch iterations per
# launch chunk (how many batches a size class opens is demand, bounded by the
# memory admission, not a schedule)
SLOT_TUNING = dict(grid={"slots": (256, 512, 1024), "chunk": (16, 32, 64)},
                   start={"slots": 512, "chunk": 32})


def run_serve(args, world, rank, local, dist, emit=True):
    import torch

    from xyce_gb300 import engine, serve
    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    # as for the transients: the FMA load build (long sums split over a block)
    # unless --exact-load
    ctx = engine.Context(local, abi.device_options(fma=0 if args.exact_load else 1))
    L = engine.lib()

    # slot shapes of the stream's size classes (its largest ring per class)
    shapes = serve.ring_class_shapes(ctx, stages=(5, 501), tstop=w["tstop"])

    def make(kind, prec, nref, params):
        if kind == "slots":
            return serve.SlotServer(ctx, shapes, precision=prec, n_refine=nref, **params)
        return serve.Server(ctx, precision=prec, n_refine=nref, **params)

    # the schedule, picked by the autotuner on a smaller probe stream of the
    # same kind (not timed), per server: long enough (half a second of
    # arrivals at 2,000/s) to hold as many requests in flight as the stream
    # does, so a schedule with too few slots shows up in the probe
    def probe():
        n = min(w["n"], 1000)
        return (serve.ring_mc_requests(n, seed=7, tstop=w["tstop"]),
                serve.poisson_arrivals(n, w["rate"], seed=8))

    def run_once(kind, prec, nref, params, reqs, arr):
        srv = make(kind, prec, nref, params)
        try:
            return srv.run(reqs, arr)
        finally:
            srv.close()

    def tune(kind):
        t = serve.Autotuner(lambda params, reqs, arr: run_once(kind, abi.LU_FP32, 0, params, reqs, arr),
                            probe, **(SLOT_TUNING if kind == "slots" else {}))
        return t.tune(), len(t.trials)

    sched, trials = tune(args.server)
    other = "batches" if args.server == "slots" else "slots"
    sched_other = tune(other)[0] if not args.no_sweep else None

    # one long-running server per form, warmed by the warm-up streams (a
    # slot server keeps its batches between streams, as a service does)
    servers = {}

    def one(prec, nref, n=None):
        n = n or w["n"]
        reqs = serve.ring_mc_requests(n, seed=1, tstop=w["tstop"])
        arr = serve.poisson_arrivals(n, w["rate"], seed=2)
        key = (prec, nref)
        if key not in servers:
            servers[key] = make(args.server, prec, nref, sched)
        res = servers[key].run(reqs, arr)
        return res, reqs

    # the mixed-precision form: FP32 factors and solves; every Newton step
    # computes the FP64 residual F(x) and solves for its correction, so the
    # Newton iteration refines the FP32 solve against the FP64 residual
    # (warm-up streams: the first 1,000 requests of the stream at most)
    for _ in range(args.warmup):
        for prec, nref in ((abi.LU_FP32, 0), (abi.LU_FP64, 0), (abi.LU_FP32, 1)):
            one(prec, nref, min(w["n"], 1000))
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    runs, fp64, refined = [], [], []
    l0 = L.xg_launch_count()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            res, reqs = one(abi.LU_FP32, 0)
            runs.append((res, reqs))
        wall = time.perf_counter() - t0
    launches = L.xg_launch_count() - l0
    for _ in range(max(1, args.steps // 2)):
        fp64.append(one(abi.LU_FP64, 0))
        refined.append(one(abi.LU_FP32, 1))
    for srv in servers.values():
        srv.close()
    # latency against offered load: the same kind of stream at other rates,
    # about two seconds of arrivals each (at most the workload's request count)
    sweep = []
    if not args.no_sweep:
        for rate in [float(r) for r in args.sweep_rates.split(",") if r]:
            n = int(min(w["n"], max(100, 2 * rate)))
            row = {"rate_per_s": rate, "requests": n}
            for kind, sch in ((args.server, sched), (other, sched_other)):
                row[kind] = {}
                for name, prec in (("mixed", abi.LU_FP32), ("fp64", abi.LU_FP64)):
                    reqs = serve.ring_mc_requests(n, seed=3, tstop=w["tstop"])
                    arr = serve.poisson_arrivals(n, rate, seed=4)
                    srv = make(kind, prec, 0, sch)
                    try:
                        # warmed first by a short burst of the same kind, as a
                        # running service is (a slot server keeps its batches)
                        srv.run(serve.ring_mc_requests(200, seed=5, tstop=w["tstop"]),
                                serve.poisson_arrivals(200, 5000.0, seed=6))
                        r = srv.run(reqs, arr)
                    finally:
                        srv.close()
                    row[kind][name] = {"solves_per_s": r["solves_per_s"], "p50_ms": r["p50_ms"],
                                       "p99_ms": r["p99_ms"]}
            sweep.append(row)
    if rank != 0:
        return 0
    # accuracy of the mixed-precision forms against the FP64 form, request by request
    def wave_diff(other):
        e = 0.0
        for (ta, va, _), (tb, vb, _) in zip((r.result for r in fp64[0][1]), (r.result for r in other)):
            vi = np.stack([np.interp(ta, tb, vb[:, k]) for k in range(vb.shape[1])], 1)
            e = max(e, float(np.abs(vi - va).max()))
        return e
    err = wave_diff(runs[0][1])
    err_ref = wave_diff(refined[0][1])
    sps = [r[0]["solves_per_s"] for r in runs]
    value = world * float(np.mean(sps))
    step_s = float(np.mean([r[0]["wall_s"] for r in runs]))
    f64 = fp64[0][0]
    cpu_v, cpu_n = serve_cpu_baseline(args.cpu_seconds)
    line = {
        "metric": SERVE_METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Monte-Carlo ring oscillators, Poisson arrivals)",
        "config": workload_config(args.workload),
        "details": {"lu": "fp32 factors and solves, corrected by Newton against the fp64 residual",
                   "load_build": "exact (reference rounding)" if args.exact_load
                   else "fma, long sums split over a block",
                   "server": args.server, "schedule": sched, "autotuner_trials": trials,
                   "other_server_schedule": sched_other},
        "p50_ms": float(np.mean([r[0]["p50_ms"] for r in runs])),
        "p99_ms": float(np.mean([r[0]["p99_ms"] for r in runs])),
        "fp64": {"solves_per_s": f64["solves_per_s"], "p50_ms": f64["p50_ms"], "p99_ms": f64["p99_ms"]},
        "fp32_plus_1_fp64_refinement": {
            "solves_per_s": refined[0][0]["solves_per_s"], "p50_ms": refined[0][0]["p50_ms"],
            "p99_ms": refined[0][0]["p99_ms"], "max_waveform_diff_vs_fp64_v": err_ref},
        "fp32_vs_fp64_max_waveform_diff_v": err,
        "rate_sweep": sweep,
        "newton_iters_per_s": float(np.mean([r[0]["newton_iters_per_s"] for r in runs])),
        "roofline": {"kernel": "batch iteration", "bound": "hbm", "achieved": None, "peak": measured_peaks()[0],
                     "unit": "GB/s", "frac": None, "traffic": None,
                     "note": "latency-bound: each request's factor runs level by level in one 128-thread block"},
        "e2e": {"value": value, "unit": "solves/s",
                "h2d_bytes_per_step": int(sum(8 * len(r.x0) for r in runs[0][1])),
                "d2h_bytes_per_step": int(sum(r.result[1].nbytes + r.result[0].nbytes for r in runs[0][1]))},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "cpu_baseline": {"value": cpu_v, "unit": "solves/s", "cores": 1, "kind": "port",
                         "sample": f"{cpu_n} requests of the same stream, one core"},
        "wall_s": wall,
    }
    return _emit(line, emit)


def run_batch(args, world, rank, local, dist):
    import torch

    from xyce_gb300 import engine, serve
    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ctx = engine.Context(local, abi.device_options(fma=0 if args.exact_load else 1))
    L = engine.lib()
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
    reqs = serve.ring_mc_requests(w["n"], seed=1, tstop=w["tstop"])
    prec, nref = (abi.LU_FP64, 0) if not args.fp32_batch else (abi.LU_FP32, 0)

    def one():
        b = engine.Batch(ctx, [r.netlist for r in reqs], [r.x0 for r in reqs],
                         [r.tstop for r in reqs], [r.out_idx for r in reqs], tstep=1e-12,
                         precision=prec, n_refine=nref, max_points=8192)
        it = 0
        while True:
            b.run(64)
            it += 64
            if b.poll(wait=True) == len(reqs):
                break
        newton = sum(b.stats(i)["newton_iters"] for i in range(len(reqs)))
        b.close()
        return it, newton

    for _ in range(args.warmup):
        one()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = L.xg_launch_count()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        res = [one() for _ in range(args.steps)]
        wall = time.perf_counter() - t0
    launches = L.xg_launch_count() - l0
    if rank != 0:
        return 0
    step_s = wall / args.steps
    batch_iters = res[0][0]
    newton = float(np.mean([r[1] for r in res]))
    value = world * len(reqs) / step_s
    cpu_v, cpu_n = serve_cpu_baseline(args.cpu_seconds)
    line = {
        "metric": "solves/sec", "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Monte-Carlo ring oscillators, 5-501 stages)",
        "config": workload_config(args.workload),
        "details": {"lu": "fp32, corrected by Newton" if args.fp32_batch else "fp64",
                   "batch_iterations": batch_iters, "newton_iters_per_step": newton,
                   "step": "set-up included (host analysis of every request)"},
        "newton_iters_per_s": newton / step_s,
        "roofline": {"kernel": "batch iteration", "bound": "hbm", "achieved": None,
                     "peak": measured_peaks()[0], "unit": "GB/s", "frac": None, "traffic": None,
                     "note": "latency-bound: each request's factor runs level by level in one block"},
        "e2e": {"value": value, "unit": "solves/s",
                "h2d_bytes_per_step": int(sum(8 * len(r.x0) for r in reqs)),
                "d2h_bytes_per_step": 0},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "cpu_baseline": {"value": cpu_v, "unit": "solves/s", "cores": 1, "kind": "port",
                         "sample": f"{cpu_n} requests of the same stream, one core"},
        "wall_s": wall,
    }
    print(json.dumps(line))
    return 0


def _serve_ref_worker(job):
    """Reference arm for serving: requests solved one after another on one core."""
    idx, n, tstop = job
    from oracle.oracle import OracleCircuit, all_params, min_degree_order, transient
    from xyce_gb300 import serve
    reqs = serve.ring_mc_requests(n, seed=1, tstop=tstop)
    opt = abi.device_options()
    t0 = time.perf_counter()
    done = 0
    for k in idx:
        r = reqs[k]
        oc = OracleCircuit(r.netlist, all_params(r.netlist, opt), opt)
        order = min_degree_order(oc.rowptr, oc.col)
        transient(oc, r.tstop, 1e-12, r.out_idx, col_order=order, x0=r.x0, uic=True)
        oc.close()
        done += 1
    return done, time.perf_counter() - t0, _mapped_libs()


def serve_cpu_baseline(seconds=10.0):
    """One core solving the stream's requests back to back for about `seconds`."""
    w = WORKLOADS["serve_ring_mc"]
    done, t = 0, 0.0
    k = 0
    while t < seconds and k < w["n"]:
        d, dt, _ = _serve_ref_worker(([k], w["n"], w["tstop"]))
        done += d
        t += dt
        k += 1
    return done / t, done


def run_serve_reference(args, world, rank, emit=True):
    """CPU arm for serving: the request stream spread over every host core,
    each request solved by the oracle's transient driver."""
    if rank != 0:
        return 0
    import multiprocessing as mp
    w = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    sample = min(w["n"], 8 * cores)
    jobs = [(list(range(c, sample, cores)), w["n"], w["tstop"]) for c in range(cores)]
    ctx = mp.get_context("spawn")
    times, libs = [], set(_mapped_libs())
    with ctx.Pool(cores) as pool:
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            out = pool.map(_serve_ref_worker, jobs)
            if k >= args.warmup:
                times.append(time.perf_counter() - t0)
            libs |= {q for r in out for q in r[2]}
    t = float(np.mean(times))
    value = sample / t
    line = {"metric": SERVE_METRIC if w["kind"] == "serve" else "solves/sec", "value": value,
            "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": workload_config(args.workload),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": f"{sample} of {w['n']} requests per step over {cores} processes",
                             "libraries": sorted(libs)},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    return _emit(line, emit)


def run_tran_reference(args, world, rank, emit=True):
    """CPU arm for transient workloads: the oracle's transient driver, one
    core per run (the reference's transient is single-threaded per rank)."""
    if rank != 0:
        return 0
    from oracle.oracle import OracleCircuit, all_params, min_degree_order, transient
    nl, guess, tstop, tstep, uic, out = build_tran(args.workload)
    opt = abi.device_options()
    oc = OracleCircuit(nl, all_params(nl, opt), opt)
    order = min_degree_order(oc.rowptr, oc.col)
    # bounded per step: the leading window of the transient that one core
    # finishes in about the budget
    _, _, window, _ = tran_cpu_baseline(args.workload, seconds=args.cpu_seconds)
    times, iters = [], []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, _, st = transient(oc, window, tstep, out, col_order=order, x0=_x0(nl, guess), uic=uic)
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
            iters.append(st["newton_iters"] + st["dcop_iters"])
    oc.close()
    t = float(np.mean(times))
    value = float(np.mean(iters)) / t
    line = {"metric": TRAN_METRIC, "value": value, "unit": "newton-iters/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": workload_config(args.workload),
            "cpu_baseline": {"value": value, "unit": "newton-iters/s", "cores": 1, "kind": "port",
                             "sample": f".TRAN window {window:.3g} s per step, one core (the "
                                       "reference's transient runs on one thread)",
                             "libraries": _mapped_libs()},
            "e2e": {"value": value, "unit": "newton-iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    return _emit(line, emit)


def build_workload(name):
    w = WORKLOADS[name]
    if w["kind"] == "random":
        models = None
        if w["dev_type"] == abi.DEV_BSIM3:
            models = (abi.Model(abi.DEV_BSIM3, 1), abi.Model(abi.DEV_BSIM3, -1))
        nl = netlists.random_mos_netlist(w["n_dev"], w["n_nodes"], dev_type=w["dev_type"], seed=2,
                                         models=models)
    else:
        nl = netlists.power_grid(200, 200, 40000, seed=0)
    return nl


def n_instances(nl):
    return sum(nl.count(t) for t in range(abi.NUM_DEV_TYPES))


def load_bytes(nl, n_unknowns, nnz, nparams):
    b = 0
    for t in range(abi.NUM_DEV_TYPES):
        n = nl.count(t)
        if n:
            b += n * (nparams[t] * 8 + NLID[t] * 4 + HIST_BYTES[t])
    b += 8 * (n_unknowns + 1)                 # solution read
    b += 4 * 8 * (n_unknowns + 1)             # F, Q, dFdxdVp, dQdxdVp written
    b += 2 * 8 * nnz                          # dF/dx, dQ/dx values written
    return b


def eval_bytes(nl, n_unknowns, nparams):
    b = 8 * (n_unknowns + 1)
    for t in range(abi.NUM_DEV_TYPES):
        n = nl.count(t)
        if n:
            b += n * (nparams[t] * 8 + NLID[t] * 4 + HIST_BYTES[t])
    return b


def ncu_counts(workload, kernel):
    """Per-launch DRAM bytes and executed FP64 flops of `kernel` on `workload`
    from the committed ncu summary (profiles/ncu_counts.json), or {}."""
    p = os.path.join(HERE, "profiles", "ncu_counts.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f).get(workload, {}).get(kernel, {})


def flop_counts(workload):
    """Algorithmic FP64 operations of one load per instance (committed counts
    of the oracle compiled over a counting scalar, oracle/count/), or {}."""
    p = os.path.join(HERE, "profiles", "flop_counts.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f).get(workload, {})


def fp64_roofline(workload, counts, n_inst, kernel_ms, peak_flops, fma, traffic):
    """The evaluation kernels are bound by the FP64 pipe.  achieved =
    algorithmic FP64 operations of the launch (the reference equations'
    adds, multiplies, divides, square roots, exponentials and logarithms,
    each counted once) over the launch time; peak = the DFMA throughput
    probed on this GPU in the same process (GB300 nominal FP64: 1.25
    TFLOP/s).  Executed FP64 flops (ncu, the exact build: a divide or
    transcendental costs many instructions) are reported beside it."""
    fc = flop_counts(workload)
    alg = fc.get("eval_per_instance", 0.0) * n_inst
    secs = kernel_ms / 1e3
    out = {"kernel": "eval", "bound": "fp64", "unit": "TFLOP/s",
           "peak": peak_flops / 1e12 if peak_flops else None, "traffic": traffic,
           "peak_source": "xg_probe_fp64_rate (DFMA chains, this GPU, this run)",
           "algorithmic_flops_per_launch": alg or None}
    if alg and peak_flops:
        out["achieved"] = alg / secs / 1e12
        out["frac"] = alg / secs / peak_flops
    else:
        out["achieved"] = out["frac"] = None
    ex = counts.get("fp64_flops")
    if ex and peak_flops and fma == (counts.get("build") == "fast"):
        out["executed_flops_per_launch"] = ex
        out["executed_achieved"] = ex / secs / 1e12
        out["frac_executed"] = ex / secs / peak_flops
        out["fp64_pipe_active_ncu"] = counts.get("fp64_pipe_active")
    return out


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "xg" else "gloo"
        if args.impl == "xg":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def slice_netlist(nl, params, t, i0, i1):
    """The instances [i0, i1) of single-type workload nl, with their parameter
    columns: a bounded sample whose load is the same per-instance work."""
    sub = abi.Netlist(nl.n_nodes)
    sub.models = nl.models
    grp = abi.Netlist._GROUPS[t]
    setattr(sub, grp, {k: np.asarray(v)[i0:i1] for k, v in getattr(nl, grp).items()
                       if v is not None})
    return sub, {t: np.ascontiguousarray(params[t][:, i0:i1])}


def cpu_baseline_sample(nl, params, opt, seconds=10.0, max_instances=200_000):
    """The oracle on one core over a bounded sample of the workload."""
    from oracle.oracle import OracleCircuit, setup_params
    t = [k for k in range(abi.NUM_DEV_TYPES) if nl.count(k)][0]
    nl, _ = slice_netlist(nl, {t: np.zeros((1, nl.count(t)))}, t, 0, min(nl.count(t), max_instances))
    oc = OracleCircuit(nl, {t: setup_params(nl, t, opt)}, opt)
    sol, sta, sto = netlists.random_state(oc.n_unknowns, oc.n_state, oc.n_store, seed=9)
    flags = abi.load_flags(transient=1, newton_iter=1, pdt=1e11)
    done = 0
    scratch = None
    t0 = time.perf_counter()
    chunk = 20000
    types = [t for t in range(abi.NUM_DEV_TYPES) if nl.count(t)]
    while time.perf_counter() - t0 < seconds:
        for t in types:
            n = nl.count(t)
            i0 = done % n
            i1 = min(n, i0 + chunk)
            scratch = oc.load_range_timed(flags, sol, sta, sto, t, i0, i1, scratch)
            done += i1 - i0
    dt = time.perf_counter() - t0
    oc.close()
    return done / dt, done


def _ref_worker(args):
    """One host process of the reference arm: loads instances [i0, i1)."""
    name, i0, i1, steps, warmup = args
    from oracle.oracle import OracleCircuit, setup_params
    nl = build_workload(name)
    opt = abi.device_options()
    t = [t for t in range(abi.NUM_DEV_TYPES) if nl.count(t)][0]
    sub = slice_netlist(nl, {t: np.zeros((1, nl.count(t)))}, t, i0, i1)[0]
    params = {t: setup_params(sub, t, opt)}
    oc = OracleCircuit(sub, params, opt)
    sol, sta, sto = netlists.random_state(oc.n_unknowns, oc.n_state, oc.n_store, seed=9)
    flags = abi.load_flags(transient=1, newton_iter=1, pdt=1e11)
    i0, i1 = 0, i1 - i0
    scratch = None
    times = []
    for k in range(warmup + steps):
        t0 = time.perf_counter()
        scratch = oc.load_range_timed(flags, sol, sta, sto, t, i0, i1, scratch)
        if k >= warmup:
            times.append(time.perf_counter() - t0)
    return times, _mapped_libs()


def run_reference(args, world, rank, emit=True):
    """CPU arm: the oracle port on all host cores (rank 0 only)."""
    if rank != 0:
        return 0
    import multiprocessing as mp
    nl = build_workload(args.workload)
    types = [t for t in range(abi.NUM_DEV_TYPES) if nl.count(t)]
    if len(types) != 1:
        print(json.dumps({"impl": "reference", "unavailable": "reference arm supports single-type workloads"}))
        return 0
    n = nl.count(types[0])
    cores = os.cpu_count() or 1
    # a bounded sample: each process loads its share of at most 2M instances
    sample = min(n, 2_000_000)
    bounds = np.linspace(0, sample, cores + 1).astype(int)
    jobs = [(args.workload, int(bounds[k]), int(bounds[k + 1]), args.steps, args.warmup)
            for k in range(cores) if bounds[k + 1] > bounds[k]]
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(jobs)) as pool:
        out = pool.map(_ref_worker, jobs)
    res = [r[0] for r in out]
    libs = sorted({q for r in out for q in r[1]} | set(_mapped_libs()))
    per_step = np.max(np.array(res), axis=0)       # slowest process per step
    t = float(np.mean(per_step))
    value = sample / t
    line = {"metric": METRIC, "value": value, "unit": "instances/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3 * n / sample,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": workload_config(args.workload),
            "cpu_baseline": {"value": value, "unit": "instances/s", "cores": len(jobs),
                             "kind": "port",
                             "sample": f"{sample} of {n} instances per step, {len(jobs)} processes",
                             "libraries": libs},
            "e2e": {"value": value, "unit": "instances/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    return _emit(line, emit)


def run_xg(args, world, rank, local, dist, emit=True):
    import ctypes as C

    import torch

    from xyce_gb300 import engine

    torch.cuda.set_device(local)
    nl = build_workload(args.workload)
    # the FMA build (contracted products, shared reciprocals; held to the
    # per-entry tolerance) unless --exact-load asks for the reference's rounding
    fma = 0 if args.exact_load else 1
    opt = abi.device_options(fma=fma)
    ctx = engine.Context(local, opt)
    t_setup = time.perf_counter()
    c = engine.Circuit(ctx, nl)
    t_setup = time.perf_counter() - t_setup
    sol, sta, sto = netlists.random_state(c.n_unknowns, c.n_state, c.n_store, seed=9)
    c.set_state(sol, sta, sto)
    flags = abi.load_flags(transient=1, newton_iter=1, pdt=1e11)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
    n_inst = n_instances(nl)
    n_types = sum(1 for t in range(abi.NUM_DEV_TYPES) if nl.count(t))

    for _ in range(args.warmup):
        c.update_state(flags)
        c.load_dae_vectors()
        c.load_dae_matrices()
    ctx.synchronize()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    L0 = engine.lib().xg_launch_count()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            c.update_state(flags)
            ev[k][1].record(stream)
            c.load_dae_vectors()
            c.load_dae_matrices()
            ev[k][2].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = engine.lib().xg_launch_count() - L0
    eval_ms = [ev[k][0].elapsed_time(ev[k][1]) for k in range(args.steps)]
    red_ms = [ev[k][1].elapsed_time(ev[k][2]) for k in range(args.steps)]
    step_ms = float(np.mean([a + b for a, b in zip(eval_ms, red_ms)]))
    step_s = step_ms / 1e3
    if dist:
        tt = torch.tensor([step_s], device=f"cuda:{local}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        step_s = float(tt.item())
    value = world * n_inst / step_s

    # e2e through the C ABI with host buffers.
    host_sol = torch.empty(c.n_unknowns + 1, dtype=torch.float64, pin_memory=True)
    host_sol.copy_(torch.from_numpy(sol[0]))
    outs = {vid: torch.empty(c.vec_size(vid), dtype=torch.float64, pin_memory=True)
            for vid in (abi.VEC_F, abi.VEC_Q, abi.VEC_DFDXDVP, abi.VEC_DQDXDVP, abi.VEC_DFDX,
                        abi.VEC_DQDX)}
    L = engine.lib()
    h2d = 8 * (c.n_unknowns + 1)
    d2h = sum(8 * t.numel() for t in outs.values())

    def e2e_step():
        engine.check(L.xg_vec_upload(c.h, abi.VEC_SOL_NEXT, C.c_void_p(host_sol.data_ptr())))
        c.load(flags)
        for vid, t in outs.items():
            engine.check(L.xg_vec_download(c.h, vid, C.c_void_p(t.data_ptr())))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    if dist:
        tt = torch.tensor([e2e_s], device=f"cuda:{local}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())

    if rank != 0:
        c.close()
        return 0

    hbm, peak_kind = measured_peaks()
    fp64_peak = C.c_double(0.0)
    if L.xg_probe_fp64_rate(local, C.byref(fp64_peak)) != 0:
        fp64_peak.value = 0.0
    fp64_peak = fp64_peak.value
    ev_ms = float(np.mean(eval_ms))
    rd_ms = float(np.mean(red_ms))
    params = {t: c.params(t) for t in range(abi.NUM_DEV_TYPES) if nl.count(t)}
    nparams = {t: p.shape[0] for t, p in params.items()}
    b_load = load_bytes(nl, c.n_unknowns, c.nnz, nparams)
    b_eval = eval_bytes(nl, c.n_unknowns, nparams)
    b_red = 4 * 8 * (c.n_unknowns + 1) + 2 * 8 * c.nnz
    dom = "eval" if ev_ms >= rd_ms else "reduce"
    ach = (b_eval / (ev_ms / 1e3) if dom == "eval" else b_red / (rd_ms / 1e3)) / 1e9
    counts = ncu_counts(args.workload, dom + ("_fma" if fma else ""))
    traffic = counts.get("dram_bytes")
    c.close()
    cpu_v, cpu_n = cpu_baseline_sample(nl, None, opt, seconds=args.cpu_seconds)
    clk = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "instances/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random netlist and node voltages)",
        "config": workload_config(args.workload),
        "details": {"unknowns": c.n_unknowns, "nnz": c.nnz,
                    "load_build": "exact (reference rounding)" if not fma
                    else "fma (contracted products, shared reciprocals)",
                    "setup_s": round(t_setup, 3)},
        "kernels_ms": {"eval": ev_ms, "reduce": rd_ms},
        "roofline": fp64_roofline(args.workload, counts, n_inst, ev_ms, fp64_peak, bool(fma),
                                  traffic) if dom == "eval" else None,
        "roofline_hbm": {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm,
                         "unit": "GB/s", "frac": ach / hbm, "traffic": traffic,
                         "peak_source": peak_kind,
                         "algorithmic_bytes": b_eval if dom == "eval" else b_red},
        "roofline_load": {"achieved": b_load / step_s / 1e9, "unit": "GB/s",
                          "frac": b_load / step_s / 1e9 / hbm, "algorithmic_bytes": b_load},
        "e2e": {"value": world * n_inst / e2e_s, "unit": "instances/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clk,
        "cpu_baseline": {"value": cpu_v, "unit": "instances/s", "cores": 1, "kind": "port",
                         "sample": f"{cpu_n} instance loads in ~{args.cpu_seconds:.0f} s, one core"},
        "wall_s": wall,
    }
    return _emit(line, emit)


DEFAULT_WORKLOAD = "single_load_bsim3_1M"
# The default run's sub-records: the other two metrics of the headline
# benchmark, each on its own workload (Newton iterations per second of the
# 1,000-stage inverter chain's whole .TRAN 1ps 20ns; served solves per second
# and latency of the 10,000-request Monte-Carlo ring stream).
SUB_NEWTON = dict(workload="tran_inverter_chain_1000", steps=3, warmup=1, fp32=False)
# the two LU-bound transients: the 200x200 power grid's first 3 ps and the
# 500k-BSIM3 random logic's first 10 ps, Newton iterations per second
SUB_NEWTON_LARGE = {
    "newton_power_grid_200x200": dict(workload="tran_power_grid_200x200", steps=2, warmup=1, fp32=False),
    "newton_random_logic_500k": dict(workload="tran_random_logic_500k", steps=2, warmup=1, fp32=False),
}
SUB_SERVE = dict(workload="serve_ring_mc_10k", steps=1, warmup=1, sweep_rates="100,2000",
                 no_sweep=False)


def _sub_args(args, over):
    a = argparse.Namespace(**vars(args))
    for k, v in over.items():
        setattr(a, k, v)
    a.cpu_seconds = min(args.cpu_seconds, 5.0)
    return a


def run_default(args, world, rank, local, dist):
    """The single load (headline line) with the Newton and serving metrics
    as sub-records of the same line: the 1,000-stage chain, the power grid
    and the random logic transients, and the served stream."""
    line = run_xg(args, world, rank, local, dist, emit=False)
    newton = run_tran(_sub_args(args, SUB_NEWTON), world, rank, local, dist, emit=False)
    large = {k: run_tran(_sub_args(args, v), world, rank, local, dist, emit=False)
             for k, v in SUB_NEWTON_LARGE.items()}
    serving = run_serve(_sub_args(args, SUB_SERVE), world, rank, local, dist, emit=False)
    if rank != 0:
        return 0
    line["newton"] = newton
    line.update(large)
    line["serving"] = serving
    line["gpu_launches_sub"] = {"newton": newton["gpu_launches"], "serving": serving["gpu_launches"]}
    line["gpu_launches_sub"].update({k: v["gpu_launches"] for k, v in large.items()})
    return _emit(line, True)


def run_default_reference(args, world, rank):
    if rank != 0:
        return 0
    line = run_reference(args, world, rank, emit=False)
    line["newton"] = run_tran_reference(_sub_args(args, SUB_NEWTON), world, rank, emit=False)
    for k, v in SUB_NEWTON_LARGE.items():
        line[k] = run_tran_reference(_sub_args(args, v), world, rank, emit=False)
    line["serving"] = run_serve_reference(_sub_args(args, SUB_SERVE), world, rank, emit=False)
    return _emit(line, True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xg", choices=["xg", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--fp32", action="store_true", help="transient: FP32 factors + FP64 refinement")
    ap.add_argument("--refine", type=int, default=2,
                    help="transient with --fp32: FP64 refinement steps per solve")
    ap.add_argument("--no-sweep", action="store_true", help="serving: skip the arrival-rate sweep")
    ap.add_argument("--server", default="slots", choices=["slots", "batches"],
                    help="serving: requests join running batches in freed slots (slots) or wait "
                         "for new fixed batches (batches); the sweep measures both")
    ap.add_argument("--sweep-rates", default="100,500,2000,5000",
                    help="serving: arrival rates [req/s] of the latency sweep")
    ap.add_argument("--no-sub", action="store_true",
                    help="default workload: the single load alone, without the Newton and "
                         "serving sub-records")
    ap.add_argument("--fp32-batch", action="store_true",
                    help="batch workload: FP32 factors (Newton-corrected)")
    ap.add_argument("--exact-load", action="store_true",
                    help="the bit-exact load build (the reference's rounding) instead of the "
                         "FMA build")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    world, rank, local, dist = dist_setup(args)
    kind = WORKLOADS[args.workload]["kind"]
    composite = args.workload == DEFAULT_WORKLOAD and not args.no_sub
    if args.impl == "reference":
        ref = {"tran": run_tran_reference, "serve": run_serve_reference,
               "batch": run_serve_reference}.get(kind, run_reference)
        rc = run_default_reference(args, world, rank) if composite else ref(args, world, rank)
    else:
        arm = {"tran": run_tran, "serve": run_serve, "batch": run_batch}.get(kind, run_xg)
        rc = (run_default(args, world, rank, local, dist) if composite
              else arm(args, world, rank, local, dist))
    if dist:
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
