"""Algorithmic FP64 operation counts of one Newton load, per instance
(TEST INFRASTRUCTURE ONLY).

The oracle's load sources are compiled over a counting scalar
(oracle/count/xgo_count.hpp) into oracle/_build/liboracle_count.so; a load
through it counts every add/subtract, multiply, divide, square root,
exponential and logarithm the reference's device equations perform, on the
branches each instance takes for its own inputs.  The counts cover
updateState + loadDAEVectors + loadDAEMatrices; the accumulation of stamp
terms into F, Q and the matrices (one add per term, the reduction kernel's
work) is reported apart from the evaluation.

    python oracle/count/count_flops.py [--sample 20000] [--out profiles/flop_counts.json]

samples the first instances of each single-load workload of bench.py with the
benchmark's own node voltages and flags.
"""
import argparse
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from xyce_gb300 import abi, netlists  # noqa: E402

KINDS = ("add", "mul", "div", "sqrt", "exp", "log")


def lib():
    from xyce_gb300 import build
    path = build.build_oracle_count()
    L = C.CDLL(path)
    vp = C.c_void_p
    L.xgo_build.argtypes = [C.POINTER(abi.XgNetlist), C.POINTER(abi.XgDeviceOptions), vp, C.POINTER(vp)]
    L.xgo_free.argtypes = [vp]
    L.xgo_sizes.argtypes = [vp] + [C.POINTER(C.c_int)] * 3 + [C.POINTER(C.c_int64)]
    L.xgo_load.argtypes = [vp, C.POINTER(abi.XgLoadFlags), vp] + [vp] * 8
    L.xgo_count_get.argtypes = [vp]
    return L


def count_load(netlist, params, flags, seed=9, options=None):
    """Operation counts of one load of `netlist` (params: dev_type -> block)
    at the seeded random state netlists.random_state(..., seed)."""
    L = lib()
    opt = options or abi.device_options()
    cnl = netlist.to_c()
    blocks = {t: np.ascontiguousarray(p, np.float64) for t, p in params.items()}
    arr = (C.c_void_p * abi.NUM_DEV_TYPES)()
    for t, b in blocks.items():
        arr[t] = b.ctypes.data
    h = C.c_void_p()
    if L.xgo_build(C.byref(cnl), C.byref(opt), arr, C.byref(h)):
        raise RuntimeError("xgo_build failed")
    n, s, t, z = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
    L.xgo_sizes(h, C.byref(n), C.byref(s), C.byref(t), C.byref(z))
    sol, sta, sto = netlists.random_state(n.value, s.value, t.value, seed=seed)
    ins = [np.array(v, np.float64) for v in list(sol) + list(sta) + list(sto)]
    ins = [v if v.size else np.zeros(1) for v in ins]
    in_arr = (C.c_void_p * 9)(*[v.ctypes.data for v in ins])
    nr = n.value + 1
    outs = [np.zeros(nr) for _ in range(4)] + [np.zeros(max(1, s.value)), np.zeros(max(1, t.value)),
                                               np.zeros(max(1, z.value)), np.zeros(max(1, z.value))]
    L.xgo_count_reset()
    rc = L.xgo_load(h, C.byref(flags), in_arr, *[o.ctypes.data for o in outs])
    got = (C.c_ulonglong * len(KINDS))()
    L.xgo_count_get(got)
    L.xgo_free(h)
    if rc:
        raise RuntimeError(f"xgo_load failed: {rc}")
    return dict(zip(KINDS, (int(x) for x in got)))


def main(argv=None):
    import bench
    from oracle.oracle import setup_params
    ap = argparse.ArgumentParser()
    ap.add_argument("--sample", type=int, default=20000)
    ap.add_argument("--out", default=os.path.join(REPO, "profiles", "flop_counts.json"))
    a = ap.parse_args(argv)
    res = {"command": "python oracle/count/count_flops.py --sample %d" % a.sample,
           "note": "algorithmic FP64 operations of one Newton load per instance, counted by the "
                   "oracle compiled over a counting scalar; eval = device equations and stamp "
                   "terms (the evaluation kernel's work), accumulate = one add per stamp term "
                   "(the reduction kernel's work)"}
    flags = abi.load_flags(transient=1, newton_iter=1, pdt=1e11)
    for name in ("single_load_bsim3_1M", "single_load_mos1_1M"):
        nl = bench.build_workload(name)
        t = [k for k in range(abi.NUM_DEV_TYPES) if nl.count(k)][0]
        sub, _ = bench.slice_netlist(nl, {t: np.zeros((1, nl.count(t)))}, t, 0, a.sample)
        params = {t: setup_params(sub, t)}
        c = count_load(sub, params, flags)
        # stamp terms: one accumulate per term of every instance
        terms = {abi.DEV_BSIM3: 50, abi.DEV_MOS1: 48}[t]
        total = sum(c.values())
        per = {k: v / a.sample for k, v in c.items()}
        acc = terms
        res[name] = {"instances_sampled": a.sample, "per_instance": per,
                     "total_per_instance": total / a.sample,
                     "accumulate_per_instance": acc,
                     "eval_per_instance": total / a.sample - acc}
        print(name, json.dumps(res[name]))
    with open(a.out, "w") as f:
        json.dump(res, f, indent=1)
        f.write("\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
