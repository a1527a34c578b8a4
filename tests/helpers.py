"""Shared test helpers: golden-fixture loading and output comparison."""
import glob
import os

import numpy as np

from xyce_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

VEC_KEYS = ("F", "Q", "dFdxdVp", "dQdxdVp", "sta_next", "sto_next")
MAT_KEYS = ("dFdx", "dQdx")

# Parity tolerance for results computed with different exp/log
# implementations or with fused multiply-add: per entry
#   |a - b| <= RTOL * |b| + ATOL_FRAC * max|b over that output|
# ATOL_FRAC floors the relative test where terms of opposite sign cancel
# (a sum far smaller than its terms cannot carry 1e-12 relative accuracy).
RTOL = 1e-12
ATOL_FRAC = 1e-13


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


class Golden:
    def __init__(self, path):
        z = np.load(path)
        self.name = os.path.splitext(os.path.basename(path))[0]
        self.z = z
        self.netlist = abi.Netlist.from_arrays({k[3:]: z[k] for k in z.files if k.startswith("nl.")})
        o = z["opt"]
        self.options = abi.device_options(gmin=o[0], temp=o[1], tnom=o[2], voltlim=int(o[3]),
                                          newmeyer=int(o[4]), fma=int(o[5]))
        self.params = {int(k.split(".")[1]): z[k] for k in z.files if k.startswith("params.")}
        self.sizes = tuple(int(x) for x in z["sizes"])
        self.n_loads = int(z["n_loads"])

    def flags(self, k):
        f = self.z[f"load{k}.flags"]
        init_tran = int(f[10]) if len(f) > 10 else 0
        return abi.XgLoadFlags(*[int(x) for x in f[:8]], float(f[8]), float(f[9]), init_tran)

    def full_params(self, options=None):
        """Parameter blocks for the oracle: the reference's own values where
        the fixture holds the whole block; for BSIM3, whose fixture holds the
        reference's raw columns only, the engine's host setup (whose raw
        columns the setup test pins to the fixture)."""
        from xyce_gb300 import engine
        out = dict(self.params)
        if abi.DEV_BSIM3 in out:
            out[abi.DEV_BSIM3] = engine.setup_params(self.netlist, abi.DEV_BSIM3,
                                                    options or self.options)
        return out

    def inputs(self, k):
        z = self.z
        sol = [z[f"load{k}.sol{j}"] for j in range(3)]
        sta = [z[f"load{k}.sta{j}"] for j in range(3)]
        sto = [z[f"load{k}.sto{j}"] for j in range(3)]
        return sol, sta, sto

    def outputs(self, k):
        return {key: self.z[f"load{k}.out.{key}"] for key in VEC_KEYS + MAT_KEYS + ("rows", "cols")}


def mat_dict(out, key):
    return {(int(r), int(c)): float(v) for r, c, v in zip(out["rows"], out["cols"], out[key])}


def compare(a, b, exact=True):
    """Compare two load results (a against reference b).  Returns a dict of
    per-output (n_entries, n_not_identical, max_violation) where violation is
    |a-b| / (RTOL|b| + ATOL_FRAC*max|b|); exact=True demands identical values."""
    rep = {}
    for k in VEC_KEYS:
        x, y = np.asarray(a[k], float), np.asarray(b[k], float)
        assert x.shape == y.shape, (k, x.shape, y.shape)
        rep[k] = _cmp(x, y)
    same_pattern = (len(a["rows"]) == len(b["rows"]) and np.array_equal(a["rows"], b["rows"])
                    and np.array_equal(a["cols"], b["cols"]))
    for k in MAT_KEYS:
        if same_pattern:
            rep[k] = _cmp(np.asarray(a[k], float), np.asarray(b[k], float))
            continue
        A, B = mat_dict(a, k), mat_dict(b, k)
        keys = sorted(set(A) | set(B))
        x = np.array([A.get(q, 0.0) for q in keys])
        y = np.array([B.get(q, 0.0) for q in keys])
        rep[k] = _cmp(x, y)
    bad = {k: v for k, v in rep.items() if (v[1] if exact else v[2] > 1.0)}
    return rep, bad


def max_rel_above_floor(a, b):
    """Largest |a-b|/|b| over the entries of every output whose reference
    value is above the absolute floor ATOL_FRAC * max|b| of that output (the
    entries the relative bound governs on its own)."""
    worst = 0.0
    same_pattern = (len(a["rows"]) == len(b["rows"]) and np.array_equal(a["rows"], b["rows"])
                    and np.array_equal(a["cols"], b["cols"]))
    for k in VEC_KEYS + MAT_KEYS:
        if k in MAT_KEYS and not same_pattern:
            A, B = mat_dict(a, k), mat_dict(b, k)
            keys = sorted(set(A) | set(B))
            x = np.array([A.get(q, 0.0) for q in keys])
            y = np.array([B.get(q, 0.0) for q in keys])
        else:
            x, y = np.asarray(a[k], float), np.asarray(b[k], float)
        if y.size == 0:
            continue
        m = np.abs(y) > ATOL_FRAC * np.max(np.abs(y))
        if m.any():
            worst = max(worst, float(np.max(np.abs(x[m] - y[m]) / np.abs(y[m]))))
    return worst


def report(rec):
    """Append one JSON record to the file XG_PARITY_REPORT names, if set: the
    measured parity figures (largest errors, identical-entry counts)."""
    import json
    path = os.environ.get("XG_PARITY_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(rec) + "\n")


def _cmp(x, y):
    if x.size == 0:
        return (0, 0, 0.0)
    neq = int(np.sum(x != y))
    scale = RTOL * np.abs(y) + ATOL_FRAC * np.max(np.abs(y)) + 1e-300
    viol = float(np.max(np.abs(x - y) / scale))
    return (int(x.size), neq, viol)


def circuit_jacobian(netlist, seed=0, pdt=1e11, options=None):
    """The trapezoid-style Newton matrix dF/dx + pdt * dQ/dx of one transient
    load of `netlist` at a seeded random state, from the oracle (CSR, scipy)."""
    import scipy.sparse as sp

    from oracle.oracle import OracleCircuit
    from xyce_gb300 import engine, netlists
    opt = options or abi.device_options()
    params = {t: engine.setup_params(netlist, t, opt) for t in range(abi.NUM_DEV_TYPES)
              if netlist.count(t)}
    oc = OracleCircuit(netlist, params, opt)
    ins = netlists.random_state(oc.n_unknowns, oc.n_state, oc.n_store, seed=seed)
    out = oc.load(abi.load_flags(transient=1, newton_iter=1, pdt=pdt), *ins)
    n = oc.n_unknowns
    A = sp.csr_matrix((out["dFdx"] + pdt * out["dQdx"], (out["rows"], out["cols"])), shape=(n, n))
    A.sort_indices()
    return A


def oracle_transient_workload(name):
    """The oracle's CPU transient of one of bench.py's transient workloads
    (same netlist, start, window and recorded unknowns); returns (t, V,
    stats).  Runs in a spawned worker process."""
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    from oracle.oracle import OracleCircuit, transient
    from xyce_gb300 import engine
    nl, guess, tstop, tstep, uic, out = bench.build_tran(name)
    opt = abi.device_options()
    params = {t: engine.setup_params(nl, t, opt) for t in range(abi.NUM_DEV_TYPES) if nl.count(t)}
    oc = OracleCircuit(nl, params, opt)
    order, _ = engine.amd_order(oc.rowptr, oc.col)
    try:
        return transient(oc, tstop, tstep, out, col_order=order, x0=bench._x0(nl, guess), uic=uic)
    finally:
        oc.close()
