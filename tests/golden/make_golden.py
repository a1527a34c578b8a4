"""Generates the golden fixtures in this folder from the reference itself.

Runs the reference's own device code (oracle/_ref/libxyceref.so, built from
the reference sources by oracle/ref_build/build_ref.py) over each circuit in
circuits.py and its load sequence, and stores, per circuit, one .npz holding
the netlist, the reference's derived per-instance parameters, and for every
load the inputs and the reference's outputs.  Needs the reference source
tree (only present where the fixtures are generated); the tests only read
the .npz files.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from xyce_gb300 import abi  # noqa: E402
import circuits  # noqa: E402
from oracle import ref  # noqa: E402


def make(name, builder, opt):
    nl = builder()
    rc = ref.RefCircuit(nl, opt)
    out = {f"nl.{k}": v for k, v in nl.to_arrays().items()}
    out["opt"] = np.array([opt.gmin, opt.temp, opt.tnom, opt.voltlim, opt.newmeyer, opt.fma], float)
    for t in range(abi.NUM_DEV_TYPES):
        if nl.count(t):
            out[f"params.{t}"] = rc.params(t)
    out["sizes"] = np.array([rc.n_unknowns, rc.n_state, rc.n_store])
    for k, fl in enumerate(circuits.FLAG_SEQUENCE):
        flags = abi.load_flags(**{**dict(transient=0), **fl})
        sol, sta, sto = circuits.load_inputs(rc.n_unknowns, rc.n_state, rc.n_store, seed=100 + k)
        res = rc.load(flags, sol, sta, sto)
        out[f"load{k}.flags"] = np.array([flags.dcop, flags.tranop, flags.acop, flags.transient,
                                          flags.init_jct, flags.init_fix, flags.newton_iter,
                                          flags.inputop, flags.pdt, flags.time,
                                          flags.init_tran], float)
        for j, v in enumerate(sol):
            out[f"load{k}.sol{j}"] = v
        for j, v in enumerate(sta):
            out[f"load{k}.sta{j}"] = v
        for j, v in enumerate(sto):
            out[f"load{k}.sto{j}"] = v
        for key in ("F", "Q", "dFdxdVp", "dQdxdVp", "sta_next", "sto_next", "rows", "cols",
                    "dFdx", "dQdx"):
            out[f"load{k}.out.{key}"] = res[key]
    out["n_loads"] = np.array(len(circuits.FLAG_SEQUENCE))
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    rc.close()
    return path


def main():
    if not ref.available():
        print("oracle/_ref/libxyceref.so is not built; run oracle/ref_build/build_ref.py")
        return 1
    for name, (builder, opt) in circuits.CIRCUITS.items():
        print(make(name, builder, opt))
    return 0


if __name__ == "__main__":
    sys.exit(main())
