"""Host plans of the grid solves' special rows (lu_chain.h, no GPU).  A test
program (chain_plan_check.cpp, compiled here with the host analysis) plans
the chain of a circuit Jacobian's last rows and checks that every L and U
entry of the chain lands once, in its block's triangle or in one thread's
rounds in the solve's column order, and that the blocked solve, emulated
with the device kernel's order of fused multiply-adds, gives the same bits
as a column-by-column solve and agrees with a row-by-row solve to rounding.
It then picks the rows a block sums after the grid solves (solo_rows, with a
low length bar) and checks that a solve leaving them to the end never reads
one before it is computed and gives the same solution."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import circuit_jacobian
from xyce_gb300 import netlists

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "xyce_gb300", "csrc")
INCLUDE = os.path.join(HERE, "..", "include")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("chain") / "chain_plan_check")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I" + CSRC, "-I" + INCLUDE,
                        os.path.join(HERE, "chain_plan_check.cpp"), os.path.join(CSRC, "lu_symbolic.cpp"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def _write(A, path):
    with open(path, "wb") as f:
        np.array([A.shape[0], A.nnz], np.int64).tofile(f)
        A.indptr.astype(np.int32).tofile(f)
        A.indices.astype(np.int32).tofile(f)
        A.data.astype(np.float64).tofile(f)


@pytest.mark.parametrize("case,rows", [("grid", 256), ("grid", 768), ("grid", 1000), ("mos", 600)])
def test_chain_plan_places_every_entry_and_keeps_column_order(checker, tmp_path, case, rows):
    if case == "grid":
        A = circuit_jacobian(netlists.power_grid(60, 60, 1200, seed=1), seed=5)
    else:
        A = circuit_jacobian(netlists.random_mos_netlist(3000, 1000, seed=2), seed=3)
    path = str(tmp_path / "a.bin")
    _write(A.tocsr(), path)
    r = subprocess.run([checker, path, str(rows)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.split("\n")
    assert lines[0].startswith("solo rows:") and lines[1].startswith("ok"), r.stdout
    assert int(lines[0].split()[4]) > 0  # some upper rows deferred: the check is not vacuous
