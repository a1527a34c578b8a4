"""The drop-in layer (integration/) driven on the GPU through
tests/integration_drive.cpp, with stand-ins shaped like Xyce's types:

  * GpuLoad::load fills F, Q, dF/dx and dQ/dx through vector[lid] and
    matrix[row][offset], equal to the oracle's load of the same circuit;
  * DirectSolver (behind N_LAS_XgSolver) solves circuit Jacobians to
    backward error 1e-13, reuses factors when asked, repivots when the kept
    pivot order meets a zero pivot, and returns a zero solution for a
    singular matrix, as the reference's Amesos solver does.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from helpers import Golden, compare, golden_files
from xyce_gb300 import abi, engine

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def drive(engine_lib, tmp_path_factory):
    libdir = os.path.dirname(engine.LIB_PATH)
    out = str(tmp_path_factory.mktemp("drive") / "libxg_drive.so")
    cmd = ["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "integration"), os.path.join(ROOT, "tests", "integration_drive.cpp"),
           "-o", out, "-L" + libdir, "-lxg", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    L = C.CDLL(out)
    vp, i = C.c_void_p, C.c_int
    L.drive_gpuload.argtypes = [C.POINTER(abi.XgNetlist), C.POINTER(abi.XgDeviceOptions), vp, vp,
                                vp, vp, vp, vp, vp]
    L.drive_direct_reset.argtypes = [i]
    L.drive_direct_solve.argtypes = [i, vp, vp, vp, vp, vp, i, C.POINTER(i), C.POINTER(i), C.POINTER(i)]
    yield L
    L.drive_direct_free()


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.mark.parametrize("name", ["mixed", "bsim3_default", "inverter_chain_24"])
def test_gpu_load_binding_matches_oracle(name, drive, oracle_lib):
    from oracle.oracle import OracleCircuit, all_params
    g = Golden([p for p in golden_files() if p.endswith(name + ".npz")][0])
    opt = g.options
    params = all_params(g.netlist, opt)
    for fl in (abi.load_flags(dcop=1, init_jct=1), abi.load_flags(transient=1, newton_iter=0, pdt=1e11,
                                                                   time=1e-9)):
        # a fresh circuit on both sides: no member carried from another load
        oc = OracleCircuit(g.netlist, params, opt)
        n = oc.n_unknowns
        sol = np.random.default_rng(5).uniform(0.0, 1.8, n + 1)
        sol[n] = 0.0
        zs, zt = np.zeros(max(1, oc.n_state)), np.zeros(max(1, oc.n_store))
        want = oc.load(fl, [sol, sol, sol], [zs, zs, zs], [zt, zt, zt])
        oc.close()
        F, Q = np.zeros(n), np.zeros(n)
        dF, dQ = np.zeros(max(1, oc.nnz)), np.zeros(max(1, oc.nnz))
        fi = np.array([fl.dcop, fl.tranop, fl.acop, fl.transient, fl.init_jct, fl.init_fix,
                       fl.newton_iter, fl.inputop, fl.init_tran], np.int32)
        fd = np.array([fl.pdt, fl.time])
        cnl = g.netlist.to_c()
        assert drive.drive_gpuload(C.byref(cnl), C.byref(opt), _p(fi), _p(fd), _p(sol), _p(F), _p(Q),
                                   _p(dF), _p(dQ)) == 0
        got = dict(want)
        got.update(F=F, Q=Q, dFdx=dF[:oc.nnz], dQdx=dQ[:oc.nnz])
        rep, bad = compare(got, want, exact=False)
        assert not bad, bad


def _solve(drive, A, b, reuse=False):
    x = np.zeros(A.shape[0])
    s, r, a = C.c_int(), C.c_int(), C.c_int()
    rp = np.ascontiguousarray(A.indptr, np.int32)
    ci = np.ascontiguousarray(A.indices, np.int32)
    v = np.ascontiguousarray(A.data, np.float64)
    rc = drive.drive_direct_solve(A.shape[0], _p(rp), _p(ci), _p(v), _p(b), _p(x), int(reuse),
                                  C.byref(s), C.byref(r), C.byref(a))
    return rc, x, s.value, r.value, a.value


def _berr(A, x, b):
    return np.abs(b - A @ x).max() / (abs(A).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())


@pytest.mark.parametrize("fp32", [0, 1])
def test_direct_solver_solves_reuses_and_refactors(fp32, drive, oracle_lib):
    from helpers import circuit_jacobian
    from xyce_gb300 import netlists
    nl = netlists.power_grid(30, 30, 300, seed=1)
    A0 = circuit_jacobian(nl, seed=4)
    A1 = circuit_jacobian(nl, seed=5)
    rng = np.random.default_rng(3)
    b0, b1 = rng.standard_normal(A0.shape[0]), rng.standard_normal(A0.shape[0])
    drive.drive_direct_reset(fp32)
    rc, x, sing, refac, an = _solve(drive, A0, b0)
    assert (rc, sing, refac, an) == (0, 0, 1, 1) and _berr(A0, x, b0) <= 1e-13
    rc, x, sing, refac, an = _solve(drive, A0, b1, reuse=True)  # same factors, new b
    assert (rc, sing, refac, an) == (0, 0, 0, 1) and _berr(A0, x, b1) <= 1e-13
    rc, x, sing, refac, an = _solve(drive, A1, b1)               # new values: refactor only
    assert (rc, sing, refac, an) == (0, 0, 1, 1) and _berr(A1, x, b1) <= 1e-13


def test_direct_solver_repivots_and_reports_singular(drive):
    import scipy.sparse as sp
    drive.drive_direct_reset(0)
    # the first matrix fixes a pivot order ...
    A = sp.csr_matrix(np.array([[4.0, 1.0, 0.0], [1.0, 4.0, 1.0], [0.0, 1.0, 4.0]]))
    b = np.array([1.0, 2.0, 3.0])
    rc, x, sing, refac, an = _solve(drive, A, b)
    assert rc == 0 and an == 1 and np.allclose(A @ x, b, rtol=0, atol=1e-14)
    # ... which meets a zero pivot on the next values: A with its first pivot
    # in that order (A[P[0], Q[0]], which no update reaches) set to zero,
    # nonsingular all the same; analysed again
    P, Q, _ = engine.lu_analyze_host(A.indptr, A.indices, A.data)
    Bd = A.toarray()
    Bd[P[0], Q[0]] = 0.0
    assert abs(np.linalg.det(Bd)) > 1.0
    B = sp.csr_matrix((Bd[A.nonzero()], A.indices, A.indptr), shape=(3, 3))
    rc, x, sing, refac, an = _solve(drive, B, b)
    assert (rc, sing, an) == (0, 0, 2) and np.allclose(B @ x, b, rtol=0, atol=1e-13)
    # a singular matrix: a zero solution and status 0 (the nonlinear solver decides)
    S = sp.csr_matrix((np.array([1.0, 1.0, 1.0, 1.0, 0.0, 0.0, 0.0]), A.indices, A.indptr), shape=(3, 3))
    rc, x, sing, refac, an = _solve(drive, S, b)
    assert rc == 0 and sing == 1 and not x.any()
