"""The CPU transient driver (oracle/xgo_tran.c), which checks the GPU time
stepper: pinned to closed-form solutions, then sanity of the reference's
benchmark circuits."""
import numpy as np
import pytest

from xyce_gb300 import abi, engine, netlists


def _oracle(nl, opt=None):
    from oracle.oracle import OracleCircuit
    opt = opt or abi.device_options()
    params = {t: engine.setup_params(nl, t, opt) for t in range(abi.NUM_DEV_TYPES) if nl.count(t)}
    return OracleCircuit(nl, params, opt)


def rc_lowpass(r=1e3, c=1e-12, td=0.1e-9, tr=1e-12, v2=1.0):
    """PULSE source -> R -> node 1 -> C -> ground."""
    nl = abi.Netlist(2)
    nl.res = dict(p=[0], m=[1], value=[r])
    nl.cap = dict(p=[1], m=[-1], value=[c])
    nl.vsrc = dict(p=[0], m=[-1], kind=[abi.SRC_PULSE], wave=[[0.0, v2, td, tr, tr, 50e-9, 0.0]])
    return nl


def rc_exact(t, r=1e3, c=1e-12, td=0.1e-9, tr=1e-12, v2=1.0):
    tau = r * c
    s = np.clip(t - td, 0, None)
    ramp = (s - tau * (1 - np.exp(-s / tau))) / tr
    after = 1 - (tau / tr) * (np.exp(tr / tau) - 1) * np.exp(-s / tau)
    return v2 * np.where(s <= tr, ramp, after)


def test_rc_step_response_matches_closed_form(oracle_lib):
    from oracle.oracle import transient
    nl = rc_lowpass()
    oc = _oracle(nl)
    t, v, st = transient(oc, 5e-9, 1e-12, [0, 1])
    assert st["status"] == 0 and st["steps"] > 20
    exact = rc_exact(t)
    # trapezoid with the local error test at reltol 1e-3: the global error
    # stays within a few reltol of the 1 V step
    assert np.abs(v[:, 1] - exact).max() < 1e-3
    assert abs(v[-1, 1] - exact[-1]) < 1e-3


def rc_current_driven(r=1e3, c=1e-12, td=0.1e-9, tr=1e-12, i2=1e-3):
    """PULSE current from ground into node 0, R and C from node 0 to ground:
    C dv/dt + v/R = I(t), the low-pass response to a step of I2*R volts."""
    nl = abi.Netlist(1)
    nl.res = dict(p=[0], m=[-1], value=[r])
    nl.cap = dict(p=[0], m=[-1], value=[c])
    nl.isrc = dict(p=[-1], m=[0], kind=[abi.SRC_PULSE], wave=[[0.0, i2, td, tr, tr, 50e-9, 0.0]])
    return nl


def test_current_source_rc_matches_closed_form(oracle_lib):
    from oracle.oracle import transient
    nl = rc_current_driven()
    t, v, st = transient(_oracle(nl), 5e-9, 1e-12, [0])
    assert st["status"] == 0 and st["steps"] > 20
    assert np.abs(v[:, 0] - rc_exact(t)).max() < 1e-3
    # the PULSE corners of a current source are breakpoints too
    for bp in (0.1e-9, 0.1e-9 + 1e-12):
        assert np.min(np.abs(t - bp)) < 1e-18


def test_breakpoints_are_hit(oracle_lib):
    from oracle.oracle import transient
    nl = rc_lowpass(td=0.3e-9, tr=50e-12)
    t, v, st = transient(_oracle(nl), 2e-9, 1e-12, [0, 1])
    for bp in (0.3e-9, 0.35e-9):
        assert np.min(np.abs(t - bp)) < 1e-18
    # the source node follows the PULSE exactly at its corners
    k = np.argmin(np.abs(t - 0.35e-9))
    assert abs(v[k, 0] - 1.0) < 1e-12


def test_inverter_chain_switches(oracle_lib):
    from oracle.oracle import transient
    stages = 20
    nl = netlists.inverter_chain(stages)
    oc = _oracle(nl)
    x0 = np.zeros(oc.n_unknowns)
    x0[:nl.n_nodes] = netlists.inverter_chain_nodeset(stages)
    order, _ = engine.amd_order(oc.rowptr, oc.col)
    t, v, st = transient(oc, 4e-9, 1e-12, [1, 2, 3], col_order=order, x0=x0)
    assert st["status"] == 0 and st["dcop_iters"] < 20
    # DC: input low, stage 1 high, stage 2 low
    assert abs(v[0, 0]) < 1e-9 and abs(v[0, 1] - 1.8) < 1e-6 and abs(v[0, 2]) < 1e-6
    # after the first input edge (0->1.8 over 0..100 ps) stage 1 falls, stage 2 rises
    k = np.searchsorted(t, 0.9e-9)
    assert v[k, 1] < 0.05 and v[k, 2] > 1.75


def test_gmin_stepping_fallback_finds_the_dc_point(oracle_lib):
    """Without a node-set guess the plain DC Newton fails on a chain (level-1
    devices with zero output conductance), and gmin stepping recovers."""
    from oracle.oracle import transient
    nl = netlists.inverter_chain(6)
    oc = _oracle(nl)
    t, v, st = transient(oc, 0.2e-9, 1e-12, [2, 3])
    assert st["status"] == 0
    assert abs(v[0, 0] - 1.8) < 1e-3 and abs(v[0, 1]) < 1e-3


def test_sparse_solve_matches_scipy(oracle_lib):
    import scipy.sparse.linalg as sla

    from helpers import circuit_jacobian
    from oracle.oracle import sparse_solve
    A = circuit_jacobian(netlists.power_grid(12, 12, 30, seed=2), seed=3)
    b = np.random.default_rng(0).standard_normal(A.shape[0])
    order, _ = engine.amd_order(A.indptr, A.indices)
    x = sparse_solve(A.indptr, A.indices, A.data, b, order)
    ref = sla.spsolve(A.tocsc(), b)
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()
