"""The GPU time stepper (xg_tran_run) against the CPU transient driver of the
oracle on the same netlists: DC operating point, trapezoid steps, Newton,
local error test and breakpoints.  The two follow the same algorithm, so they
take the same time points; node waveforms agree to within the simulation's
own tolerance (reltol 1e-3 of the 1.8 V swing), in practice to ~1e-15 V.
Also: the closed-form RC response, FP32 factors with refinement, and run-to-run
bitwise determinism."""
import numpy as np
import pytest

from xyce_gb300 import abi, engine, netlists

pytestmark = pytest.mark.gpu

VTOL = 1e-3 * 1.8


def _both(ctx, nl, x0, tstop, out, uic=False, precision=abi.LU_FP64, n_refine=0, fma=0):
    from oracle.oracle import OracleCircuit, transient
    opt = abi.device_options()
    params = {t: engine.setup_params(nl, t, opt) for t in range(abi.NUM_DEV_TYPES) if nl.count(t)}
    oc = OracleCircuit(nl, params, opt)
    order, _ = engine.amd_order(oc.rowptr, oc.col)
    xx = np.zeros(oc.n_unknowns)
    xx[:len(x0)] = x0
    tc, vc, sc = transient(oc, tstop, 1e-12, out, col_order=order, x0=xx, uic=uic)
    ctx.set_options(abi.device_options(fma=fma))
    c = engine.Circuit(ctx, nl)
    tg, vg, sg = engine.transient(c, tstop, 1e-12, out, x0=xx, uic=uic, precision=precision,
                                  n_refine=n_refine)
    c.close()
    return (tc, vc, sc), (tg, vg, sg)


def _agree(cpu, gpu):
    (tc, vc, sc), (tg, vg, sg) = cpu, gpu
    assert sc["status"] == 0 and sg["status"] == 0
    assert abs(len(tg) - len(tc)) <= 0.02 * len(tc) + 2, (len(tg), len(tc))
    vi = np.stack([np.interp(tc, tg, vg[:, k]) for k in range(vg.shape[1])], 1)
    err = np.abs(vi - vc).max()
    assert err <= VTOL, err
    return err


@pytest.mark.parametrize("precision,n_refine,fma", [(abi.LU_FP64, 0, 0), (abi.LU_FP32, 2, 0),
                                                    (abi.LU_FP64, 0, 1), (abi.LU_FP32, 0, 1)])
def test_inverter_chain_waveforms(precision, n_refine, fma, gpu_ctx, oracle_lib):
    """fma=1: the FMA load build, whose supply-rail sums (one term per
    device) are split over a block; FP32 factors with no extra refinement
    rely on Newton's FP64 residual alone."""
    stages = 100
    cpu, gpu = _both(gpu_ctx, netlists.inverter_chain(stages), netlists.inverter_chain_nodeset(stages),
                     4e-9, [1, 2, 3, 50, stages + 1], precision=precision, n_refine=n_refine, fma=fma)
    _agree(cpu, gpu)
    assert gpu[2]["newton_iters"] > 300


def test_power_grid_waveforms(gpu_ctx, oracle_lib):
    cpu, gpu = _both(gpu_ctx, netlists.power_grid(20, 20, 60, seed=1),
                     netlists.power_grid_nodeset(20, 20, 60), 2e-9, [0, 10, 200, 399])
    _agree(cpu, gpu)


def test_ring_oscillator_from_initial_condition(gpu_ctx, oracle_lib):
    cpu, gpu = _both(gpu_ctx, netlists.ring_oscillator(11, seed=3), netlists.ring_oscillator_nodeset(11),
                     2e-9, [1, 2, 6, 11], uic=True)
    _agree(cpu, gpu)
    # it oscillates: every ring node crosses mid-rail
    v = gpu[1]
    assert ((v > 1.6).any(axis=0) & (v < 0.2).any(axis=0)).all()


def test_rc_closed_form(gpu_ctx):
    from test_tran_cpu import rc_exact, rc_lowpass
    gpu_ctx.set_options(abi.device_options())
    c = engine.Circuit(gpu_ctx, rc_lowpass())
    t, v, st = engine.transient(c, 5e-9, 1e-12, [0, 1])
    c.close()
    assert np.abs(v[:, 1] - rc_exact(t)).max() < 1e-3


def test_current_source_rc(gpu_ctx, oracle_lib):
    """PULSE current source into an RC: closed form, and the oracle's steps."""
    from test_tran_cpu import rc_current_driven, rc_exact
    cpu, gpu = _both(gpu_ctx, rc_current_driven(), np.zeros(1), 5e-9, [0])
    _agree(cpu, gpu)
    t, v, _ = gpu
    assert np.abs(v[:, 0] - rc_exact(t)).max() < 1e-3


def test_transient_is_deterministic(gpu_ctx):
    nl = netlists.inverter_chain(40)
    x0 = netlists.inverter_chain_nodeset(40)
    gpu_ctx.set_options(abi.device_options())
    runs = []
    for _ in range(2):
        c = engine.Circuit(gpu_ctx, nl)
        runs.append(engine.transient(c, 2e-9, 1e-12, [2, 20, 41], x0=np.r_[x0, 0.0, 0.0]))
        c.close()
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


def test_random_logic_bsim3_waveforms(gpu_ctx, oracle_lib):
    """2,000 BSIM3 MOSFETs of seeded random NAND/NOR/INV logic, from its
    logic state, 20 ps: the BSIM3 load inside the time loop."""
    nl = netlists.random_logic(2000, seed=0)
    o = nl.logic["out"]
    cpu, gpu = _both(gpu_ctx, nl, netlists.random_logic_nodeset(nl), 20e-12,
                     [1, int(o[len(o) // 2]), int(o[-1])], uic=True)
    _agree(cpu, gpu)


def test_second_transient_on_a_circuit_reuses_the_lu_analysis(gpu_ctx):
    """The first transient leaves its LU analysis with the circuit; a second
    one from the same start takes it back (no analysis) and gives the same
    bits; a different start analyses afresh."""
    nl = netlists.inverter_chain(40)
    x0 = np.r_[netlists.inverter_chain_nodeset(40), 0.0, 0.0]
    gpu_ctx.set_options(abi.device_options())
    c = engine.Circuit(gpu_ctx, nl)
    a = engine.transient(c, 1e-9, 1e-12, [2, 20, 41], x0=x0)
    b = engine.transient(c, 1e-9, 1e-12, [2, 20, 41], x0=x0)
    d = engine.transient(c, 1e-9, 1e-12, [2, 20, 41], x0=x0 * 0.5)
    c.close()
    assert a[2]["analyses"] >= 1 and b[2]["analyses"] == 0 and d[2]["analyses"] >= 1
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
