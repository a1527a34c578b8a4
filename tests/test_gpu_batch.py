"""Batched transients (the serving path): each request gives the same result
alone and inside a mix of uneven requests, to within the simulation's own
tolerance (reltol 1e-3 of the 1.8 V swing); the mix matches the CPU
transient driver; FP32 factors with FP64 refinement match FP64 factors; and
batches repeat bit for bit.  Requests whose level schedule fits in shared
memory use it (one block per request, level by level); the others are
walked row by row by one lane; both give the same waveforms."""
import numpy as np
import pytest

from xyce_gb300 import abi, engine, netlists

pytestmark = pytest.mark.gpu

VTOL = 1e-3 * 1.8
TSTOP = 1e-9


def _ring(stages, seed):
    nl = netlists.ring_oscillator(stages, seed=seed)
    x0 = np.zeros(nl.n_nodes + nl.count(abi.DEV_VSRC))
    x0[:nl.n_nodes] = netlists.ring_oscillator_nodeset(stages)
    return nl, x0, [1, 2, stages // 2 + 1]


MIX = [(5, 1), (11, 2), (51, 3), (101, 4), (31, 5)]


def _batch(ctx, reqs, precision=abi.LU_FP64, n_refine=0, tstop=TSTOP):
    nls, x0s, outs = zip(*reqs)
    b = engine.Batch(ctx, list(nls), list(x0s), [tstop] * len(reqs), list(outs), precision=precision,
                     n_refine=n_refine, max_points=8192)
    engine.run_batch(b)
    res = [b.results(i) for i in range(len(reqs))]
    b.close()
    return res


def _agree(a, b, same_steps=True):
    (ta, va, sa), (tb, vb, sb) = a, b
    assert sa["status"] == 0 and sb["status"] == 0
    if same_steps:
        assert abs(len(ta) - len(tb)) <= 0.02 * len(tb) + 2, (len(ta), len(tb))
    vi = np.stack([np.interp(tb, ta, va[:, k]) for k in range(va.shape[1])], 1)
    err = np.abs(vi - vb).max()
    assert err <= VTOL, err
    return err


def test_each_request_alone_and_in_the_mix(gpu_ctx):
    gpu_ctx.set_options(abi.device_options())
    reqs = [_ring(k, s) for k, s in MIX]
    mixed = _batch(gpu_ctx, reqs)
    for r, m in zip(reqs, mixed):
        alone = _batch(gpu_ctx, [r])[0]
        _agree(m, alone)
        assert abs(m[0][-1] - TSTOP) < 1e-18


def test_mix_matches_standalone_transient_and_oracle(gpu_ctx, oracle_lib):
    from oracle.oracle import OracleCircuit, transient
    gpu_ctx.set_options(abi.device_options())
    reqs = [_ring(k, s) for k, s in MIX[:3]]
    mixed = _batch(gpu_ctx, reqs)
    for (nl, x0, out), m in zip(reqs, mixed):
        c = engine.Circuit(gpu_ctx, nl)
        single = engine.transient(c, TSTOP, 1e-12, out, x0=x0, uic=True)
        c.close()
        _agree(m, single)
        opt = abi.device_options()
        params = {t: engine.setup_params(nl, t, opt) for t in range(abi.NUM_DEV_TYPES) if nl.count(t)}
        oc = OracleCircuit(nl, params, opt)
        order, _ = engine.amd_order(oc.rowptr, oc.col)
        cpu = transient(oc, TSTOP, 1e-12, out, col_order=order, x0=x0, uic=True)
        _agree(m, cpu)


def test_fp32_factors_with_refinement_match_fp64(gpu_ctx):
    gpu_ctx.set_options(abi.device_options())
    reqs = [_ring(k, s) for k, s in MIX]
    a = _batch(gpu_ctx, reqs)
    b = _batch(gpu_ctx, reqs, precision=abi.LU_FP32, n_refine=2)
    for x, y in zip(a, b):
        _agree(x, y)


def test_batches_repeat_bit_for_bit(gpu_ctx):
    gpu_ctx.set_options(abi.device_options())
    reqs = [_ring(k, s) for k, s in MIX[:3]]
    a = _batch(gpu_ctx, reqs)
    b = _batch(gpu_ctx, reqs)
    for x, y in zip(a, b):
        assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])


def test_level_schedule_and_row_walk_agree(gpu_ctx, monkeypatch):
    """XG_BATCH_NO_LVL sends every request to the row walk; the level-by-level
    kernel (nested-dissection order, a 128-thread block per request) gives the
    same waveforms; FP32 factors corrected by Newton alone agree too."""
    gpu_ctx.set_options(abi.device_options(fma=1))
    reqs = [_ring(k, s) for k, s in MIX]
    lvl = _batch(gpu_ctx, reqs)
    monkeypatch.setenv("XG_BATCH_NO_LVL", "1")
    walk = _batch(gpu_ctx, reqs)
    monkeypatch.delenv("XG_BATCH_NO_LVL")
    f32 = _batch(gpu_ctx, reqs, precision=abi.LU_FP32, n_refine=0)
    for a, b, c in zip(lvl, walk, f32):
        _agree(a, b)
        _agree(c, a)


def _chain(stages, tr, per):
    nl = netlists.inverter_chain(stages, tr=tr, per=per)
    x0 = np.zeros(nl.n_nodes + nl.count(abi.DEV_VSRC))
    x0[:nl.n_nodes] = netlists.inverter_chain_nodeset(stages)
    return nl, x0, [1, 2, stages + 1]


PULSED = [(5, 50e-12, 1e-9), (11, 100e-12, 2e-9), (21, 80e-12, 1.6e-9)]


def _corners(tr, per, tstop):
    """The PULSE corners of an inverter chain's input (td 0, tr = tf,
    pw = per / 2 - tr) inside (0, tstop)."""
    pw, out, k = per / 2 - tr, [], 0
    while per * k < tstop:
        base = per * k
        out += [t for t in (base, base + tr, base + tr + pw, base + 2 * tr + pw) if 0 < t < tstop]
        k += 1
    return out


@pytest.mark.parametrize("precision,n_refine", [(abi.LU_FP64, 0), (abi.LU_FP32, 0)])
def test_pulsed_requests_step_to_their_own_breakpoints(precision, n_refine, gpu_ctx):
    """Inverter chains with different PULSE edges and periods and an RC driven
    by a PULSE current, in one batch: every request lands on each of its own
    PULSE corners (and restarts there at first order), and its waveforms
    match the standalone transient from the same initial condition.  FP32
    factors corrected by Newton alone converge more slowly at the edges, so
    more Newton solves fail and those steps are retried smaller: the
    waveforms agree, the number of steps does not."""
    from test_tran_cpu import rc_current_driven
    gpu_ctx.set_options(abi.device_options(fma=1))
    tstop = 2e-9
    reqs = [_chain(*p) for p in PULSED]
    rc = rc_current_driven()
    rc.type_order = reqs[0][0].type_order  # one load order per batch
    reqs.append((rc, np.zeros(1), [0, 0, 0]))  # as many outputs as the others
    mixed = _batch(gpu_ctx, reqs, precision=precision, n_refine=n_refine, tstop=tstop)
    for (nl, x0, out), m in zip(reqs, mixed):
        c = engine.Circuit(gpu_ctx, nl)
        single = engine.transient(c, tstop, 1e-12, out, x0=x0, uic=True)
        c.close()
        _agree(m, single, same_steps=precision == abi.LU_FP64)
        assert abs(m[0][-1] - tstop) < 1e-18
    corners = [_corners(*p[1:], tstop) for p in PULSED] + [[0.1e-9, 0.1e-9 + 1e-12]]
    for bps, (t, _, _) in zip(corners, mixed):
        assert len(bps) >= 2
        for bp in bps:
            assert np.min(np.abs(t - bp)) < 1e-18, bp
