"""GPU parity tests of the Newton load through the C ABI.

  * against the golden fixtures the reference itself produced (exact build),
  * against the oracle on the same seeded inputs (exact and FMA builds),
  * run-to-run bitwise determinism, split vs fused entry points, call order,
  * the full-size single-load workload (1,000,000 MOSFETs on 250k nodes)
    against the oracle entry by entry.
"""
import numpy as np
import pytest

from helpers import Golden, compare, golden_files
from xyce_gb300 import abi, engine, netlists

pytestmark = pytest.mark.gpu


def _gpu_run(ctx, netlist, options, loads):
    """loads: list of (flags, (sol, sta, sto)). Returns list of output dicts."""
    ctx.set_options(options)
    c = engine.Circuit(ctx, netlist)
    res = []
    for flags, ins in loads:
        c.set_state(*ins)
        c.load(flags)
        res.append(c.outputs())
    c.close()
    return res


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_gpu_matches_reference_golden(path, gpu_ctx):
    """Exact build against the reference's own outputs: identical except where
    CUDA's exp/log differ from glibc's by an ulp, then within the stated
    tolerance."""
    g = Golden(path)
    loads = [(g.flags(k), g.inputs(k)) for k in range(g.n_loads)]
    outs = _gpu_run(gpu_ctx, g.netlist, g.options, loads)
    total = ident = 0
    for k, got in enumerate(outs):
        rep, bad = compare(got, g.outputs(k), exact=False)
        assert not bad, f"load {k}: {bad}"
        total += sum(v[0] for v in rep.values())
        ident += sum(v[0] - v[1] for v in rep.values())
    assert ident / total > 0.99, f"only {ident}/{total} entries bit-identical"


def _oracle(netlist, options, ctx_params):
    from oracle.oracle import OracleCircuit
    return OracleCircuit(netlist, ctx_params, options)


@pytest.mark.parametrize("fma", [0, 1])
def test_gpu_matches_oracle_random(fma, gpu_ctx, oracle_lib):
    from golden import circuits
    from test_oracle_cpu import _random_mixed
    nl = _random_mixed(31, 20000, 5000)
    opt = abi.device_options(fma=fma)
    params = {t: engine.setup_params(nl, t, opt) for t in range(abi.NUM_DEV_TYPES) if nl.count(t)}
    oc = _oracle(nl, opt, params)
    loads = []
    for k, fl in enumerate(circuits.FLAG_SEQUENCE):
        flags = abi.load_flags(**{**dict(transient=0), **fl})
        loads.append((flags, circuits.load_inputs(oc.n_unknowns, oc.n_state, oc.n_store, seed=500 + k)))
    outs = _gpu_run(gpu_ctx, nl, opt, loads)
    for k, (flags, ins) in enumerate(loads):
        rep, bad = compare(outs[k], oc.load(flags, *ins), exact=False)
        assert not bad, (fma, k, bad)


def test_gpu_deterministic_and_split_equals_fused(gpu_ctx):
    """Three fresh circuits, same inputs: two fused loads and one split
    load give identical bits.  (Fresh circuits, because a diode carries its
    limited junction voltage from one load to the next, as the reference's
    Diode::Instance::Vd member does.)"""
    nl = netlists.power_grid(30, 30, 300, seed=7)
    gpu_ctx.set_options(abi.device_options())
    flags = abi.load_flags(transient=1, newton_iter=1, time=1.1e-9, pdt=1e11)
    res = []
    for mode in ("fused", "fused", "split"):
        c = engine.Circuit(gpu_ctx, nl)
        ins = netlists.random_state(c.n_unknowns, c.n_state, c.n_store, seed=3)
        c.set_state(*ins)
        if mode == "fused":
            c.load(flags)
        else:
            c.update_state(flags)
            c.load_dae_vectors()
            c.load_dae_matrices()
        res.append(c.outputs())
        c.close()
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k]), k
        assert np.array_equal(res[0][k], res[2][k]), k


def test_call_order_is_checked(gpu_ctx):
    gpu_ctx.set_options(abi.device_options())
    c = engine.Circuit(gpu_ctx, netlists.inverter_chain(4))
    with pytest.raises(engine.XgError) as e:
        c.load_dae_vectors()
    assert e.value.status == -7
    c.close()


def test_gpu_full_size_single_load_matches_oracle(gpu_ctx, oracle_lib):
    """1,000,000 level-1 MOSFETs on 250k random nodes, node voltages U[0,1.8],
    one transient Newton load: every entry of F, Q, dFdxdVp, dQdxdVp, the
    state/store vectors and both Jacobians against the oracle."""
    nl = netlists.random_mos_netlist(1_000_000, 250_000, seed=2)
    opt = abi.device_options()
    gpu_ctx.set_options(opt)
    c = engine.Circuit(gpu_ctx, nl)
    ins = netlists.random_state(c.n_unknowns, c.n_state, c.n_store, seed=9)
    flags = abi.load_flags(transient=1, newton_iter=1, time=0.0, pdt=1e11)
    c.set_state(*ins)
    c.load(flags)
    got = c.outputs()
    assert c.nnz > 10_000_000
    params = {abi.DEV_MOS1: c.params(abi.DEV_MOS1)}
    c.close()
    want = _oracle(nl, opt, params).load(flags, *ins)
    rep, bad = compare(got, want, exact=False)
    assert not bad, bad
    for k in ("F", "dFdx", "sto_next"):
        assert np.isfinite(got[k]).all()
