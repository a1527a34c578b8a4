"""GPU parity tests of the Newton load through the C ABI.

  * against the golden fixtures the reference itself produced (exact build),
  * against the oracle on the same seeded inputs (exact and FMA builds),
  * run-to-run bitwise determinism, split vs fused entry points, call order,
  * the full-size single-load workload (1,000,000 MOSFETs on 250k nodes)
    against the oracle entry by entry.
"""
import numpy as np
import pytest

from helpers import Golden, compare, golden_files, max_rel_above_floor, report
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
    worst = 0.0
    for k, got in enumerate(outs):
        want = g.outputs(k)
        rep, bad = compare(got, want, exact=False)
        assert not bad, f"load {k}: {bad}"
        total += sum(v[0] for v in rep.values())
        ident += sum(v[0] - v[1] for v in rep.values())
        worst = max(worst, max_rel_above_floor(got, want))
    report({"test": "golden", "fixture": g.name, "entries": total, "bit_identical": ident,
            "max_rel_err_above_floor": worst})
    # the rest differ by CUDA's vs glibc's last-ulp exp/log/pow rounding;
    # measured at least 98.4% identical on every fixture
    assert ident / total > 0.98, f"only {ident}/{total} entries bit-identical"
    # entries above the absolute floor (no cancellation to near zero) are
    # within a few ulp: measured at most 3.7e-15 relative over the fixtures
    assert worst <= 1e-14, worst


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


@pytest.mark.parametrize("fma", [0, 1])
@pytest.mark.parametrize("variant", [0, 1, 2])
def test_gpu_bsim3_matches_oracle(variant, fma, gpu_ctx, oracle_lib):
    """BSIM3 variants (default cards; capMod 2 / mobMod 2 / RSH; capMod 1 and 3
    with binning and temperature) on 3,000 instances, the whole load
    sequence, against the oracle."""
    from golden import circuits
    nl = circuits.bsim3(variant, seed=40)
    nl = netlists.random_mos_netlist(3000, 700, dev_type=abi.DEV_BSIM3, seed=41 + variant,
                                     models=tuple(nl.models))
    opt = abi.device_options(fma=fma, temp=320.0 if variant == 2 else 300.15)
    params = {abi.DEV_BSIM3: engine.setup_params(nl, abi.DEV_BSIM3, opt)}
    oc = _oracle(nl, opt, params)
    loads = []
    for k, fl in enumerate(circuits.FLAG_SEQUENCE):
        flags = abi.load_flags(**{**dict(transient=0), **fl})
        loads.append((flags, circuits.load_inputs(oc.n_unknowns, oc.n_state, oc.n_store, seed=700 + k)))
    outs = _gpu_run(gpu_ctx, nl, opt, loads)
    for k, (flags, ins) in enumerate(loads):
        rep, bad = compare(outs[k], oc.load(flags, *ins), exact=False)
        assert not bad, (variant, fma, k, bad)


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


@pytest.mark.parametrize("fma", [0, 1])
def test_gpu_full_size_bsim3_single_load_matches_oracle(fma, gpu_ctx, oracle_lib):
    """1,000,000 BSIM3 instances (default level-9 model cards, half NMOS,
    half PMOS, W~U[0.2,10]um, L~U[0.1,1]um) on 250k random nodes, node
    voltages U[0,1.8] V, one transient Newton load, every output entry
    against the oracle: the bit-exact build and the FMA build (contracted
    products, shared reciprocals), both within the per-entry tolerance."""
    nl = netlists.random_mos_netlist(1_000_000, 250_000, dev_type=abi.DEV_BSIM3, seed=2,
                                     models=(abi.Model(abi.DEV_BSIM3, 1), abi.Model(abi.DEV_BSIM3, -1)))
    opt = abi.device_options(fma=fma)
    gpu_ctx.set_options(opt)
    c = engine.Circuit(gpu_ctx, nl)
    ins = netlists.random_state(c.n_unknowns, c.n_state, c.n_store, seed=9)
    flags = abi.load_flags(transient=1, newton_iter=1, time=0.0, pdt=1e11)
    c.set_state(*ins)
    c.load(flags)
    got = c.outputs()
    params = {abi.DEV_BSIM3: c.params(abi.DEV_BSIM3)}
    c.close()
    want = _oracle(nl, opt, params).load(flags, *ins)
    rep, bad = compare(got, want, exact=False)
    total = sum(v[0] for v in rep.values())
    ident = sum(v[0] - v[1] for v in rep.values())
    worst = max_rel_above_floor(got, want)
    report({"test": "bsim3_1M_single_load", "fma": fma, "entries": total, "bit_identical": ident,
            "max_violation": max(v[2] for v in rep.values()), "max_rel_err_above_floor": worst})
    assert not bad, bad
    if not fma:
        assert ident / total > 0.98, f"{ident}/{total} bit-identical"


def test_fast_reciprocal_within_two_ulp_of_ieee(engine_lib):
    """The FMA load build's reciprocal (Newton-Raphson from the hardware's
    approximation) against IEEE 1.0 / b: within 2 ulp on normal values over
    the whole fast range, the IEEE quotient itself outside it (zero,
    subnormal, huge, infinite, NaN)."""
    import ctypes as C
    rng = np.random.default_rng(3)
    n = 1 << 20
    b = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-1000, 1001, n)) * rng.choice([-1.0, 1.0], n)
    edge = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -1e-310, 2.0 ** -1000, 2.0 ** -1001,
                     2.0 ** 1000, 2.0 ** 1001, 1.7976931348623157e308, 1.0, 3.0, 0.1, -7.0])
    b = np.concatenate([b, edge])
    out = np.zeros_like(b)
    assert engine_lib.xg_probe_reciprocal(len(b), b.ctypes.data_as(C.c_void_p),
                                          out.ctypes.data_as(C.c_void_p)) == 0
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = 1.0 / b
    fin = np.isfinite(ref) & (ref != 0)
    ulps = np.abs(out[fin] - ref[fin]) / np.spacing(np.abs(ref[fin]))
    assert ulps.max() <= 2.0, ulps.max()
    special = ~fin
    assert np.array_equal(np.isnan(out[special]), np.isnan(ref[special]))
    ok = ~np.isnan(ref[special])
    assert np.array_equal(out[special][ok], ref[special][ok])
