"""CPU tests: the oracle against the golden fixtures made by the reference
itself, the engine's host setup against the reference's derived parameters,
and (where oracle/_ref is built) the oracle against the live reference on
further seeded circuits."""
import numpy as np
import pytest

from helpers import Golden, compare, golden_files
from xyce_gb300 import abi, engine, netlists


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_matches_reference_golden(path, oracle_lib):
    from oracle.oracle import OracleCircuit
    g = Golden(path)
    oc = OracleCircuit(g.netlist, g.full_params(), g.options)
    assert (oc.n_unknowns, oc.n_state, oc.n_store) == g.sizes
    for k in range(g.n_loads):
        got = oc.load(g.flags(k), *g.inputs(k))
        rep, bad = compare(got, g.outputs(k), exact=True)
        assert not bad, f"load {k}: {bad}"


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_setup_params_match_reference(path, engine_lib):
    """The engine's host setup reproduces the reference's derived instance
    parameters (bit for bit on x86-64; within 2 ulp where libm differs)."""
    g = Golden(path)
    for t, want in g.params.items():
        got = engine.setup_params(g.netlist, t, g.options)
        if t == abi.DEV_BSIM3:  # the fixture holds the raw columns only
            got = got[: want.shape[0]]
        assert got.shape == want.shape
        rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-300)
        assert np.all((got == want) | (rel <= 4.5e-16)), (t, np.argwhere(got != want)[:5])


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_setup_matches_reference(path, oracle_lib):
    """The oracle's own set-up reproduces the reference's derived instance
    parameters bit for bit."""
    from oracle import oracle
    g = Golden(path)
    for t, want in g.params.items():
        got = oracle.setup_params(g.netlist, t, g.options)
        if t == abi.DEV_BSIM3:  # the fixture holds the raw columns only
            got = got[: want.shape[0]]
        assert got.shape == want.shape
        assert np.array_equal(got, want), (t, np.argwhere(got != want)[:5])


def _bsim3_cards(seed, n, variant):
    from golden import circuits
    cards = circuits.bsim3(variant, seed=seed)
    nl = netlists.random_mos_netlist(n, n // 4, dev_type=abi.DEV_BSIM3, seed=seed,
                                     models=tuple(cards.models))
    rng = np.random.default_rng(seed)
    for k, hi in (("ad", 2e-12), ("as", 2e-12), ("pd", 8e-6), ("ps", 8e-6)):
        nl.bsim3[k] = rng.uniform(0, hi, n)
    nl.bsim3["m"] = rng.integers(1, 3, n).astype(float)
    return nl


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_oracle_setup_matches_engine_setup(variant, oracle_lib, engine_lib):
    """Oracle and engine set-up, two restatements of the reference's, give
    the same full parameter blocks (hoisted BSIM3 columns included) on random
    geometries of every device type."""
    from oracle import oracle
    nl = _random_mixed(40 + variant, 600, 150)
    b3 = _bsim3_cards(50 + variant, 800, variant)
    for net in (nl, b3):
        for t in range(abi.NUM_DEV_TYPES):
            if net.count(t):
                a = oracle.setup_params(net, t)
                b = engine.setup_params(net, t, abi.device_options())
                assert np.array_equal(a, b), (variant, t, np.argwhere(a != b)[:5])


def test_netlist_arrays_roundtrip():
    nl = netlists.power_grid(4, 4, 5, seed=1)
    back = abi.Netlist.from_arrays(nl.to_arrays())
    a, b = nl.to_arrays(), back.to_arrays()
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def _random_mixed(seed, n_mos, n_nodes):
    rng = np.random.default_rng(seed)
    nl = netlists.random_mos_netlist(n_mos, n_nodes, seed=seed)
    nl.models[0].params.update(LAMBDA=0.02, GAMMA=0.3, CJ=3e-4, TOX=2e-8, CGSO=2e-10)
    nl.models[1].params.update(LAMBDA=0.04, RD=5.0, RS=3.0, CJSW=1e-10, TOX=2e-8)
    nl.mos1["ad"] = rng.uniform(1e-12, 1e-11, n_mos)
    nl.mos1["as"] = rng.uniform(1e-12, 1e-11, n_mos)
    nl.mos1["pd"] = rng.uniform(1e-6, 1e-5, n_mos)
    nl.mos1["ps"] = rng.uniform(1e-6, 1e-5, n_mos)
    dm = nl.add_model(abi.Model(abi.DEV_DIODE, 1, IS=3e-14, CJO=2e-13, RS=1.0, BV=3.0))
    nd = n_mos // 4
    nl.diode = dict(a=rng.integers(-1, n_nodes, nd), c=rng.integers(-1, n_nodes, nd),
                    model=np.full(nd, dm), area=rng.uniform(0.5, 2, nd))
    nl.res = dict(p=rng.integers(-1, n_nodes, nd), m=rng.integers(-1, n_nodes, nd),
                  value=rng.uniform(1, 1e5, nd))
    nl.cap = dict(p=rng.integers(-1, n_nodes, nd), m=rng.integers(-1, n_nodes, nd),
                  value=rng.uniform(1e-16, 1e-12, nd))
    return nl


def test_oracle_matches_live_reference_random(oracle_lib, engine_lib):
    from oracle import ref
    if not ref.available():
        pytest.skip("oracle/_ref not built (needs the reference source tree)")
    from golden import circuits
    from oracle.oracle import OracleCircuit
    for seed in (21, 22):
        nl = _random_mixed(seed, 400, 120)
        opt = abi.device_options()
        rc = ref.RefCircuit(nl, opt)
        from oracle import oracle
        params = oracle.all_params(nl, opt)
        for t in (abi.DEV_MOS1, abi.DEV_DIODE, abi.DEV_RES, abi.DEV_CAP):
            assert np.array_equal(params[t], rc.params(t)), t
            assert np.array_equal(engine.setup_params(nl, t, opt), rc.params(t)), t
        oc = OracleCircuit(nl, params, opt)
        for k, fl in enumerate(circuits.FLAG_SEQUENCE):
            flags = abi.load_flags(**{**dict(transient=0), **fl})
            ins = circuits.load_inputs(rc.n_unknowns, rc.n_state, rc.n_store, seed=seed * 10 + k)
            rep, bad = compare(oc.load(flags, *ins), rc.load(flags, *ins), exact=True)
            assert not bad, (seed, k, bad)
