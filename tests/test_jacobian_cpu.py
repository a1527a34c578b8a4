"""Numerical-Jacobian check of the oracle's matrix loads, after the
reference's device Jacobian test (N_DEV_NumericalJacobian.C:295-500): each
unknown is perturbed by dx = sqrtEta (1 + |x|), F and Q are reloaded, and the
forward difference is compared with the loaded dF/dx and dQ/dx entry by entry,

    |analytic - numeric| <= relTol |numeric| + absTol,

with the reference's defaults relTol 0.01, absTol 1e-8, sqrtEta 1e-8
(testJac_*, N_DEV_DeviceOptions.C:95-97).  Here the whole circuit is
perturbed at once, so a column collects every device's contribution, and
entries outside the matrix pattern are checked too (a numeric derivative
there would be a missing stamp).  absTol for dQ/dx is scaled to charges
(1e-20 C/V).

The loads are transient Newton loads with voltage limiting off, where F and Q
are smooth functions of the solution, at physical biases: MOSFET bulks on the
rails, terminals within them, diodes between 1 V reverse and 0.65 V forward.
(At a 2 V forward junction the exponential makes F ~1e20 and its rounding
swamps any difference quotient.)  Level-1 MOSFETs keep their Meyer gate
charges incrementally (qgs = qgs_old + C (vgs - vgs_old),
N_DEV_MOSFET1.C:2530-2560), so their dQ/dx is C, not the derivative of that
charge; dQ/dx is checked on the circuits without them.

The GPU load is bit-identical to the oracle on the same inputs (the parity
tests), so this pins the GPU matrices too.
"""
import numpy as np
import pytest

from xyce_gb300 import abi, engine, netlists

REL_TOL, ABS_TOL_F, ABS_TOL_Q, SQRT_ETA = 0.01, 1e-8, 1e-20, 1e-8

MOS1_CARDS = [
    (1, dict(VTO=0.7, KP=110e-6, LAMBDA=0.02, GAMMA=0.4, CJ=2e-4, CJSW=1e-9, TOX=2e-8,
             CGSO=1e-10, CGDO=1e-10, CGBO=1e-11, RD=10.0)),
    (-1, dict(VTO=-0.7, KP=50e-6, LAMBDA=0.03, MJ=0.4, CJ=2e-4, TOX=2e-8)),
    (1, dict(VTO=0.5, KP=80e-6, JS=1e-6, CBD=1e-15, CBS=2e-15, PB=0.7, RSH=20.0, NSUB=1e16,
             TOX=3e-8)),
]
BSIM3_CARDS = {
    "default": [(1, {}), (-1, {})],
    "cap2_mob2_rsh": [(1, dict(CAPMOD=2, XPART=0.5, MOBMOD=2, RSH=5.0)),
                      (-1, dict(CAPMOD=0, XPART=0.0, NGATE=5e19, ALPHA0=1e-6))],
    "cap13_bin": [(1, dict(CAPMOD=1, XPART=1.0, MOBMOD=3, IJTH=0.0, TOX=1e-8, K1=0.5, K2=0.01,
                           LVTH0=1e-8, WU0=1e-9, PK3=1e-3)),
                  (-1, dict(CAPMOD=3, XPART=0.7, PSCBE2=0.0, A1=0.5, A2=0.5, DVT2=-0.1, KETA=-0.5,
                            TNOM=40.0, LINT=1e-8, WINT=2e-8, CJSWG=2e-10))],
}
VDD = 1.8


def structured(dev_type, cards, seed=0, n_logic=16, n_mos=24, n_diode=4):
    """Node 0 is the upper rail; nodes 1..n_logic-1 carry MOSFET terminals
    (bulks on the rail of their polarity); the next n_diode nodes are diode
    anodes (cathodes at ground, the first half with series resistance, so
    their internal nodes are the first internal unknowns).  Resistors,
    capacitors, DC and PULSE voltage and current sources join the logic
    nodes."""
    rng = np.random.default_rng(seed)
    nl = abi.Netlist(n_logic + n_diode)
    anodes = n_logic + np.arange(n_diode)
    if dev_type is not None:
        ms = [nl.add_model(abi.Model(dev_type, pol, **card)) for pol, card in cards]
        pol = np.array([pol for pol, _ in cards])
        k = rng.integers(0, len(ms), n_mos)
        d = dict(d=rng.integers(1, n_logic, n_mos), g=rng.integers(1, n_logic, n_mos),
                 s=rng.integers(1, n_logic, n_mos), b=np.where(pol[k] > 0, -1, 0),
                 model=np.array(ms)[k], w=rng.uniform(1e-6, 1e-5, n_mos),
                 l=rng.uniform(0.2e-6, 2e-6, n_mos), ad=rng.uniform(1e-12, 1e-11, n_mos),
                 pd=rng.uniform(1e-6, 1e-5, n_mos), nrd=rng.uniform(0.5, 2, n_mos),
                 nrs=rng.uniform(0.5, 2, n_mos), m=rng.integers(1, 3, n_mos).astype(float))
        d["as"] = rng.uniform(1e-12, 1e-11, n_mos)
        d["ps"] = rng.uniform(1e-6, 1e-5, n_mos)
        setattr(nl, "mos1" if dev_type == abi.DEV_MOS1 else "bsim3", d)
    drs = nl.add_model(abi.Model(abi.DEV_DIODE, 1, IS=1e-14, CJO=1e-12, BV=5.0, RS=2.0, TT=1e-9))
    dnr = nl.add_model(abi.Model(abi.DEV_DIODE, 1, IS=2e-15, N=1.2, M=0.33, CJO=5e-13))
    half = n_diode // 2
    nl.diode = dict(a=anodes, c=np.full(n_diode, -1), area=rng.uniform(0.5, 2, n_diode),
                    model=np.r_[np.full(half, drs), np.full(n_diode - half, dnr)])
    nr = 8
    nl.res = dict(p=rng.integers(0, n_logic, nr), m=rng.integers(-1, n_logic, nr),
                  value=rng.uniform(100, 1e4, nr))
    nl.cap = dict(p=rng.integers(0, n_logic, nr), m=rng.integers(-1, n_logic, nr),
                  value=rng.uniform(1e-15, 1e-13, nr))
    nl.vsrc = dict(p=[0, 3], m=[-1, 4], kind=[abi.SRC_DC, abi.SRC_PULSE],
                   wave=[[VDD, 0, 0, 0, 0, 0, 0], [0, 1.0, 1e-10, 1e-10, 1e-10, 5e-10, 2e-9]])
    nl.isrc = dict(p=[5, -1], m=[-1, 6], kind=[abi.SRC_DC, abi.SRC_PULSE],
                   wave=[[1e-4, 0, 0, 0, 0, 0, 0], [0, 2e-4, 1e-10, 1e-10, 1e-10, 5e-10, 0]])
    nl.type_order = [abi.DEV_DIODE, abi.DEV_VSRC, abi.DEV_ISRC, abi.DEV_RES, abi.DEV_CAP,
                     abi.DEV_MOS1, abi.DEV_BSIM3]
    return nl, np.r_[anodes, nl.n_nodes + np.arange(half)]


def _check(nl, diode_unknowns, check_q, seed=7, vrange=(0.0, VDD), opt=None):
    from oracle.oracle import OracleCircuit
    opt = opt or abi.device_options(voltlim=0)
    params = {t: engine.setup_params(nl, t, opt) for t in range(abi.NUM_DEV_TYPES) if nl.count(t)}
    oc = OracleCircuit(nl, params, opt)
    n = oc.n_unknowns
    rng = np.random.default_rng(seed)

    def state():
        v = rng.uniform(*vrange, n)
        v[0] = VDD
        v[diode_unknowns] = rng.uniform(-1.0, 0.65, len(diode_unknowns))
        return np.r_[v, 0.0]

    sol = [state() for _ in range(3)]
    sta = [rng.uniform(-1e-13, 1e-13, oc.n_state) for _ in range(3)]
    sto = [rng.uniform(-1.0, 2.2, oc.n_store) for _ in range(3)]
    flags = abi.load_flags(transient=1, newton_iter=2, pdt=1e11, time=3e-10)
    base = oc.load(flags, sol, sta, sto)
    checks = [("dFdx", "F", ABS_TOL_F)] + ([("dQdx", "Q", ABS_TOL_Q)] if check_q else [])
    J = {}
    for key, _, _ in checks:
        J[key] = np.zeros((n, n))
        np.add.at(J[key], (base["rows"], base["cols"]), base[key])
    worst = {key: 0.0 for key, _, _ in checks}
    for j in range(n):
        dx = SQRT_ETA * (1.0 + abs(sol[0][j]))
        pert = [s.copy() for s in sol]
        pert[0][j] += dx
        out = oc.load(flags, pert, sta, sto)
        for key, vec, atol in checks:
            num = (out[vec] - base[vec]) / dx
            ana = J[key][:, j]
            err = np.abs(ana - num) / (REL_TOL * np.abs(num) + atol)
            worst[key] = max(worst[key], float(err.max()))
            bad = np.flatnonzero(err > 1.0)
            assert bad.size == 0, (key, j, [(int(r), ana[r], num[r]) for r in bad[:4]])
    return worst


def test_mos1_circuit_dfdx(oracle_lib):
    nl, du = structured(abi.DEV_MOS1, MOS1_CARDS)
    _check(nl, du, check_q=False)


@pytest.mark.parametrize("cards", sorted(BSIM3_CARDS))
def test_bsim3_circuit_dfdx_and_dqdx(cards, oracle_lib):
    nl, du = structured(abi.DEV_BSIM3, BSIM3_CARDS[cards], seed=1)
    _check(nl, du, check_q=True)


def test_passive_source_diode_circuit_at_temperature(oracle_lib):
    nl, du = structured(None, None, seed=2)
    _check(nl, du, check_q=True, opt=abi.device_options(voltlim=0, temp=350.0, gmin=1e-10))


@pytest.mark.parametrize("name", ["inverter_chain", "ring_oscillator", "power_grid"])
def test_benchmark_circuits_dfdx(name, oracle_lib):
    nl = {"inverter_chain": lambda: netlists.inverter_chain(12),
          "ring_oscillator": lambda: netlists.ring_oscillator(7, seed=5),
          "power_grid": lambda: netlists.power_grid(4, 4, 6, seed=3)}[name]()
    _check(nl, np.zeros(0, int), check_q=False)
