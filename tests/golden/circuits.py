"""Small seeded circuits for the golden fixtures and the parity tests.

Each entry builds a Netlist and lists the load sequence (solver flags) that
the fixture records.  The circuits cover every supported device (current
sources, DC and PULSE, in the mixed circuit), every
per-instance branch the flags reach (limiting on/off, dcop/initJct/transient,
newton_iter 0 / >0), internal nodes (RD, diode RS) and ground terminals.
"""
import numpy as np

from xyce_gb300 import abi, netlists


def mixed(seed=1):
    rng = np.random.default_rng(seed)
    nn = 30
    nl = abi.Netlist(nn)
    mn = nl.add_model(abi.Model(abi.DEV_MOS1, 1, VTO=0.7, KP=110e-6, LAMBDA=0.02, GAMMA=0.4,
                                CJ=2e-4, CJSW=1e-9, TOX=2e-8, CGSO=1e-10, CGDO=1e-10,
                                CGBO=1e-11, RD=10.0))
    mp = nl.add_model(abi.Model(abi.DEV_MOS1, -1, VTO=-0.7, KP=50e-6, LAMBDA=0.03, MJ=0.4,
                                CJ=2e-4, TOX=2e-8))
    m3 = nl.add_model(abi.Model(abi.DEV_MOS1, 1, VTO=0.5, KP=80e-6, JS=1e-6, CBD=1e-15,
                                CBS=2e-15, PB=0.7, RSH=20.0, NSUB=1e16, TOX=3e-8))
    dm = nl.add_model(abi.Model(abi.DEV_DIODE, 1, IS=1e-14, CJO=1e-12, BV=5.0, RS=2.0, TT=1e-9))
    dm2 = nl.add_model(abi.Model(abi.DEV_DIODE, 1, IS=2e-15, N=1.2, M=0.33))
    nm = 60
    nl.mos1 = dict(d=rng.integers(-1, nn, nm), g=rng.integers(-1, nn, nm),
                   s=rng.integers(-1, nn, nm), b=rng.integers(-1, nn, nm),
                   model=rng.integers(0, 3, nm), w=rng.uniform(1e-6, 1e-5, nm),
                   l=rng.uniform(1e-6, 2e-6, nm), ad=rng.uniform(1e-12, 1e-11, nm),
                   pd=rng.uniform(1e-6, 1e-5, nm))
    nl.mos1["as"] = rng.uniform(1e-12, 1e-11, nm)
    nl.mos1["ps"] = rng.uniform(1e-6, 1e-5, nm)
    nl.mos1["nrd"] = rng.uniform(0.5, 2, nm)
    nl.mos1["nrs"] = rng.uniform(0.5, 2, nm)
    nl.mos1["m"] = rng.integers(1, 3, nm).astype(float)
    nd = 12
    nl.diode = dict(a=rng.integers(-1, nn, nd), c=rng.integers(-1, nn, nd),
                    model=rng.choice([dm, dm2], nd), area=rng.uniform(0.5, 2, nd))
    nl.cap = dict(p=rng.integers(-1, nn, 10), m=rng.integers(-1, nn, 10),
                  value=rng.uniform(1e-15, 1e-13, 10))
    nl.res = dict(p=rng.integers(-1, nn, 10), m=rng.integers(-1, nn, 10),
                  value=rng.uniform(10, 1e4, 10))
    nl.vsrc = dict(p=[0, 1, 2], m=[-1, -1, 3], kind=[abi.SRC_DC, abi.SRC_PULSE, abi.SRC_PULSE],
                   wave=[[1.8, 0, 0, 0, 0, 0, 0], [0, 1.8, 1e-10, 1e-10, 1e-10, 9e-10, 2e-9],
                         [0.2, 1.2, 0, 5e-11, 2e-10, 3e-10, 1e-9]])
    nl.isrc = dict(p=[4, -1, 7, 9], m=[-1, 5, 8, 4],
                   kind=[abi.SRC_DC, abi.SRC_PULSE, abi.SRC_PULSE, abi.SRC_DC],
                   wave=[[1e-4, 0, 0, 0, 0, 0, 0], [0, 2e-3, 5e-11, 1e-10, 2e-10, 4e-10, 1.5e-9],
                         [-1e-3, 1e-3, 0, 3e-10, 1e-10, 2e-10, 0], [-5e-5, 0, 0, 0, 0, 0, 0]])
    nl.type_order = [abi.DEV_VSRC, abi.DEV_RES, abi.DEV_MOS1, abi.DEV_DIODE, abi.DEV_CAP,
                     abi.DEV_ISRC, abi.DEV_BSIM3]
    return nl


def bsim3(variant, seed=3):
    """BSIM3 (level 9) NMOS/PMOS pairs on a small random netlist.  Variant 0
    uses the default model cards; 1 and 2 walk the other mobility models,
    charge models, charge partitions, internal drain/source nodes and
    optional effects."""
    cards = [
        ({}, {}),
        (dict(CAPMOD=2, XPART=0.5, MOBMOD=2, RSH=5.0),
         dict(CAPMOD=0, XPART=0.0, NGATE=5e19, ALPHA0=1e-6)),
        (dict(CAPMOD=1, XPART=1.0, MOBMOD=3, IJTH=0.0, TOX=1e-8, K1=0.5, K2=0.01, LVTH0=1e-8,
              WU0=1e-9, PK3=1e-3),
         dict(CAPMOD=3, XPART=0.7, PSCBE2=0.0, A1=0.5, A2=0.5, DVT2=-0.1, KETA=-0.5,
              TNOM=40.0, LINT=1e-8, WINT=2e-8, CJSWG=2e-10)),
    ]
    n, cn, cp = cards[variant][0], cards[variant][1], None
    nl = netlists.random_mos_netlist(60, 20, dev_type=abi.DEV_BSIM3, seed=seed + variant,
                                     models=(abi.Model(abi.DEV_BSIM3, 1, **n),
                                             abi.Model(abi.DEV_BSIM3, -1, **cn)))
    rng = np.random.default_rng(seed)
    nl.bsim3["ad"] = rng.uniform(0, 2e-12, 60)
    nl.bsim3["as"] = rng.uniform(0, 2e-12, 60)
    nl.bsim3["pd"] = rng.uniform(0, 8e-6, 60)
    nl.bsim3["ps"] = rng.uniform(0, 8e-6, 60)
    nl.bsim3["m"] = rng.integers(1, 3, 60).astype(float)
    return nl


FLAG_SEQUENCE = [
    dict(dcop=1, transient=0, newton_iter=0, init_jct=1),
    dict(dcop=1, transient=0, newton_iter=1),
    dict(dcop=1, transient=0, newton_iter=2, init_fix=1),
    dict(tranop=1, transient=0, newton_iter=3),
    dict(transient=1, newton_iter=0, time=1.5e-10, pdt=1e11),
    dict(transient=1, newton_iter=1, time=3.0e-10, pdt=1e11),
    dict(transient=1, newton_iter=2, time=2.05e-9, pdt=2e11),
    dict(dcop=1, transient=0, newton_iter=1),
    dict(transient=1, newton_iter=0, init_tran=1, time=1e-12, pdt=1e12),
]

CIRCUITS = {
    "mixed": (mixed, abi.device_options()),
    "mixed_nolim": (mixed, abi.device_options(voltlim=0, gmin=1e-10, temp=320.0, tnom=300.15)),
    "inverter_chain_24": (lambda: netlists.inverter_chain(24), abi.device_options()),
    "power_grid_6x6": (lambda: netlists.power_grid(6, 6, 10, seed=3), abi.device_options()),
    "ring_7": (lambda: netlists.ring_oscillator(7, seed=5), abi.device_options()),
    "bsim3_default": (lambda: bsim3(0), abi.device_options()),
    "bsim3_cap2_mob2_rsh": (lambda: bsim3(1), abi.device_options()),
    "bsim3_cap13_bin_temp": (lambda: bsim3(2), abi.device_options(temp=320.0)),
}


def load_inputs(n_unknowns, n_state, n_store, seed):
    """Seeded inputs for one load in the sequence: voltages in [-0.5, 2.2] V
    so every region (cutoff, linear, saturation, reverse) is visited."""
    rng = np.random.default_rng(seed)
    sol = [np.r_[rng.uniform(-0.5, 2.2, n_unknowns), 0.0] for _ in range(3)]
    sta = [rng.uniform(-1e-13, 1e-13, n_state) for _ in range(3)]
    sto = [rng.uniform(-1.0, 2.2, n_store) for _ in range(3)]
    return sol, sta, sto
