"""Seeded synthetic circuits with the shapes of the workloads the engine is
measured on.  No external netlists or datasets are used; every circuit is
built from a numpy seed.

  inverter_chain(stages)        1,000-stage CMOS inverter chain, MOSFET level 1
  random_mos_netlist(n_dev, ...) n MOSFETs (half NMOS, half PMOS) on a random
                                 node set, W~U[0.2,10]um, L~U[0.1,1]um, for a
                                 single Newton load with random node voltages
  power_grid(nx, ny, n_sinks)   resistive mesh with diode-clamped MOSFET sinks
                                 switched by PULSE sources
  ring_oscillator(stages, ...)  odd-stage CMOS ring, VTO/KP perturbed
"""
import numpy as np

from . import abi

# Level-1 model cards of the inverter-chain workload: NMOS VTO=0.7 KP=110u,
# PMOS VTO=-0.7 KP=50u (no TOX/CJ given: no gate or junction capacitance).
NMOS1 = dict(VTO=0.7, KP=110e-6)
PMOS1 = dict(VTO=-0.7, KP=50e-6)


def inverter_chain(stages=1000, cload=10e-15, vdd=1.8, tr=100e-12, per=2e-9):
    """Nodes: 0 vdd, 1 input, 2.. stage outputs.  PULSE 0->vdd, 50% duty."""
    n_nodes = stages + 2
    nl = abi.Netlist(n_nodes)
    mn = nl.add_model(abi.Model(abi.DEV_MOS1, 1, **NMOS1))
    mp = nl.add_model(abi.Model(abi.DEV_MOS1, -1, **PMOS1))
    ins = np.arange(1, stages + 1)
    outs = np.arange(2, stages + 2)
    gnd = np.full(stages, -1)
    vddn = np.zeros(stages, int)
    nl.mos1 = dict(d=np.r_[outs, outs], g=np.r_[ins, ins], s=np.r_[gnd, vddn], b=np.r_[gnd, vddn],
                   model=np.r_[np.full(stages, mn), np.full(stages, mp)],
                   w=np.r_[np.full(stages, 2e-6), np.full(stages, 4e-6)],
                   l=np.full(2 * stages, 1e-6))
    # interleave so instance order follows the chain: N0, P0, N1, P1, ...
    order = np.ravel(np.column_stack([np.arange(stages), np.arange(stages) + stages]))
    nl.mos1 = {k: np.asarray(v)[order] for k, v in nl.mos1.items()}
    nl.cap = dict(p=outs, m=gnd, value=np.full(stages, cload))
    pw = per / 2 - tr
    nl.vsrc = dict(p=[0, 1], m=[-1, -1], kind=[abi.SRC_DC, abi.SRC_PULSE],
                   wave=[[vdd, 0, 0, 0, 0, 0, 0], [0.0, vdd, 0.0, tr, tr, pw, per]])
    nl.type_order = [abi.DEV_VSRC, abi.DEV_MOS1, abi.DEV_CAP, abi.DEV_RES, abi.DEV_ISRC,
                     abi.DEV_DIODE, abi.DEV_BSIM3]
    return nl


def inverter_chain_nodeset(stages=1000, vdd=1.8):
    """Node-voltage guess (.NODESET) of the chain's DC state with the input
    low: supply high, input low, stage outputs alternating high/low."""
    v = np.zeros(stages + 2)
    v[0] = vdd
    v[2::2] = vdd
    return v


def random_mos_netlist(n_dev, n_nodes, dev_type=abi.DEV_MOS1, seed=0, models=None):
    """n_dev MOSFETs whose terminals are drawn uniformly from n_nodes nodes
    (about 4*n_dev/n_nodes attachments per node), first half NMOS, second half
    PMOS, W~U[0.2,10]um, L~U[0.1,1]um."""
    rng = np.random.default_rng(seed)
    nl = abi.Netlist(n_nodes)
    if models is None:
        models = (abi.Model(dev_type, 1, **NMOS1), abi.Model(dev_type, -1, **PMOS1))
    mn, mp = nl.add_model(models[0]), nl.add_model(models[1])
    term = rng.integers(0, n_nodes, size=(4, n_dev), dtype=np.int64)
    half = n_dev // 2
    d = dict(d=term[0], g=term[1], s=term[2], b=term[3],
             model=np.r_[np.full(half, mn), np.full(n_dev - half, mp)],
             w=rng.uniform(0.2e-6, 10e-6, n_dev), l=rng.uniform(0.1e-6, 1e-6, n_dev))
    if dev_type == abi.DEV_MOS1:
        nl.mos1 = d
    else:
        nl.bsim3 = d
    return nl


def power_grid(nx=200, ny=200, n_sinks=40000, seed=0, r_seg=0.1, c_node=1e-15, vdd=1.8):
    """nx*ny resistive mesh (r_seg per segment, c_node per node) fed by a DC
    supply at one corner; n_sinks level-1 NMOS current sinks from mesh nodes to
    ground, each gate driven by its own PULSE source (delay ~U[0,5ns]) and
    clamped to ground by a diode."""
    rng = np.random.default_rng(seed)
    n_mesh = nx * ny
    n_nodes = n_mesh + 1 + n_sinks          # mesh, supply pin, sink gates
    supply = n_mesh
    gates = n_mesh + 1 + np.arange(n_sinks)
    nl = abi.Netlist(n_nodes)
    mn = nl.add_model(abi.Model(abi.DEV_MOS1, 1, **NMOS1))
    dm = nl.add_model(abi.Model(abi.DEV_DIODE, 1, IS=1e-14))
    idx = np.arange(n_mesh).reshape(ny, nx)
    h = np.c_[idx[:, :-1].ravel(), idx[:, 1:].ravel()]
    v = np.c_[idx[:-1, :].ravel(), idx[1:, :].ravel()]
    seg = np.r_[h, v]
    nl.res = dict(p=np.r_[seg[:, 0], supply], m=np.r_[seg[:, 1], 0],
                  value=np.r_[np.full(len(seg), r_seg), r_seg])
    nl.cap = dict(p=np.arange(n_mesh), m=np.full(n_mesh, -1), value=np.full(n_mesh, c_node))
    sink_nodes = rng.choice(n_mesh, size=n_sinks, replace=n_sinks > n_mesh)
    nl.mos1 = dict(d=sink_nodes, g=gates, s=np.full(n_sinks, -1), b=np.full(n_sinks, -1),
                   model=np.full(n_sinks, mn), w=np.full(n_sinks, 2e-6), l=np.full(n_sinks, 1e-6))
    nl.diode = dict(a=np.full(n_sinks, -1), c=gates, model=np.full(n_sinks, dm))
    td = rng.uniform(0, 5e-9, n_sinks)
    wave = np.zeros((n_sinks + 1, 7))
    wave[0, 0] = vdd
    wave[1:, 1] = vdd
    wave[1:, 2] = td
    wave[1:, 3] = 100e-12
    wave[1:, 4] = 100e-12
    wave[1:, 5] = 0.9e-9
    wave[1:, 6] = 2e-9
    nl.vsrc = dict(p=np.r_[supply, gates], m=np.full(n_sinks + 1, -1),
                   kind=np.r_[abi.SRC_DC, np.full(n_sinks, abi.SRC_PULSE)], wave=wave)
    return nl


def power_grid_nodeset(nx=200, ny=200, n_sinks=40000, vdd=1.8):
    """Mesh and supply pin at the supply voltage, sink gates low."""
    return np.r_[np.full(nx * ny + 1, vdd), np.zeros(n_sinks)]


def ring_oscillator(stages=5, seed=0, sigma=0.10 / 3, cload=10e-15, vdd=1.8):
    """Odd-stage CMOS ring; each stage's VTO and KP scaled by (1+d), d~N(0,
    sigma) truncated at +-10% (a Monte-Carlo variant per seed)."""
    assert stages % 2 == 1
    rng = np.random.default_rng(seed)
    nl = abi.Netlist(stages + 1)          # 0 vdd, 1..stages ring nodes
    nodes = np.arange(1, stages + 1)
    nxt = np.roll(nodes, -1)
    dv = np.clip(rng.normal(0, sigma, (2, stages)), -0.1, 0.1)
    dk = np.clip(rng.normal(0, sigma, (2, stages)), -0.1, 0.1)
    # the cards per stage: NMOS then PMOS, each its own variant
    vto = np.ravel(np.column_stack([0.7 * (1 + dv[0]), -0.7 * (1 + dv[1])]))
    kp = np.ravel(np.column_stack([110e-6 * (1 + dk[0]), 50e-6 * (1 + dk[1])]))
    mods = nl.add_model(abi.ModelSet(abi.DEV_MOS1, np.tile([1, -1], stages), VTO=vto, KP=kp))
    d = np.repeat(nxt, 2)
    g = np.repeat(nodes, 2)
    s = np.ravel(np.column_stack([np.full(stages, -1), np.zeros(stages, int)]))
    nl.mos1 = dict(d=d, g=g, s=s, b=s.copy(), model=mods,
                   w=np.tile([2e-6, 4e-6], stages), l=np.full(2 * stages, 1e-6))
    nl.cap = dict(p=nodes, m=np.full(stages, -1), value=np.full(stages, cload))
    nl.vsrc = dict(p=[0], m=[-1], kind=[abi.SRC_DC], wave=[[vdd, 0, 0, 0, 0, 0, 0]])
    return nl


def ring_oscillator_nodeset(stages=5, vdd=1.8):
    """Initial condition that starts the ring: supply high, ring nodes
    alternating high/low (the odd ring breaks the pattern at one stage)."""
    v = np.zeros(stages + 1)
    v[0] = vdd
    v[1::2] = vdd
    return v


def random_logic(n_mos=500_000, seed=0, n_inputs=200, cwire=5e-15, vdd=1.8, wn=1e-6, wp=2e-6,
                 l=0.18e-6, period=(1e-9, 4e-9), tr=50e-12, window=64):
    """Seeded random combinational logic of 2-input NAND / NOR and inverters
    on BSIM3 (level-9 default cards, NMOS W=1u, PMOS W=2u, L=0.18u), built
    in topological order: every gate input is an earlier gate output or a
    primary input, each driver feeding 1-4 gate inputs (drawn uniformly)
    among the `window` most recent drivers with fan-out left (the locality of
    a placed design: uniform draws over all earlier gates make an expander
    graph whose LU fill grows quadratically: 51x the matrix at 50,000
    transistors, against 2.8x with a window of 32 and ~4x with 64); a 5 fF wire capacitance on every
    gate output; 200 primary inputs driven by PULSE sources of seeded delay,
    period and pulse width.

    Nodes: 0 supply, 1..n_inputs primary inputs, then per gate its output and,
    for NAND/NOR, the node between its two series transistors."""
    rng = np.random.default_rng(seed)
    kinds = []
    n = 0
    while n < n_mos:
        k = int(rng.integers(0, 3))          # 0 INV, 1 NAND2, 2 NOR2
        kinds.append(k)
        n += 2 if k == 0 else 4
    kinds = np.array(kinds)
    n_g = len(kinds)
    out_node = np.empty(n_g, np.int64)
    mid_node = np.full(n_g, -1, np.int64)
    nxt = 1 + n_inputs
    for g in range(n_g):
        out_node[g] = nxt
        nxt += 1
        if kinds[g] != 0:
            mid_node[g] = nxt
            nxt += 1
    n_nodes = nxt
    # drivers with remaining fan-out: primary inputs and gate outputs as they appear
    drivers = list(range(1, n_inputs + 1))
    budget = list(rng.integers(1, 5, n_inputs))
    ins = np.empty((n_g, 2), np.int64)
    for g in range(n_g):
        need = 1 if kinds[g] == 0 else 2
        for j in range(need):
            if not drivers:              # every driver used up: reuse a primary input
                drivers.append(int(rng.integers(1, n_inputs + 1)))
                budget.append(1)
            k = int(rng.integers(max(0, len(drivers) - window), len(drivers)))
            ins[g, j] = drivers[k]
            budget[k] -= 1
            if budget[k] == 0:
                del drivers[k]
                del budget[k]
        if need == 1:
            ins[g, 1] = ins[g, 0]
        drivers.append(int(out_node[g]))
        budget.append(int(rng.integers(1, 5)))
    d, gt, sr, bk, mdl, w = [], [], [], [], [], []
    nl = abi.Netlist(n_nodes)
    mn = nl.add_model(abi.Model(abi.DEV_BSIM3, 1))
    mp = nl.add_model(abi.Model(abi.DEV_BSIM3, -1))

    def fet(dd, gg, ss, pol):
        d.append(dd)
        gt.append(gg)
        sr.append(ss)
        bk.append(-1 if pol > 0 else 0)
        mdl.append(mn if pol > 0 else mp)
        w.append(wn if pol > 0 else wp)

    for g in range(n_g):
        o, a, b2, m = int(out_node[g]), int(ins[g, 0]), int(ins[g, 1]), int(mid_node[g])
        if kinds[g] == 0:                    # inverter
            fet(o, a, -1, 1)
            fet(o, a, 0, -1)
        elif kinds[g] == 1:                  # NAND2: series NMOS, parallel PMOS
            fet(o, a, m, 1)
            fet(m, b2, -1, 1)
            fet(o, a, 0, -1)
            fet(o, b2, 0, -1)
        else:                                # NOR2: parallel NMOS, series PMOS
            fet(o, a, -1, 1)
            fet(o, b2, -1, 1)
            fet(m, a, 0, -1)
            fet(o, b2, m, -1)
    nm = len(d)
    nl.bsim3 = dict(d=np.array(d), g=np.array(gt), s=np.array(sr), b=np.array(bk),
                    model=np.array(mdl), w=np.array(w), l=np.full(nm, l))
    nl.cap = dict(p=out_node, m=np.full(n_g, -1), value=np.full(n_g, cwire))
    per = rng.uniform(period[0], period[1], n_inputs)
    td = rng.uniform(0, per)
    pw = rng.uniform(0.2, 0.6, n_inputs) * per
    wave = np.zeros((n_inputs + 1, 7))
    wave[0, 0] = vdd
    wave[1:, 1] = vdd
    wave[1:, 2] = td
    wave[1:, 3] = tr
    wave[1:, 4] = tr
    wave[1:, 5] = pw
    wave[1:, 6] = per
    nl.vsrc = dict(p=np.r_[0, np.arange(1, n_inputs + 1)], m=np.full(n_inputs + 1, -1),
                   kind=np.r_[abi.SRC_DC, np.full(n_inputs, abi.SRC_PULSE)], wave=wave)
    nl.type_order = [abi.DEV_VSRC, abi.DEV_BSIM3, abi.DEV_CAP, abi.DEV_RES, abi.DEV_ISRC,
                     abi.DEV_DIODE, abi.DEV_MOS1]
    nl.logic = dict(kinds=kinds, ins=ins, out=out_node, mid=mid_node, n_inputs=n_inputs, vdd=vdd)
    return nl


def random_logic_nodeset(nl):
    """Node-voltage guess of random_logic's DC state: the gates evaluated in
    order with every primary input low (PULSE V1 = 0)."""
    lg = nl.logic
    vdd = lg["vdd"]
    v = np.zeros(nl.n_nodes)
    v[0] = vdd
    hi = np.zeros(nl.n_nodes, bool)
    for g in range(len(lg["kinds"])):
        a, b = hi[lg["ins"][g, 0]], hi[lg["ins"][g, 1]]
        k = lg["kinds"][g]
        o = (not a) if k == 0 else (not (a and b)) if k == 1 else (not (a or b))
        hi[lg["out"][g]] = o
        if k == 2:
            v[lg["mid"][g]] = vdd if not b else 0.0
    v[hi] = vdd
    return v


def random_state(n_unknowns, n_state, n_store, seed=0, vmax=1.8):
    """Node voltages i.i.d. U[0, vmax] (next/curr/last) and seeded state/store
    history: a second draw supplies the previous Newton iterate so the
    limiters take their limiting branches."""
    rng = np.random.default_rng(seed)
    sol = [np.r_[rng.uniform(0.0, vmax, n_unknowns), 0.0] for _ in range(3)]
    sta = [rng.uniform(0.0, 1e-14, n_state) for _ in range(3)]
    sto = [rng.uniform(-0.5, vmax, n_store) for _ in range(3)]
    return sol, sta, sto
