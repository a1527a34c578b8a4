"""SPICE netlist front end: text -> xg_netlist (abi.Netlist) plus the .TRAN
analysis, its options and the requested outputs.

It follows the reference's reading of a netlist (the circuit block's line
handling, src/IOInterfacePKG/src/N_IO_CircuitBlock.C:798-1006, and
DeviceMgr::addDeviceInstance, src/DeviceModelPKG/Core/src/N_DEV_DeviceMgr.C:1075)
for the devices this library evaluates:

  * the first line is the title; '*' lines are comments, ';' starts an
    inline comment, '+' continues the previous line; case does not matter;
  * numbers take the SPICE scale suffixes (T G MEG K MIL M U N P F, any unit
    letters after them ignored), the value multiplied by the scale as the
    reference does (N_UTL_Misc.C);
  * node 0 is ground; every other node name is a node, numbered in order of
    first appearance;
  * R, C, V, I (DC value, or PULSE(V1 V2 TD TR TF PW PER) with the reference's
    defaults for omitted values: TD 0, TR and TF the .TRAN step, PW and PER
    the .TRAN stop time, PulseData::initializeSource,
    src/DeviceModelPKG/Core/src/N_DEV_SourceData.C:905-918), D (model,
    optional area) and M (d g s b model, W L AD AS PD PS NRD NRS M);
  * .MODEL name D | NMOS | PMOS (LEVEL 1: MOSFET level 1; LEVEL 9 or 49:
    BSIM3 v3.2) with its parameters; the device set-up checks them, and
    refuses what the reference refuses (a level-1 diode given level-2
    parameters, N_DEV_Diode.C:1879-1907) or what this library does not
    evaluate;
  * .TRAN tstep tstop [tstart [tmax]] [UIC], .OPTIONS TIMEINT RELTOL ABSTOL
    (other option blocks are read and ignored), .PRINT TRAN V(node)...,
    .END.

Anything else (subcircuits, other device letters, other source shapes,
expressions) is refused with the line it stands on.
"""
import re

import numpy as np

from . import abi

_SCALE = [("MEG", 1e6), ("MIL", 25.4e-6), ("T", 1e12), ("G", 1e9), ("K", 1e3), ("M", 1e-3),
          ("U", 1e-6), ("N", 1e-9), ("P", 1e-12), ("F", 1e-15)]
_NUM = re.compile(r"^([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)([A-Za-z]*)$")


class ParseError(ValueError):
    def __init__(self, line_no, line, msg):
        super().__init__(f"line {line_no}: {msg}: {line.strip()}")
        self.line_no = line_no


def spice_number(tok):
    """A SPICE number: 1k, 10pF, 2.5meg, 1e-3, 25mil."""
    m = _NUM.match(tok.strip())
    if not m:
        raise ValueError(f"not a number: {tok!r}")
    v = float(m.group(1))
    suf = m.group(2).upper()
    for s, f in _SCALE:
        if suf.startswith(s):
            return v * f
    return v


class ParsedCircuit:
    """The parsed netlist and its analysis: netlist (abi.Netlist), node_names
    (index -> name), tran {tstep, tstop, tstart, tmax, uic} or None,
    options {reltol, abstol}, outputs [(label, unknown index)]."""

    def __init__(self):
        self.title = ""
        self.netlist = None
        self.node_names = []
        self.tran = None
        self.options = {"reltol": 1e-3, "abstol": 1e-6}
        self.outputs = []

    @property
    def out_idx(self):
        return [k for _, k in self.outputs]


def _logical_lines(text):
    """(line number, text) of each logical line: title dropped, comments
    stripped, continuations joined."""
    out = []
    lines = text.splitlines()
    for no, raw in enumerate(lines[1:], start=2):
        s = raw.split(";")[0].rstrip()
        if not s.strip() or s.lstrip().startswith("*"):
            continue
        if s.lstrip().startswith("+"):
            if not out:
                raise ParseError(no, raw, "continuation without a line to continue")
            out[-1] = (out[-1][0], out[-1][1] + " " + s.lstrip()[1:])
        else:
            out.append((no, s.strip()))
    return lines[0].strip() if lines else "", out


def _tokens(s):
    # parentheses, '=' and ',' separate tokens; keep '=' to pair names and values
    return re.sub(r"([()=,])", r" \1 ", s).split()


def _pairs(toks, no, line):
    """NAME = value pairs (in any order), values as numbers."""
    out = {}
    toks = [t for t in toks if t not in ("(", ")", ",")]
    k = 0
    while k < len(toks):
        if k + 1 >= len(toks) or toks[k + 1] != "=":
            raise ParseError(no, line, f"expected NAME=value, found {toks[k]!r}")
        if k + 2 >= len(toks):
            raise ParseError(no, line, f"no value for {toks[k]}")
        try:
            out[toks[k].upper()] = spice_number(toks[k + 2])
        except ValueError:
            raise ParseError(no, line, f"bad value for {toks[k]}") from None
        k += 3
    return out


def parse_netlist(text):
    """Parse SPICE text into a ParsedCircuit (ParseError on what it cannot
    read or this library does not support)."""
    pc = ParsedCircuit()
    pc.title, lines = _logical_lines(text)
    nodes = {}

    def node(name):
        n = name.upper()
        if n == "0":
            return -1
        if n not in nodes:
            nodes[n] = len(nodes)
            pc.node_names.append(name)
        return nodes[n]

    models = {}          # name -> (dev_type, polarity, params)
    elems = []           # (letter, no, line, tokens)
    prints = []
    for no, line in lines:
        toks = _tokens(line)
        head = toks[0].upper()
        if head == ".END":
            break
        if head.startswith("."):
            if head == ".MODEL":
                if len(toks) < 3:
                    raise ParseError(no, line, ".MODEL needs a name and a type")
                kind = toks[2].upper()
                params = _pairs(toks[3:], no, line)
                if kind == "D":
                    models[toks[1].upper()] = (abi.DEV_DIODE, 1, params)
                elif kind in ("NMOS", "PMOS"):
                    level = int(params.pop("LEVEL", 1))
                    if level == 1:
                        t = abi.DEV_MOS1
                    elif level in (9, 49):
                        t = abi.DEV_BSIM3
                    else:
                        raise ParseError(no, line, f"MOSFET level {level} is not supported")
                    models[toks[1].upper()] = (t, 1 if kind == "NMOS" else -1, params)
                else:
                    raise ParseError(no, line, f"model type {kind} is not supported")
            elif head == ".TRAN":
                rest = [t for t in toks[1:] if t.upper() != "UIC"]
                try:
                    vals = [spice_number(t) for t in rest]
                except ValueError:
                    raise ParseError(no, line, "bad .TRAN value") from None
                if len(vals) < 2:
                    raise ParseError(no, line, ".TRAN needs tstep and tstop")
                pc.tran = {"tstep": vals[0], "tstop": vals[1], "tstart": vals[2] if len(vals) > 2 else 0.0,
                           "tmax": vals[3] if len(vals) > 3 else 0.0,
                           "uic": any(t.upper() == "UIC" for t in toks[1:])}
            elif head == ".OPTIONS" or head == ".OPTION":
                if len(toks) > 1 and toks[1].upper() == "TIMEINT":
                    opts = _pairs(toks[2:], no, line)
                    for k in ("RELTOL", "ABSTOL"):
                        if k in opts:
                            pc.options[k.lower()] = opts[k]
            elif head == ".PRINT":
                if len(toks) < 2 or toks[1].upper() != "TRAN":
                    raise ParseError(no, line, "only .PRINT TRAN is supported")
                rest = toks[2:]
                k = 0
                while k < len(rest):
                    if rest[k].upper() == "V" and k + 2 < len(rest) and rest[k + 1] == "(":
                        if rest[k + 3] != ")":
                            raise ParseError(no, line, "only single-node voltages V(node)")
                        prints.append((no, line, rest[k + 2]))
                        k += 4
                    else:
                        raise ParseError(no, line, f"output {rest[k]!r} is not supported")
            elif head in (".SUBCKT", ".ENDS", ".INCLUDE", ".INC", ".LIB", ".PARAM", ".FUNC", ".STEP",
                          ".DC", ".AC", ".OP", ".IC", ".NODESET"):
                raise ParseError(no, line, f"{head} is not supported")
            else:
                raise ParseError(no, line, f"unknown control line {head}")
            continue
        letter = head[0]
        if letter not in "RCVIDM":
            raise ParseError(no, line, f"device {head} is not supported")
        # nodes are numbered in the order the netlist first names them
        for t in toks[1:1 + (4 if letter == "M" else 2)]:
            if t not in ("(", ")", "=", ","):
                node(t)
        elems.append((letter, no, line, toks))

    if pc.tran is None and any(e[0] in "VI" and "PULSE" in [t.upper() for t in e[3]] for e in elems):
        raise ParseError(0, "", "a PULSE source needs a .TRAN line for its defaults")
    groups = {k: [] for k in "RCVIDM"}
    for letter, no, line, toks in elems:
        groups[letter].append((no, line, toks))
    # models in first-use order, so a netlist's cards have stable indices
    model_index = {}
    nl_models = []

    def model_of(name, no, line, want):
        key = name.upper()
        if key not in models:
            raise ParseError(no, line, f"model {name} is not defined")
        t, pol, params = models[key]
        if t not in want:
            raise ParseError(no, line, f"model {name} is not a model of this device")
        if key not in model_index:
            model_index[key] = len(nl_models)
            nl_models.append(abi.Model(t, pol, **params))
        return model_index[key], t

    res, cap = {"p": [], "m": [], "value": []}, {"p": [], "m": [], "value": []}
    src = {"V": {"p": [], "m": [], "kind": [], "wave": []}, "I": {"p": [], "m": [], "kind": [], "wave": []}}
    dio = {"a": [], "c": [], "model": [], "area": []}
    mos = {t: {k: [] for k in ("d", "g", "s", "b", "model", "w", "l", "ad", "as", "pd", "ps", "nrd", "nrs",
                               "m")} for t in (abi.DEV_MOS1, abi.DEV_BSIM3)}
    geo_keys = ("W", "L", "AD", "AS", "PD", "PS", "NRD", "NRS", "M")
    for letter in "RCVIDM":
        for no, line, toks in groups[letter]:
            try:
                if letter in "RC":
                    if len(toks) != 4:
                        raise ParseError(no, line, f"{letter} needs two nodes and a value (no other parameters)")
                    g = res if letter == "R" else cap
                    g["p"].append(node(toks[1]))
                    g["m"].append(node(toks[2]))
                    g["value"].append(spice_number(toks[3]))
                elif letter in "VI":
                    if len(toks) < 4:
                        raise ParseError(no, line, f"{letter} needs two nodes and a value")
                    g = src[letter]
                    p, m = node(toks[1]), node(toks[2])
                    rest = toks[3:]
                    if rest[0].upper() == "DC":
                        rest = rest[1:]
                    if rest[0].upper() == "PULSE":
                        vals = [spice_number(t) for t in rest[1:] if t not in ("(", ")", ",")]
                        if len(vals) > 7:
                            raise ParseError(no, line, "PULSE takes at most 7 values")
                        tr = pc.tran
                        dflt = [0.0, 0.0, 0.0, tr["tstep"], tr["tstep"], tr["tstop"], tr["tstop"]]
                        wave = vals + dflt[len(vals):]
                        kind = abi.SRC_PULSE
                    elif len(rest) == 1:
                        wave = [spice_number(rest[0])] + [0.0] * 6
                        kind = abi.SRC_DC
                    else:
                        raise ParseError(no, line, f"source shape {rest[0]} is not supported")
                    g["p"].append(p)
                    g["m"].append(m)
                    g["kind"].append(kind)
                    g["wave"].append(wave)
                elif letter == "D":
                    if len(toks) < 4:
                        raise ParseError(no, line, "D needs two nodes and a model")
                    a, c = node(toks[1]), node(toks[2])
                    mi, _ = model_of(toks[3], no, line, (abi.DEV_DIODE,))
                    area = 1.0
                    rest = toks[4:]
                    if rest and rest[0] not in ("=",) and (len(rest) == 1 or rest[1] != "="):
                        area = spice_number(rest[0])
                        rest = rest[1:]
                    extra = _pairs(rest, no, line)
                    area = extra.pop("AREA", area)
                    if extra:
                        raise ParseError(no, line, f"diode parameter(s) {sorted(extra)} not supported")
                    dio["a"].append(a)
                    dio["c"].append(c)
                    dio["model"].append(mi)
                    dio["area"].append(area)
                else:  # M
                    if len(toks) < 6:
                        raise ParseError(no, line, "M needs four nodes and a model")
                    d, gg, s, b = (node(t) for t in toks[1:5])
                    mi, t = model_of(toks[5], no, line, (abi.DEV_MOS1, abi.DEV_BSIM3))
                    given = _pairs(toks[6:], no, line)
                    for k in given:
                        if k not in geo_keys:
                            raise ParseError(no, line, f"MOSFET parameter {k} not supported")
                    g = mos[t]
                    for k, v in zip(("d", "g", "s", "b"), (d, gg, s, b)):
                        g[k].append(v)
                    g["model"].append(mi)
                    for k in geo_keys:
                        g[k.lower()].append(given.get(k, np.nan))
            except ValueError as e:
                if isinstance(e, ParseError):
                    raise
                raise ParseError(no, line, str(e)) from None

    nl = abi.Netlist(len(pc.node_names))
    for m in nl_models:
        nl.add_model(m)
    if res["p"]:
        nl.res = {k: np.asarray(v) for k, v in res.items()}
    if cap["p"]:
        nl.cap = {k: np.asarray(v) for k, v in cap.items()}
    for letter, attr in (("V", "vsrc"), ("I", "isrc")):
        g = src[letter]
        if g["p"]:
            setattr(nl, attr, {"p": np.asarray(g["p"]), "m": np.asarray(g["m"]), "kind": np.asarray(g["kind"]),
                               "wave": np.asarray(g["wave"], np.float64).reshape(-1, 7)})
    if dio["a"]:
        nl.diode = {k: np.asarray(v) for k, v in dio.items()}
    for t, attr in ((abi.DEV_MOS1, "mos1"), (abi.DEV_BSIM3, "bsim3")):
        g = mos[t]
        if g["d"]:
            arr = {k: np.asarray(v) for k, v in g.items() if v}
            # an instance parameter that no instance gives stays the model's
            # (or the device options') default; the set-up takes a given array
            # as given on every instance
            for k in [x.lower() for x in geo_keys]:
                if np.isnan(arr[k]).all():
                    del arr[k]
                elif np.isnan(arr[k]).any():
                    raise ParseError(0, "", f"MOSFET {k.upper()} given on some instances of a type only")
            setattr(nl, attr, arr)
    pc.netlist = nl
    for no, line, name in prints:
        n = name.upper()
        if n == "0":
            raise ParseError(no, line, "V(0) is ground")
        if n not in nodes:
            raise ParseError(no, line, f"node {name} is not in the circuit")
        pc.outputs.append((f"V({name})", nodes[n]))
    return pc


def parse_file(path):
    with open(path) as f:
        return parse_netlist(f.read())


def run_transient(ctx, pc, precision=abi.LU_FP64, n_refine=0, x0=None, max_points=200000):
    """The parsed .TRAN on the GPU (engine.transient): (t, V[len(t), outputs],
    stats)."""
    from . import engine
    if pc.tran is None:
        raise ValueError("the netlist has no .TRAN line")
    ckt = engine.Circuit(ctx, pc.netlist)
    try:
        tr = pc.tran
        return engine.transient(ckt, tr["tstop"], tr["tstep"], pc.out_idx, x0=x0, uic=tr["uic"],
                                precision=precision, n_refine=n_refine, max_points=max_points,
                                maxstep=tr["tmax"], reltol=pc.options["reltol"], abstol=pc.options["abstol"])
    finally:
        ckt.close()
