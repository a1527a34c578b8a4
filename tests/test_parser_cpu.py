"""The SPICE netlist front end (xyce_gb300/netlist_parser.py) on CPU: SPICE
numbers, the netlist it builds, the reference's PULSE defaults, comments and
continuation lines, refusals with the line they stand on, and the host
set-up of what it parses.  The reference's examples/dio.cir, where the
reference tree is present, is read and then refused at set-up as the
reference refuses it: a level-1 diode given the level-2 parameters IKF, ISR
and NR (N_DEV_Diode.C:1879-1907)."""
import os

import numpy as np
import pytest

from xyce_gb300 import abi, engine
from xyce_gb300.netlist_parser import ParseError, parse_netlist, spice_number

INVERTER = """CMOS inverter into 10 fF
* supply and input
VDD vdd 0 DC 1.8
VIN in 0 PULSE(0 1.8 0 100p 100p 1n 2n)
M1 out in 0 0 NM W=2u L=1u
M2 out in vdd vdd PM
+ W=4u L=1u    ; the PMOS is twice as wide
C1 out 0 10fF
.model NM NMOS (LEVEL=1 VTO=0.7 KP=110u)
.MODEL pm pmos level=1 vto=-0.7 kp=50u
.tran 1p 2n
.options TIMEINT reltol=1e-4 abstol=1e-7
.options NONLIN maxstep=100
.print tran v(out) V(in)
.end
"""


def test_spice_numbers():
    cases = {"1k": 1e3, "10pF": 1e-11, "2.5meg": 2.5e6, "1e-3": 1e-3, "25mil": 25 * 25.4e-6,
             "3M": 3e-3, "4u": 4e-6, "7n": 7e-9, "1.5f": 1.5e-15, "2G": 2e9, "1T": 1e12, "-0.5": -0.5,
             ".25": 0.25, "1kOhm": 1e3}
    for tok, want in cases.items():
        assert spice_number(tok) == pytest.approx(want, rel=1e-15), tok
    with pytest.raises(ValueError):
        spice_number("abc")


def test_inverter_netlist():
    pc = parse_netlist(INVERTER)
    nl = pc.netlist
    assert pc.title == "CMOS inverter into 10 fF"
    assert pc.node_names == ["vdd", "in", "out"] and nl.n_nodes == 3
    assert list(nl.vsrc["kind"]) == [abi.SRC_DC, abi.SRC_PULSE]
    assert np.array_equal(nl.vsrc["wave"][1], [0, 1.8, 0, 100e-12, 100e-12, 1e-9, 2e-9])
    assert list(nl.mos1["d"]) == [2, 2] and list(nl.mos1["g"]) == [1, 1]
    assert list(nl.mos1["s"]) == [-1, 0] and list(nl.mos1["b"]) == [-1, 0]
    assert np.allclose(nl.mos1["w"], [2e-6, 4e-6]) and "ad" not in nl.mos1
    cards = list(nl.cards())
    assert [(c.type, c.polarity) for c in cards] == [(abi.DEV_MOS1, 1), (abi.DEV_MOS1, -1)]
    assert cards[1].params == {"VTO": -0.7, "KP": pytest.approx(50e-6)}
    assert nl.cap["value"][0] == pytest.approx(10e-15)
    assert pc.tran == {"tstep": 1e-12, "tstop": 2e-9, "tstart": 0.0, "tmax": 0.0, "uic": False}
    assert pc.options == {"reltol": 1e-4, "abstol": 1e-7}
    assert pc.outputs == [("V(out)", 2), ("V(in)", 1)]


def test_pulse_defaults_are_the_references():
    pc = parse_netlist("t\nV1 a 0 PULSE(0 5)\nR1 a 0 1k\n.TRAN 2n 1u\n.END\n")
    # TD 0, TR = TF = the .TRAN step, PW = PER = the stop time
    assert np.array_equal(pc.netlist.vsrc["wave"][0], [0, 5, 0, 2e-9, 2e-9, 1e-6, 1e-6])


@pytest.mark.parametrize("text, where, what", [
    ("t\nX1 a b sub\n.END\n", 2, "not supported"),
    ("t\n.SUBCKT inv a b\n.ENDS\n", 2, "not supported"),
    ("t\nV1 a 0 SIN(0 1 1k)\n.TRAN 1n 1u\n", 2, "not supported"),
    ("t\nD1 a 0 NODEF\n", 2, "not defined"),
    ("t\nR1 a 0 1k\n.model M1 NMOS (LEVEL=3)\n", 3, "level 3"),
    ("t\nM1 d g s b NM W=1u X=2\n.model NM NMOS\n", 2, "parameter X"),
    ("t\nR1 a 0 1k\n.PRINT TRAN V(zz)\n", 3, "not in the circuit"),
])
def test_refusals_name_their_line(text, where, what):
    with pytest.raises(ParseError) as e:
        parse_netlist(text)
    assert e.value.line_no == where and what in str(e.value)


def test_parsed_circuit_sets_up_like_a_built_one(engine_lib):
    pc = parse_netlist(INVERTER)
    got = engine.setup_params(pc.netlist, abi.DEV_MOS1)
    # the same two devices built directly
    nl = abi.Netlist(3)
    # "110u" is 110 * 1e-6, the reference's conversion (a scale multiply)
    nl.add_model(abi.Model(abi.DEV_MOS1, 1, VTO=0.7, KP=110 * 1e-6))
    nl.add_model(abi.Model(abi.DEV_MOS1, -1, VTO=-0.7, KP=50 * 1e-6))
    nl.mos1 = dict(d=np.array([2, 2]), g=np.array([1, 1]), s=np.array([-1, 0]), b=np.array([-1, 0]),
                   model=np.array([0, 1]), w=np.array([2 * 1e-6, 4 * 1e-6]), l=np.array([1e-6, 1e-6]))
    want = engine.setup_params(nl, abi.DEV_MOS1)
    assert np.array_equal(got, want)


def _reference_tree():
    from oracle.ref_build import build_ref
    return os.environ.get("XYCE_REFERENCE") or build_ref.DEFAULT_REF


REF_DIO = os.path.join(_reference_tree(), "examples", "dio.cir")


@pytest.mark.skipif(not os.path.exists(REF_DIO), reason="the reference tree is not present")
def test_reference_example_is_refused_as_the_reference_refuses_it(engine_lib):
    with open(REF_DIO) as f:
        text = f.read()
    pc = parse_netlist(text)
    nl = pc.netlist
    assert nl.n_nodes == 2 and pc.outputs == [("V(1)", 0), ("V(2)", 1)]
    assert pc.tran["tstep"] == 1e-5 and pc.tran["tstop"] == 0.1
    assert np.array_equal(nl.vsrc["wave"][0], [1, 5, 0, 6e-5, 0, 1e20, 0])
    card = next(nl.cards())
    assert card.params["CJO"] == pytest.approx(175e-12) and card.params["IBV"] == pytest.approx(20.245e-3)
    # a level-1 diode given level-2 parameters: refused at set-up, as the
    # reference's Diode::Model refuses it
    with pytest.raises(engine.XgError) as e:
        engine.setup_params(nl, abi.DEV_DIODE)
    assert e.value.status == -8 and any(p in str(e.value) for p in ("IKF", "ISR", "NR"))
    # without them the same netlist sets up
    for p in ("ikf=0", "isr=1.859n", "nr=2"):
        text = text.replace(p, "")
    blk = engine.setup_params(parse_netlist(text).netlist, abi.DEV_DIODE)
    assert blk.shape[1] == 1
