"""Parsed SPICE netlists run end to end: netlist text -> xg_netlist -> the
GPU's .TRAN (xg_tran_run), its waveforms equal to the oracle's transient of
the same parsed netlist within reltol 1e-3 of the signal swing, and the same
number of time points within 2%.  A diode clamp driven by a pulse and a
CMOS inverter, each using its .TRAN, .OPTIONS TIMEINT and .PRINT lines."""
import numpy as np
import pytest

from xyce_gb300 import abi
from xyce_gb300.netlist_parser import parse_netlist, run_transient

pytestmark = pytest.mark.gpu

CLAMP = """diode clamp
VP in 0 PULSE(0 5 0 1n 1n 5n 20n)
R1 in out 1k
D1 out 0 DMOD
C1 out 0 1p
.MODEL DMOD D (IS=1e-14 CJO=2p RS=10)
.TRAN 10p 20n
.PRINT TRAN V(in) V(out)
.END
"""

INVERTER = """CMOS inverter into 10 fF
VDD vdd 0 DC 1.8
VIN in 0 PULSE(0 1.8 0 100p 100p 1n 2n)
M1 out in 0 0 NM W=2u L=1u
M2 out in vdd vdd PM W=4u L=1u
C1 out 0 10fF
.model NM NMOS (LEVEL=1 VTO=0.7 KP=110u)
.model PM PMOS (LEVEL=1 VTO=-0.7 KP=50u)
.tran 1p 4n
.options TIMEINT reltol=1e-3 abstol=1e-6
.print tran v(out) v(in)
.end
"""


@pytest.mark.parametrize("name, text", [("clamp", CLAMP), ("inverter", INVERTER)])
def test_parsed_netlist_transient_matches_oracle(name, text, gpu_ctx, oracle_lib):
    from oracle.oracle import OracleCircuit, all_params, transient
    gpu_ctx.set_options(abi.device_options(fma=0))
    pc = parse_netlist(text)
    t, v, st = run_transient(gpu_ctx, pc)
    opt = abi.device_options()
    oc = OracleCircuit(pc.netlist, all_params(pc.netlist, opt), opt)
    tr = pc.tran
    tc, vc, sc = transient(oc, tr["tstop"], tr["tstep"], pc.out_idx, reltol=pc.options["reltol"],
                           abstol=pc.options["abstol"])
    oc.close()
    assert st["status"] == 0 and abs(t[-1] - tr["tstop"]) <= 1e-12 * tr["tstop"]
    assert abs(len(t) - len(tc)) <= 0.02 * len(tc) + 2, (len(t), len(tc))
    swing = max(1.0, float(np.ptp(vc)))
    vi = np.stack([np.interp(tc, t, v[:, k]) for k in range(v.shape[1])], 1)
    err = float(np.abs(vi - vc).max())
    assert err <= 1e-3 * swing, (name, err)
