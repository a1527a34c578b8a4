"""CPU tests of the C ABI: the library loads, exports every entry point the
headers declare, and rejects bad input with the documented status codes."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from xyce_gb300 import abi, engine, netlists

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(xg_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "xg_load" in names and "xg_update_state" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(engine_lib):
    missing = [n for n in declared_functions() if not hasattr(engine_lib, n)]
    assert not missing, missing


def test_abi_version(engine_lib):
    assert engine_lib.xg_abi_version() == 1


def _status(nl, dev_type=abi.DEV_MOS1, opt=None):
    L = engine.lib()
    c_nl = nl.to_c()
    o = opt or abi.device_options()
    npar, ninst = C.c_int(), C.c_int()
    return L.xg_setup_params(C.byref(c_nl), C.byref(o), dev_type, None, C.byref(npar), C.byref(ninst))


def test_setup_rejects_node_out_of_range(engine_lib):
    nl = netlists.inverter_chain(3)
    nl.mos1["g"][0] = nl.n_nodes  # one past the last node
    assert _status(nl) == -1  # XG_ERR_ARG


def test_setup_rejects_unknown_model_parameter(engine_lib):
    nl = netlists.inverter_chain(3)
    nl.models[0].params["XYZZY"] = 1.0
    assert _status(nl) == -8  # XG_ERR_UNSUPPORTED
    assert b"XYZZY" in engine.lib().xg_last_error()


def test_setup_rejects_newmeyer_and_bad_sources(engine_lib):
    nl = netlists.inverter_chain(3)
    assert _status(nl, opt=abi.device_options(newmeyer=1)) == -8
    nl = netlists.inverter_chain(3)
    nl.isrc = dict(p=[1], m=[-1], kind=[7], wave=[[1e-3, 0, 0, 0, 0, 0, 0]])
    assert _status(nl) == -1  # XG_ERR_ARG: unknown waveform kind
    nl.isrc = dict(p=[1], m=[99], kind=[0], wave=[[1e-3, 0, 0, 0, 0, 0, 0]])
    assert _status(nl) != 0   # terminal outside the circuit
    nl.isrc = dict(p=[1], m=[-1], kind=[0], wave=[[1e-3, 0, 0, 0, 0, 0, 0]])
    assert _status(nl) == 0


def test_setup_rejects_wrong_model_type(engine_lib):
    nl = netlists.inverter_chain(3)
    nl.models[0].type = abi.DEV_DIODE
    assert _status(nl) != 0


def test_setup_params_host_only(engine_lib):
    nl = netlists.inverter_chain(10)
    p = engine.setup_params(nl, abi.DEV_MOS1)
    assert p.shape == (37, 20)
    assert np.all(p[0] == np.tile([1.0, -1.0], 10))  # dtype column: N, P, N, P ...


def test_empty_netlist(engine_lib):
    nl = abi.Netlist(0)
    assert _status(nl, abi.DEV_RES) == 0


def test_context_without_gpu_fails_cleanly(engine_lib):
    if os.environ.get("XG_HAVE_GPU") == "1":
        pytest.skip("GPU present")
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = engine.lib().xg_ctx_create(0, C.byref(h))
    assert rc in (-1, -2) and not h.value


def test_model_set_matches_separate_cards(engine_lib):
    """A ModelSet (Monte-Carlo cards as arrays) gives the same set-up as the
    same cards added one Model at a time, and the same flat arrays."""
    nl = netlists.ring_oscillator(9, seed=4)
    assert isinstance(nl.models[0], abi.ModelSet) and nl.n_models == 18
    per_card = netlists.ring_oscillator(9, seed=4)
    per_card.models = list(nl.cards())
    assert all(isinstance(m, abi.Model) for m in per_card.models)
    opt = abi.device_options()
    for t in range(abi.NUM_DEV_TYPES):
        if nl.count(t):
            assert np.array_equal(engine.setup_params(nl, t, opt), engine.setup_params(per_card, t, opt))
    a, b = nl.to_arrays(), per_card.to_arrays()
    assert a.keys() == b.keys() and all(np.array_equal(a[k], b[k]) for k in a)
