"""xg_load_noalloc: the load for callers that cannot allocate device memory
where they load (a host simulator that gives the GPU a fixed memory budget up
front, a real-time loop that must never enter the allocator).  Its stamp-term
scratch is a fixed array inside the library instead of a per-circuit buffer,
and its outputs go to a buffer the caller passes in.  Checked through the C
ABI against xg_load: on two calls in a row on a level-1 circuit, on a BSIM3
circuit (its members carried between loads start from zero in two circuits
set up alike), and for its size limit.  Kept in a file collected last.
"""
import ctypes as C

import numpy as np
import pytest

from xyce_gb300 import abi, engine, netlists

pytestmark = pytest.mark.gpu


def _noalloc(c, flags, out_ptr, out_len):
    return engine.lib().xg_load_noalloc(c.h, C.byref(flags), C.c_void_p(out_ptr), C.c_int64(out_len))


def test_noalloc_load_matches_regular_load_twice(engine_lib):
    import torch
    L = engine.lib()
    L.xg_load_noalloc.argtypes = [C.c_void_p, C.POINTER(abi.XgLoadFlags), C.c_void_p, C.c_int64]
    ctx = engine.Context(0, abi.device_options())
    # level-1 inverters with load capacitors and sources: no member carried
    # from one load to the next, so each load depends on its inputs alone
    c = engine.Circuit(ctx, netlists.inverter_chain(2000))
    n_out = 4 * (c.n_unknowns + 1) + 2 * c.nnz
    assert c.info.n_terms <= 2 * 1024 * 1024
    out = torch.full((n_out,), float("nan"), dtype=torch.float64, device="cuda:0")
    for k in range(2):
        ins = netlists.random_state(c.n_unknowns, c.n_state, c.n_store, seed=20 + k)
        flags = abi.load_flags(transient=1, newton_iter=1 + k, time=0.4e-9 * (k + 1), pdt=1e11)
        c.set_state(*ins)
        c.load(flags)
        want = c.outputs()
        want_state = (c.download(abi.VEC_STA_NEXT), c.download(abi.VEC_STO_NEXT))
        c.set_state(*ins)
        assert _noalloc(c, flags, out.data_ptr(), n_out) == 0, L.xg_last_error()
        ctx.synchronize()
        got = out.cpu().numpy()
        n1 = c.n_unknowns + 1
        np.testing.assert_array_equal(got[0:c.n_unknowns], want["F"])
        np.testing.assert_array_equal(got[n1:n1 + c.n_unknowns], want["Q"])
        np.testing.assert_array_equal(got[2 * n1:2 * n1 + c.n_unknowns], want["dFdxdVp"])
        np.testing.assert_array_equal(got[3 * n1:3 * n1 + c.n_unknowns], want["dQdxdVp"])
        np.testing.assert_array_equal(got[4 * n1:4 * n1 + c.nnz], want["dFdx"])
        np.testing.assert_array_equal(got[4 * n1 + c.nnz:4 * n1 + 2 * c.nnz], want["dQdx"])
        np.testing.assert_array_equal(c.download(abi.VEC_STA_NEXT), want_state[0])
        np.testing.assert_array_equal(c.download(abi.VEC_STO_NEXT), want_state[1])
    c.close()
    ctx.close()


def _compare_outputs(c, got, want):
    n1 = c.n_unknowns + 1
    np.testing.assert_array_equal(got[0:c.n_unknowns], want["F"])
    np.testing.assert_array_equal(got[n1:n1 + c.n_unknowns], want["Q"])
    np.testing.assert_array_equal(got[2 * n1:2 * n1 + c.n_unknowns], want["dFdxdVp"])
    np.testing.assert_array_equal(got[3 * n1:3 * n1 + c.n_unknowns], want["dQdxdVp"])
    np.testing.assert_array_equal(got[4 * n1:4 * n1 + c.nnz], want["dFdx"])
    np.testing.assert_array_equal(got[4 * n1 + c.nnz:4 * n1 + 2 * c.nnz], want["dQdx"])


def test_noalloc_load_matches_regular_load_bsim3(engine_lib):
    import torch
    L = engine.lib()
    L.xg_load_noalloc.argtypes = [C.c_void_p, C.POINTER(abi.XgLoadFlags), C.c_void_p, C.c_int64]
    ctx = engine.Context(0, abi.device_options())
    models = (abi.Model(abi.DEV_BSIM3, 1), abi.Model(abi.DEV_BSIM3, -1))
    nl = netlists.random_mos_netlist(20_000, 5_000, dev_type=abi.DEV_BSIM3, seed=4, models=models)
    ref = engine.Circuit(ctx, nl)
    c = engine.Circuit(ctx, nl)
    assert c.info.n_terms <= 2 * 1024 * 1024
    ins = netlists.random_state(c.n_unknowns, c.n_state, c.n_store, seed=31)
    flags = abi.load_flags(transient=1, newton_iter=1, time=0.0, pdt=1e11)
    ref.set_state(*ins)
    ref.load(flags)
    want = ref.outputs()
    n_out = 4 * (c.n_unknowns + 1) + 2 * c.nnz
    out = torch.full((n_out,), float("nan"), dtype=torch.float64, device="cuda:0")
    c.set_state(*ins)
    assert _noalloc(c, flags, out.data_ptr(), n_out) == 0, L.xg_last_error()
    ctx.synchronize()
    _compare_outputs(c, out.cpu().numpy(), want)
    np.testing.assert_array_equal(c.download(abi.VEC_STA_NEXT), ref.download(abi.VEC_STA_NEXT))
    np.testing.assert_array_equal(c.download(abi.VEC_STO_NEXT), ref.download(abi.VEC_STO_NEXT))
    ref.close()
    c.close()
    ctx.close()


def test_noalloc_rejects_oversized_circuits_and_short_buffers(engine_lib):
    import torch
    L = engine.lib()
    L.xg_load_noalloc.argtypes = [C.c_void_p, C.POINTER(abi.XgLoadFlags), C.c_void_p, C.c_int64]
    ctx = engine.Context(0, abi.device_options())
    big = engine.Circuit(ctx, netlists.random_mos_netlist(60_000, 20_000, seed=1))
    assert big.info.n_terms > 2 * 1024 * 1024
    out = torch.zeros(16, dtype=torch.float64, device="cuda:0")
    flags = abi.load_flags()
    assert _noalloc(big, flags, out.data_ptr(), 16) == -1
    n_out = 4 * (big.n_unknowns + 1) + 2 * big.nnz
    assert _noalloc(big, flags, out.data_ptr(), n_out) == -1
    assert b"scratch" in L.xg_last_error()
    big.close()
    small = engine.Circuit(ctx, netlists.inverter_chain(10))
    assert _noalloc(small, flags, out.data_ptr(), 16) == -1  # buffer too short
    assert b"shorter" in L.xg_last_error()
    small.close()
    ctx.close()


def _split(got, c):
    n1, n = c.n_unknowns + 1, c.n_unknowns
    return {"F": got[0:n], "Q": got[n1:n1 + n], "dFdxdVp": got[2 * n1:2 * n1 + n],
            "dQdxdVp": got[3 * n1:3 * n1 + n], "dFdx": got[4 * n1:4 * n1 + c.nnz],
            "dQdx": got[4 * n1 + c.nnz:4 * n1 + 2 * c.nnz]}


def test_noalloc_load_matches_regular_load_bsim3(engine_lib):
    """BSIM3 keeps capacitances and charges from one load to the next, so the
    two entry points each run on a circuit of their own, fed the same inputs
    in the same order; both calls of each must agree bit for bit."""
    import torch
    L = engine.lib()
    L.xg_load_noalloc.argtypes = [C.c_void_p, C.POINTER(abi.XgLoadFlags), C.c_void_p, C.c_int64]
    ctx = engine.Context(0, abi.device_options())
    nl = netlists.random_mos_netlist(3000, 700, dev_type=abi.DEV_BSIM3, seed=41,
                                     models=(abi.Model(abi.DEV_BSIM3, 1), abi.Model(abi.DEV_BSIM3, -1)))
    ref = engine.Circuit(ctx, nl)
    na = engine.Circuit(ctx, nl)
    n_out = 4 * (na.n_unknowns + 1) + 2 * na.nnz
    assert na.info.n_terms <= 2 * 1024 * 1024
    out = torch.full((n_out,), float("nan"), dtype=torch.float64, device="cuda:0")
    for k in range(2):
        ins = netlists.random_state(ref.n_unknowns, ref.n_state, ref.n_store, seed=30 + k)
        flags = abi.load_flags(transient=1, newton_iter=1 + k, time=0.4e-9 * (k + 1), pdt=1e11)
        ref.set_state(*ins)
        ref.load(flags)
        want = ref.outputs()
        na.set_state(*ins)
        assert _noalloc(na, flags, out.data_ptr(), n_out) == 0, L.xg_last_error()
        ctx.synchronize()
        got = _split(out.cpu().numpy(), na)
        for key, v in got.items():
            np.testing.assert_array_equal(v, want[key], err_msg=f"call {k}: {key}")
        np.testing.assert_array_equal(na.download(abi.VEC_STA_NEXT), want["sta_next"])
        np.testing.assert_array_equal(na.download(abi.VEC_STO_NEXT), want["sto_next"])
    ref.close()
    na.close()
    ctx.close()
