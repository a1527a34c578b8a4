"""Python driver for the C oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; never by the engine.
"""
import ctypes as C
import os

import numpy as np

from xyce_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from xyce_gb300 import build
            build.build_oracle()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.xgo_build.argtypes = [C.POINTER(abi.XgNetlist), C.POINTER(abi.XgDeviceOptions), vp,
                                C.POINTER(vp)]
        L.xgo_free.argtypes = [vp]
        L.xgo_sizes.argtypes = [vp] + [C.POINTER(C.c_int)] * 3 + [C.POINTER(C.c_int64)]
        L.xgo_pattern.argtypes = [vp, vp, vp]
        L.xgo_reset_members.argtypes = [vp]
        L.xgo_load.argtypes = [vp, C.POINTER(abi.XgLoadFlags), vp] + [vp] * 8
        L.xgo_load_range.argtypes = [vp, C.POINTER(abi.XgLoadFlags), vp, C.c_int, C.c_int,
                                     C.c_int] + [vp] * 8
        L.xgo_tran_run.argtypes = [vp, C.POINTER(TranOpts), vp, vp, C.POINTER(C.c_int),
                                   C.POINTER(TranStats)]
        L.xgo_sparse_solve.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp]
        L.xgo_min_degree.argtypes = [C.c_int, vp, vp, vp]
        L.xgo_setup_params.argtypes = [C.POINTER(abi.XgNetlist), C.POINTER(abi.XgDeviceOptions),
                                       C.c_int, vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _lib = L
    return _lib


class TranOpts(C.Structure):
    _fields_ = [("tstop", C.c_double), ("tstep", C.c_double), ("maxstep", C.c_double),
                ("reltol", C.c_double), ("abstol", C.c_double), ("n_out", C.c_int),
                ("out_idx", C.c_void_p), ("max_points", C.c_int), ("col_order", C.c_void_p),
                ("x0", C.c_void_p), ("uic", C.c_int)]


class TranStats(C.Structure):
    _fields_ = [("status", C.c_int), ("steps", C.c_int), ("steps_attempted", C.c_int),
                ("rejected", C.c_int), ("newton_iters", C.c_int), ("factorizations", C.c_int),
                ("loads", C.c_int), ("dcop_iters", C.c_int), ("dcop_solves", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def setup_params(netlist, dev_type, options=None):
    """The (n_params, n_instances) parameter block of one device type from the
    oracle's own restatement of the reference's set-up."""
    cnl = netlist.to_c()
    opt = options or abi.device_options()
    npar, ninst = C.c_int(), C.c_int()
    rc = lib().xgo_setup_params(C.byref(cnl), C.byref(opt), dev_type, None, C.byref(npar),
                                C.byref(ninst))
    if rc != 0:
        raise RuntimeError(f"xgo_setup_params failed: {rc}")
    out = np.zeros((npar.value, ninst.value))
    if ninst.value:
        rc = lib().xgo_setup_params(C.byref(cnl), C.byref(opt), dev_type, _ptr(out), None, None)
        if rc != 0:
            raise RuntimeError(f"xgo_setup_params failed: {rc}")
    return out


def all_params(netlist, options=None):
    """Parameter blocks of every device type present, from the oracle's set-up."""
    return {t: setup_params(netlist, t, options) for t in range(abi.NUM_DEV_TYPES)
            if netlist.count(t)}


def min_degree_order(rowptr, col):
    """Minimum-degree column order (dense rows last) of a CSR pattern for the
    transient driver's sparse LU."""
    rp = np.ascontiguousarray(rowptr, np.int32)
    ci = np.ascontiguousarray(col, np.int32)
    order = np.zeros(rp.size - 1, np.int32)
    rc = lib().xgo_min_degree(rp.size - 1, _ptr(rp), _ptr(ci), _ptr(order))
    if rc != 0:
        raise RuntimeError(f"xgo_min_degree failed: {rc}")
    return order


def sparse_solve(rowptr, col, val, b, col_order=None):
    """x = A^-1 b with the transient driver's partial-pivoting sparse LU."""
    rp = np.ascontiguousarray(rowptr, np.int32)
    ci = np.ascontiguousarray(col, np.int32)
    v = np.ascontiguousarray(val, np.float64)
    bb = np.ascontiguousarray(b, np.float64)
    x = np.zeros_like(bb)
    q = None if col_order is None else np.ascontiguousarray(col_order, np.int32)
    rc = lib().xgo_sparse_solve(rp.size - 1, _ptr(rp), _ptr(ci), _ptr(v),
                                None if q is None else _ptr(q), _ptr(bb), _ptr(x))
    if rc != 0:
        raise RuntimeError(f"xgo_sparse_solve failed: {rc}")
    return x


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleCircuit:
    """params: dict dev_type -> (n_params, n_instances) array from setup."""

    def __init__(self, netlist, params, options=None):
        self._nl = netlist.to_c()
        self._opt = options or abi.device_options()
        self._blocks = {t: np.ascontiguousarray(p, np.float64) for t, p in params.items()}
        arr = (C.c_void_p * abi.NUM_DEV_TYPES)()
        for t, b in self._blocks.items():
            arr[t] = _ptr(b)
        self._arr = arr
        h = C.c_void_p()
        rc = lib().xgo_build(C.byref(self._nl), C.byref(self._opt), arr, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"xgo_build failed: {rc}")
        self.h = h
        n, s, t, z = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
        lib().xgo_sizes(h, C.byref(n), C.byref(s), C.byref(t), C.byref(z))
        self.n_unknowns, self.n_state, self.n_store, self.nnz = n.value, s.value, t.value, z.value
        self.rowptr = np.zeros(self.n_unknowns + 1, np.int32)
        self.col = np.zeros(max(1, self.nnz), np.int32)
        lib().xgo_pattern(h, _ptr(self.rowptr), _ptr(self.col))
        self.col = self.col[: self.nnz]

    def close(self):
        if getattr(self, "h", None):
            lib().xgo_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset_members(self):
        lib().xgo_reset_members(self.h)

    def _inputs(self, sol, sta, sto):
        # copies: a BSIM3 load on the first transient step writes the current
        # state vector (N_DEV_MOSFET_B3.C:9264-9278), which must not reach the
        # caller's arrays
        ins = [np.array(v, dtype=np.float64, copy=True) for v in list(sol) + list(sta) + list(sto)]
        ins = [v if v.size else np.zeros(1) for v in ins]
        return ins, (C.c_void_p * 9)(*[_ptr(a) for a in ins])

    def load(self, flags, sol, sta, sto):
        nr = self.n_unknowns + 1
        ins, arr = self._inputs(sol, sta, sto)
        out = {k: np.zeros(nr) for k in ("F", "Q", "dFdxdVp", "dQdxdVp")}
        out["sta_next"] = np.zeros(max(1, self.n_state))
        out["sto_next"] = np.zeros(max(1, self.n_store))
        out["dFdx"] = np.zeros(max(1, self.nnz))
        out["dQdx"] = np.zeros(max(1, self.nnz))
        rc = lib().xgo_load(self.h, C.byref(flags), arr, *[_ptr(out[k]) for k in (
            "F", "Q", "dFdxdVp", "dQdxdVp", "sta_next", "sto_next", "dFdx", "dQdx")])
        if rc != 0:
            raise RuntimeError(f"xgo_load failed: {rc}")
        for k in ("F", "Q", "dFdxdVp", "dQdxdVp"):
            out[k] = out[k][: self.n_unknowns]
        out["sta_next"] = out["sta_next"][: self.n_state]
        out["sto_next"] = out["sto_next"][: self.n_store]
        out["dFdx"] = out["dFdx"][: self.nnz]
        out["dQdx"] = out["dQdx"][: self.nnz]
        out["rows"] = np.repeat(np.arange(self.n_unknowns, dtype=np.int32), np.diff(self.rowptr))
        out["cols"] = self.col.copy()
        return out

    def load_range_timed(self, flags, sol, sta, sto, dev_type, i0, i1, scratch=None):
        """Load instances [i0, i1) of one type into scratch outputs; returns scratch."""
        nr = self.n_unknowns + 1
        ins, arr = self._inputs(sol, sta, sto)
        if scratch is None:
            scratch = [np.zeros(nr) for _ in range(4)] + [
                np.array(ins[3], copy=True), np.array(ins[6], copy=True),
                np.zeros(max(1, self.nnz)), np.zeros(max(1, self.nnz))]
        rc = lib().xgo_load_range(self.h, C.byref(flags), arr, dev_type, i0, i1,
                                  *[_ptr(a) for a in scratch])
        if rc != 0:
            raise RuntimeError(f"xgo_load_range failed: {rc}")
        return scratch


def transient(oc, tstop, tstep, out_idx, col_order=None, max_points=200000, maxstep=0.0,
              reltol=1e-3, abstol=1e-6, x0=None, uic=False):
    """DC operating point (from the guess x0, or x0 itself with uic) then
    .TRAN tstep tstop on an OracleCircuit; returns (t, V[len(t), len(out_idx)],
    stats dict)."""
    idx = np.ascontiguousarray(out_idx, np.int32)
    q = None if col_order is None else np.ascontiguousarray(col_order, np.int32)
    x0a = None if x0 is None else np.ascontiguousarray(x0, np.float64)
    o = TranOpts(tstop, tstep, maxstep, reltol, abstol, idx.size, _ptr(idx).value, max_points,
                 None if q is None else _ptr(q).value, None if x0a is None else _ptr(x0a).value,
                 int(bool(uic)))
    t = np.zeros(max_points)
    v = np.zeros((max_points, max(1, idx.size)))
    npts = C.c_int()
    st = TranStats()
    rc = lib().xgo_tran_run(oc.h, C.byref(o), _ptr(t), _ptr(v), C.byref(npts), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"xgo_tran_run failed: {rc} {st.as_dict()}")
    n = npts.value
    return t[:n], v[:n, : idx.size], st.as_dict()


# ---- the integrator's formulas (xgo_tran.c), one call each -----------------

def _d(a):
    return np.ascontiguousarray(a, np.float64)


def _tia_lib(L):
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    if getattr(L, "_tia_ready", False):
        return L
    names = {"update_coeffs": "xgo_tia_update_coeffs", "predictor": "xgo_tia_predictor",
             "residual": "xgo_tia_residual", "jacobian": "xgo_tia_jacobian",
             "error_estimate": "xgo_tia_error_estimate", "converged": "xgo_nls_converged"}
    if not hasattr(L, names["update_coeffs"]):  # the reference's harness uses xref_ names
        names = {k: v.replace("xgo_tia", "xref_tia").replace("xgo_nls", "xref_nls")
                 for k, v in names.items()}
    L._tia = {k: getattr(L, v) for k, v in names.items()}
    L._tia["update_coeffs"].argtypes = [i, d, d, vp, vp, vp, vp]
    L._tia["predictor"].argtypes = [i, i, vp, vp, vp, vp, vp, vp, vp]
    L._tia["residual"].argtypes = [i, i, d, d, i, vp, vp, vp, vp, vp, vp, vp]
    L._tia["jacobian"].argtypes = [C.c_int64, i, d, d, vp, vp, vp]
    pre = "xref_tia_" if hasattr(L, "xref_tia_update_coeffs") else "xgo_tia_"
    L._tia["complete_step"] = getattr(L, pre + "complete_step")
    L._tia["complete_step"].argtypes = [i, vp, vp, vp, vp, vp, vp]
    L._tia["reject_step"] = getattr(L, pre + "reject_step")
    L._tia["reject_step"].argtypes = [vp, vp]
    L._tia_ready = True
    return L


class Integrator:
    """The integrator's formulas of one library: the oracle's (default) or,
    given oracle.ref's TIA library, the reference's own compiled code, with
    the same calls."""

    def __init__(self, L=None):
        self.L = _tia_lib(L or lib())
        self.ref = hasattr(self.L, "xref_tia_update_coeffs")
        t = self.L._tia
        if self.ref:
            t["error_estimate"].argtypes = [C.c_int, C.c_double, C.c_int] + [C.c_void_p] * 8
            t["converged"].argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_double] * 8 + [
                C.POINTER(C.c_int), C.POINTER(C.c_double)]
        else:
            t["error_estimate"].argtypes = [C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_double,
                                            C.c_double]
            t["converged"].argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_double] * 7 + [
                C.POINTER(C.c_int), C.POINTER(C.c_double)]
        t["error_estimate"].restype = C.c_double
        t["converged"].restype = C.c_int

    def update_coeffs(self, order, h, h_sum, psi):
        psi = _d(psi).copy()
        beta = np.zeros(3)
        a, ck = C.c_double(), C.c_double()
        self.L._tia["update_coeffs"](order, h, h_sum, _ptr(psi), _ptr(beta), C.byref(a), C.byref(ck))
        return psi, beta, a.value, ck.value

    def predictor(self, order, beta, xh0, xh1, xh2, qh0):
        n = len(xh0)
        ins = [_d(v).copy() for v in (beta, xh0, xh1, xh2, qh0)]
        xn0, qn0 = np.zeros(n), np.zeros(n)
        self.L._tia["predictor"](n, order, *[_ptr(v) for v in ins], _ptr(xn0), _ptr(qn0))
        return xn0, qn0

    def residual(self, order, h, alphas, limiter, Q, qn0, F, qh2, fvp, qvp):
        n = len(Q)
        ins = [_d(v).copy() for v in (Q, qn0, F, qh2, fvp, qvp)]
        rhs = np.zeros(n)
        self.L._tia["residual"](n, order, h, alphas, int(limiter), *[_ptr(v) for v in ins], _ptr(rhs))
        return rhs

    def jacobian(self, order, h, alphas, dqdx, dfdx):
        ins = [_d(v).copy() for v in (dqdx, dfdx)]
        jac = np.zeros(len(dqdx))
        self.L._tia["jacobian"](len(dqdx), order, h, alphas, *[_ptr(v) for v in ins], _ptr(jac))
        return jac

    def error_estimate(self, ck, x_curr, corr, reltol, abstol):
        n = len(x_curr)
        if self.ref:
            ins = [_d(v).copy() for v in (x_curr, corr, np.zeros(n), np.zeros(n),
                                          np.full(n, reltol), np.full(n, abstol))]
            wt, qwt = np.zeros(n), np.zeros(n)
            return self.L._tia["error_estimate"](n, ck, 1, *[_ptr(v) for v in ins], _ptr(wt), _ptr(qwt))
        a, b = _d(x_curr), _d(corr)
        return self.L._tia["error_estimate"](n, ck, _ptr(a), _ptr(b), reltol, abstol)

    def converged(self, transient, step, max_step, rhs_tol, dx_tol, small_update, max_rhs, upd,
                  rhs_rel, rate, count=0, stall_rate=0.0):
        """(status, count, stall_rate) after one Newton step."""
        c, r = C.c_int(count), C.c_double(stall_rate)
        if self.ref:  # wtNormDX / stepLength with a full step
            s = self.L._tia["converged"](int(transient), step, max_step, rhs_tol, dx_tol, small_update,
                                         max_rhs, upd, 1.0, rhs_rel, rate, C.byref(c), C.byref(r))
        else:
            s = self.L._tia["converged"](int(transient), step, max_step, rhs_tol, dx_tol, small_update,
                                         max_rhs, upd, rhs_rel, rate, C.byref(c), C.byref(r))
        return s, c.value, r.value

    # step control: state = [order, steps, failures, estOverTol, h, t, t_next,
    # stop time, min step, max step, last step, h_sum, psi0, psi1, psi2,
    # Newton status, saved step]; result = [order, steps, failures, h, t,
    # t_next, last step, h_sum, saved step, psi0, psi1, psi2]
    def complete_step(self, state, hist, x_next, Q, F):
        """OneStep::completeStep: the result, and the six history vectors
        (solution 0..2, charge 0..2) rotated."""
        st = _d(state).copy()
        hs = [_d(v).copy() for v in hist]
        arr = (C.c_void_p * 6)(*[v.ctypes.data for v in hs])
        ins = [_d(v).copy() for v in (x_next, Q, F)]
        out = np.zeros(12)
        self.L._tia["complete_step"](len(x_next), _ptr(st), arr, *[_ptr(v) for v in ins], _ptr(out))
        return out, hs

    def reject_step(self, state):
        st = _d(state).copy()
        out = np.zeros(12)
        self.L._tia["reject_step"](_ptr(st), _ptr(out))
        return out
