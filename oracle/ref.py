"""Python driver for oracle/_ref/libxyceref.so — the reference's own device
code compiled by oracle/ref_build/build_ref.py.  Test infrastructure only:
used to pin the C oracle and to generate golden fixtures, never by the product.
"""
import ctypes as C
import os

import numpy as np

from xyce_gb300 import abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libxyceref.so")
_lib = None


TIA_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libxyceref_tia.so")
_tia = None


def available():
    return os.path.exists(LIB_PATH)


def tia_available():
    return os.path.exists(TIA_LIB_PATH)


def integrator():
    """The reference's own OneStep / DataStore / DampedNewton code
    (libxyceref_tia.so, xref_tia.C) behind oracle.oracle.Integrator's calls."""
    global _tia
    from oracle.oracle import Integrator
    if _tia is None:
        _tia = Integrator(C.CDLL(TIA_LIB_PATH))
    return _tia


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB_PATH)
        _lib.xref_build.argtypes = [C.POINTER(abi.XgNetlist), C.POINTER(abi.XgDeviceOptions),
                                    C.POINTER(C.c_void_p)]
        _lib.xref_free.argtypes = [C.c_void_p]
        _lib.xref_sizes.argtypes = [C.c_void_p] + [C.POINTER(C.c_int)] * 3 + [C.POINTER(C.c_int64)]
        _lib.xref_pattern.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.xref_load.argtypes = [C.c_void_p, C.POINTER(abi.XgLoadFlags), C.c_void_p] + [C.c_void_p] * 8
        _lib.xref_params.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_int)]
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class RefCircuit:
    """One circuit built inside the reference device code."""

    def __init__(self, netlist, options=None):
        self._nl = netlist.to_c()
        self._opt = options or abi.device_options()
        h = C.c_void_p()
        rc = lib().xref_build(C.byref(self._nl), C.byref(self._opt), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"xref_build failed: {rc}")
        self.h = h
        n, s, t, z = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
        lib().xref_sizes(h, C.byref(n), C.byref(s), C.byref(t), C.byref(z))
        self.n_unknowns, self.n_state, self.n_store, self.nnz_gnd = n.value, s.value, t.value, z.value
        self.rowptr = np.zeros(self.n_unknowns + 2, np.int32)
        self.col = np.zeros(self.nnz_gnd, np.int32)
        lib().xref_pattern(h, _ptr(self.rowptr), _ptr(self.col))

    def close(self):
        if self.h:
            lib().xref_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, dev_type):
        """Derived parameters of one device type as the reference computed them,
        shape (n_params, n_instances) in the layout of include/xg_params.h."""
        npar = C.c_int(0)
        n = lib().xref_params(self.h, dev_type, None, C.byref(npar))
        if n <= 0:
            return np.zeros((0, 0))
        out = np.zeros(npar.value * n)
        lib().xref_params(self.h, dev_type, _ptr(out), C.byref(npar))
        return out.reshape(npar.value, n)

    def load(self, flags, sol, sta, sto):
        """sol/sta/sto: sequences (next, curr, last). Returns dict of outputs;
        matrices are returned as dense-free COO over the ground-excluded pattern."""
        nr = self.n_unknowns + 1
        ins = [np.ascontiguousarray(v, np.float64) for v in list(sol) + list(sta) + list(sto)]
        arr = (C.c_void_p * 9)(*[_ptr(a) for a in ins])
        out = {k: np.zeros(nr) for k in ("F", "Q", "dFdxdVp", "dQdxdVp")}
        out["sta_next"] = np.zeros(max(1, self.n_state))
        out["sto_next"] = np.zeros(max(1, self.n_store))
        dfdx = np.zeros(self.nnz_gnd)
        dqdx = np.zeros(self.nnz_gnd)
        rc = lib().xref_load(self.h, C.byref(flags), arr, _ptr(out["F"]), _ptr(out["Q"]),
                             _ptr(out["dFdxdVp"]), _ptr(out["dQdxdVp"]), _ptr(out["sta_next"]),
                             _ptr(out["sto_next"]), _ptr(dfdx), _ptr(dqdx))
        if rc != 0:
            raise RuntimeError(f"xref_load failed: {rc}")
        out["sta_next"] = out["sta_next"][: self.n_state]
        out["sto_next"] = out["sto_next"][: self.n_store]
        rows = np.repeat(np.arange(nr, dtype=np.int32), np.diff(self.rowptr))
        keep = (rows < self.n_unknowns) & (self.col < self.n_unknowns)
        out["rows"], out["cols"] = rows[keep], self.col[keep]
        out["dFdx"], out["dQdx"] = dfdx[keep], dqdx[keep]
        for k in ("F", "Q", "dFdxdVp", "dQdxdVp"):
            out[k] = out[k][: self.n_unknowns]
        return out


KSPARSE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libksparse.so")
_ks = None


def ksparse_available():
    return os.path.exists(KSPARSE_PATH)


def ksparse_solve(rowptr, col, val, b, rel_threshold=1e-3, abs_threshold=1e-13, diag_pivoting=1):
    """x = A \\ b with the reference's Kundert sparse solver, driven as its
    Epetra_CrsKundertSparse wrapper does (ksparse/src/Epetra_CrsKundertSparse.C:
    spGetElement per entry with 1-based indices, spOrderAndFactor with the
    wrapper's default thresholds, spSolve on 1-based vectors).  The library
    keeps state between matrices inside one process (a second matrix of
    another size does not finish), so every solve runs in a fresh process."""
    import concurrent.futures as cf
    import multiprocessing as mp
    args = (np.asarray(rowptr), np.asarray(col), np.asarray(val, np.float64), np.asarray(b, np.float64),
            rel_threshold, abs_threshold, diag_pivoting)
    with cf.ProcessPoolExecutor(1, mp_context=mp.get_context("spawn")) as ex:
        return ex.submit(_ksparse_solve_here, *args).result(timeout=300)


def _ksparse_solve_here(rowptr, col, val, b, rel_threshold, abs_threshold, diag_pivoting):
    global _ks
    if _ks is None:
        _ks = C.CDLL(KSPARSE_PATH)
        _ks.spCreate.restype = C.c_void_p
        _ks.spCreate.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int)]
        _ks.spGetElement.restype = C.POINTER(C.c_double)
        _ks.spGetElement.argtypes = [C.c_void_p, C.c_int, C.c_int]
        _ks.spOrderAndFactor.restype = C.c_int
        _ks.spOrderAndFactor.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int]
        _ks.spSolve.restype = C.c_int
        _ks.spSolve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _ks.spDestroy.argtypes = [C.c_void_p]
    n = len(rowptr) - 1
    err = C.c_int(0)
    m = _ks.spCreate(n, 0, C.byref(err))
    if not m or err.value != 0:
        raise RuntimeError(f"spCreate failed: {err.value}")
    try:
        for i in range(n):
            for p in range(rowptr[i], rowptr[i + 1]):
                e = _ks.spGetElement(m, i + 1, int(col[p]) + 1)
                e[0] += float(val[p])
        rhs = np.zeros(n + 1)
        rhs[1:] = b
        x = np.zeros(n + 1)
        st = _ks.spOrderAndFactor(m, _ptr(rhs), rel_threshold, abs_threshold, diag_pivoting)
        if st != 0:
            raise RuntimeError(f"spOrderAndFactor failed: {st}")
        _ks.spSolve(m, _ptr(rhs), _ptr(x), None, None)
        return x[1:]
    finally:
        _ks.spDestroy(m)
