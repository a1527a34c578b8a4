"""Python host API over libxg's C ABI (include/xg.h).

Mirrors the reference's load interface: a `Circuit` is the set of device
Masters of one netlist, `update_state` / `load_dae_vectors` /
`load_dae_matrices` are Device::updateState / loadDAEVectors /
loadDAEMatrices, and `load` runs all three.  Every call goes to the CUDA
engine; there is no CPU fallback — a missing library or GPU raises.
"""
import atexit
import ctypes as C
import os
import weakref

import numpy as np

from . import abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libxg.so")
_lib = None

# Handles still open at interpreter exit are closed while the library and the
# CUDA runtime are intact, batches, factorisations and circuits before the
# contexts whose streams they use (finalisation would otherwise free them in
# no fixed order).
_OPEN = {k: weakref.WeakSet() for k in ("batch", "lu", "circuit", "context")}


@atexit.register
def _close_open_handles():
    for kind in ("batch", "lu", "circuit", "context"):
        for obj in list(_OPEN[kind]):
            try:
                obj.close()
            except Exception:
                pass


class XgError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"{abi.STATUS.get(status, status)}: {msg}")


def lib():
    """Load libxg.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libxg.so not built ({LIB_PATH}); run python -m xyce_gb300.build")
    L = C.CDLL(LIB_PATH)
    vp, i, i64p = C.c_void_p, C.c_int, C.POINTER(C.c_int64)
    L.xg_abi_version.restype = i
    L.xg_launch_count.restype = C.c_longlong
    L.xg_last_error.restype = C.c_char_p
    L.xg_status_string.restype = C.c_char_p
    L.xg_status_string.argtypes = [i]
    L.xg_ctx_create.argtypes = [i, C.POINTER(vp)]
    L.xg_ctx_destroy.argtypes = [vp]
    L.xg_ctx_set_options.argtypes = [vp, C.POINTER(abi.XgDeviceOptions)]
    L.xg_ctx_get_options.argtypes = [vp, C.POINTER(abi.XgDeviceOptions)]
    L.xg_ctx_synchronize.argtypes = [vp]
    L.xg_ctx_stream.argtypes = [vp, C.POINTER(vp)]
    L.xg_circuit_create.argtypes = [vp, C.POINTER(abi.XgNetlist), C.POINTER(vp)]
    L.xg_circuit_destroy.argtypes = [vp]
    L.xg_circuit_get_info.argtypes = [vp, C.POINTER(abi.XgCircuitInfo)]
    L.xg_circuit_get_pattern.argtypes = [vp, vp, vp]
    L.xg_circuit_get_params.argtypes = [vp, i, vp, C.POINTER(i), C.POINTER(i)]
    L.xg_setup_params.argtypes = [C.POINTER(abi.XgNetlist), C.POINTER(abi.XgDeviceOptions), i, vp,
                                  C.POINTER(i), C.POINTER(i)]
    L.xg_vec_size.argtypes = [vp, i, i64p]
    L.xg_vec_upload.argtypes = [vp, i, vp]
    L.xg_vec_download.argtypes = [vp, i, vp]
    L.xg_vec_device_ptr.argtypes = [vp, i, C.POINTER(vp)]
    L.xg_rotate_history.argtypes = [vp]
    L.xg_update_state.argtypes = [vp, C.POINTER(abi.XgLoadFlags)]
    L.xg_load_dae_vectors.argtypes = [vp]
    L.xg_load_dae_matrices.argtypes = [vp]
    L.xg_load.argtypes = [vp, C.POINTER(abi.XgLoadFlags)]
    L.xg_load_noalloc.argtypes = [vp, C.POINTER(abi.XgLoadFlags), vp, C.c_int64]
    L.xg_probe_fp64_rate.argtypes = [i, C.POINTER(C.c_double)]
    L.xg_probe_reciprocal.argtypes = [i, vp, vp]
    L.xg_lu_analyze.argtypes = [vp, i, vp, vp, vp, i, C.POINTER(vp)]
    L.xg_lu_refactor.argtypes = [vp, vp]
    L.xg_lu_solve.argtypes = [vp, vp, vp, i]
    L.xg_lu_refactor_solve.argtypes = [vp, vp, vp, vp, i]
    L.xg_lu_status.argtypes = [vp, C.POINTER(i), C.POINTER(i)]
    L.xg_lu_set_wait_limit.argtypes = [vp, i]
    L.xg_lu_get_info.argtypes = [vp, C.POINTER(abi.XgLuInfo)]
    L.xg_lu_get_symbolic.argtypes = [vp, vp, vp, vp, vp]
    L.xg_lu_destroy.argtypes = [vp]
    L.xg_lu_order.argtypes = [i, vp, vp, vp, C.POINTER(i)]
    L.xg_lu_analyze_host.argtypes = [i, vp, vp, vp, vp, vp, i64p, C.POINTER(abi.XgLuInfo)]
    L.xg_tran_run.argtypes = [vp, C.POINTER(abi.XgTranOptions), vp, i, vp, i, vp, vp,
                              C.POINTER(i), C.POINTER(abi.XgTranStats)]
    L.xg_batch_create.argtypes = [vp, i, vp, vp, vp, vp, C.POINTER(abi.XgBatchOptions),
                                  C.POINTER(vp)]
    L.xg_batch_run.argtypes = [vp, i]
    L.xg_batch_poll.argtypes = [vp, i, C.POINTER(i)]
    L.xg_batch_inflight.argtypes = [vp, C.POINTER(i)]
    L.xg_batch_results.argtypes = [vp, i, vp, vp, C.POINTER(i), C.POINTER(abi.XgTranStats)]
    L.xg_batch_info.argtypes = [vp, C.POINTER(i), i64p]
    L.xg_batch_destroy.argtypes = [vp]
    L.xg_slot_need.argtypes = [vp, vp, vp, C.c_double, C.c_double, C.POINTER(abi.XgSlotShape)]
    L.xg_slot_bytes.argtypes = [C.POINTER(abi.XgSlotShape), C.POINTER(abi.XgBatchOptions), i64p]
    L.xg_batch_create_slots.argtypes = [vp, i, C.POINTER(abi.XgSlotShape), C.POINTER(abi.XgBatchOptions),
                                        C.POINTER(vp)]
    L.xg_batch_submit.argtypes = [vp, i, vp, vp, vp, vp, vp]
    L.xg_batch_release.argtypes = [vp, i]
    L.xg_batch_slots.argtypes = [vp, C.POINTER(i), C.POINTER(i)]
    L.xg_batch_finished.argtypes = [vp, i, vp, C.POINTER(i)]
    L.xg_mem_info.argtypes = [vp, i64p, i64p]
    _lib = L
    return L


def check(rc):
    if rc != 0:
        raise XgError(rc, lib().xg_last_error().decode())
    return rc


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def setup_params(netlist, dev_type, options=None):
    """Host-only setup: the derived parameter block of one device type,
    shape (n_params, n_instances) (include/xg_params.h)."""
    nl = netlist if isinstance(netlist, abi.XgNetlist) else netlist.to_c()
    opt = options or abi.device_options()
    npar, ninst = C.c_int(), C.c_int()
    check(lib().xg_setup_params(C.byref(nl), C.byref(opt), dev_type, None, C.byref(npar),
                                C.byref(ninst)))
    out = np.zeros(max(1, npar.value * ninst.value))
    check(lib().xg_setup_params(C.byref(nl), C.byref(opt), dev_type, _ptr(out), C.byref(npar),
                                C.byref(ninst)))
    return out[: npar.value * ninst.value].reshape(npar.value, ninst.value)


class Context:
    """One GPU and one CUDA stream (the DeviceMgr of one simulation)."""

    def __init__(self, device=0, options=None):
        h = C.c_void_p()
        check(lib().xg_ctx_create(device, C.byref(h)))
        self.h = h
        _OPEN["context"].add(self)
        if options is not None:
            self.set_options(options)

    def set_options(self, options):
        check(lib().xg_ctx_set_options(self.h, C.byref(options)))

    def synchronize(self):
        check(lib().xg_ctx_synchronize(self.h))

    def stream(self):
        s = C.c_void_p()
        check(lib().xg_ctx_stream(self.h, C.byref(s)))
        return s.value

    def close(self):
        if getattr(self, "h", None):
            lib().xg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Circuit:
    """A netlist set up on the GPU: parameters, numbering, pattern, load plan."""

    def __init__(self, ctx, netlist):
        self.ctx = ctx
        self._nl = netlist.to_c()
        h = C.c_void_p()
        check(lib().xg_circuit_create(ctx.h, C.byref(self._nl), C.byref(h)))
        self.h = h
        _OPEN["circuit"].add(self)
        info = abi.XgCircuitInfo()
        check(lib().xg_circuit_get_info(h, C.byref(info)))
        self.info = info
        self.n_unknowns, self.n_state, self.n_store = info.n_unknowns, info.n_state, info.n_store
        self.nnz = info.nnz
        self.rowptr = np.zeros(self.n_unknowns + 1, np.int32)
        self.colidx = np.zeros(max(1, self.nnz), np.int32)
        check(lib().xg_circuit_get_pattern(h, _ptr(self.rowptr), _ptr(self.colidx)))
        self.colidx = self.colidx[: self.nnz]

    def close(self):
        if getattr(self, "h", None):
            lib().xg_circuit_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, dev_type):
        npar, ninst = C.c_int(), C.c_int()
        check(lib().xg_circuit_get_params(self.h, dev_type, None, C.byref(npar), C.byref(ninst)))
        out = np.zeros(max(1, npar.value * ninst.value))
        check(lib().xg_circuit_get_params(self.h, dev_type, _ptr(out), None, None))
        return out[: npar.value * ninst.value].reshape(npar.value, ninst.value)

    def vec_size(self, vec_id):
        n = C.c_int64()
        check(lib().xg_vec_size(self.h, vec_id, C.byref(n)))
        return n.value

    def upload(self, vec_id, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        if a.size != self.vec_size(vec_id):
            raise ValueError(f"vector {vec_id}: expected {self.vec_size(vec_id)} values, got {a.size}")
        check(lib().xg_vec_upload(self.h, vec_id, _ptr(a)))

    def download(self, vec_id):
        a = np.zeros(self.vec_size(vec_id))
        if a.size:
            check(lib().xg_vec_download(self.h, vec_id, _ptr(a)))
        return a

    def device_ptr(self, vec_id):
        p = C.c_void_p()
        check(lib().xg_vec_device_ptr(self.h, vec_id, C.byref(p)))
        return p.value

    def rotate_history(self):
        check(lib().xg_rotate_history(self.h))

    def update_state(self, flags):
        check(lib().xg_update_state(self.h, C.byref(flags)))

    def load_dae_vectors(self):
        check(lib().xg_load_dae_vectors(self.h))

    def load_dae_matrices(self):
        check(lib().xg_load_dae_matrices(self.h))

    def load(self, flags):
        check(lib().xg_load(self.h, C.byref(flags)))

    def set_state(self, sol, sta, sto):
        """sol/sta/sto: (next, curr, last) host vectors; sto next = previous iterate."""
        for k, vid in enumerate((abi.VEC_SOL_NEXT, abi.VEC_SOL_CURR, abi.VEC_SOL_LAST)):
            self.upload(vid, sol[k])
        for k, vid in enumerate((abi.VEC_STA_NEXT, abi.VEC_STA_CURR, abi.VEC_STA_LAST)):
            if self.n_state:
                self.upload(vid, sta[k])
        for k, vid in enumerate((abi.VEC_STO_NEXT, abi.VEC_STO_CURR, abi.VEC_STO_LAST)):
            if self.n_store:
                self.upload(vid, sto[k])

    def outputs(self):
        """F, Q, dFdxdVp, dQdxdVp (ground row dropped), next sta/sto, dFdx/dQdx values."""
        n = self.n_unknowns
        out = {
            "F": self.download(abi.VEC_F)[:n], "Q": self.download(abi.VEC_Q)[:n],
            "dFdxdVp": self.download(abi.VEC_DFDXDVP)[:n],
            "dQdxdVp": self.download(abi.VEC_DQDXDVP)[:n],
            "sta_next": self.download(abi.VEC_STA_NEXT), "sto_next": self.download(abi.VEC_STO_NEXT),
            "dFdx": self.download(abi.VEC_DFDX), "dQdx": self.download(abi.VEC_DQDX),
        }
        out["rows"] = np.repeat(np.arange(n, dtype=np.int32), np.diff(self.rowptr))
        out["cols"] = self.colidx.copy()
        return out


class LU:
    """Sparse LU of an n x n CSR matrix (the Newton-solve factorisation):
    host analysis at construction, GPU refactor and solve on device buffers
    (raw device pointers as ints)."""

    def __init__(self, ctx, rowptr, colidx, values, precision=abi.LU_FP64):
        self.ctx = ctx  # the context (its stream) must outlive the factorisation
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        self.colidx = np.ascontiguousarray(colidx, dtype=np.int32)
        vals = np.ascontiguousarray(values, dtype=np.float64)
        self.n = self.rowptr.size - 1
        h = C.c_void_p()
        check(lib().xg_lu_analyze(ctx.h, self.n, _ptr(self.rowptr), _ptr(self.colidx), _ptr(vals),
                                  precision, C.byref(h)))
        self.h = h
        _OPEN["lu"].add(self)
        info = abi.XgLuInfo()
        check(lib().xg_lu_get_info(h, C.byref(info)))
        self.info = info

    def refactor(self, dev_values):
        check(lib().xg_lu_refactor(self.h, C.c_void_p(dev_values)))

    def refactor_solve(self, dev_values, dev_b, dev_x, n_refine=0):
        check(lib().xg_lu_refactor_solve(self.h, C.c_void_p(dev_values), C.c_void_p(dev_b),
                                         C.c_void_p(dev_x), n_refine))

    def solve(self, dev_b, dev_x, n_refine=0):
        check(lib().xg_lu_solve(self.h, C.c_void_p(dev_b), C.c_void_p(dev_x), n_refine))

    def status(self):
        st, row = C.c_int(), C.c_int()
        check(lib().xg_lu_status(self.h, C.byref(st), C.byref(row)))
        return st.value, row.value

    def set_wait_limit(self, polls):
        """Polls a device wait makes before it gives up (status bit 2)."""
        check(lib().xg_lu_set_wait_limit(self.h, int(polls)))

    def symbolic(self):
        n, nnz = self.n, self.info.nnz_lu
        P, Q = np.zeros(n, np.int32), np.zeros(n, np.int32)
        rp, ci = np.zeros(n + 1, np.int32), np.zeros(nnz, np.int32)
        check(lib().xg_lu_get_symbolic(self.h, _ptr(P), _ptr(Q), _ptr(rp), _ptr(ci)))
        return P, Q, rp, ci

    def close(self):
        if getattr(self, "h", None):
            lib().xg_lu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lu_analyze_host(rowptr, colidx, values, with_info=False):
    """Host-only analysis: (P, Q, nnz of L\\U) of the CSR matrix, and its
    XgLuInfo when with_info."""
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colidx, dtype=np.int32)
    v = np.ascontiguousarray(values, dtype=np.float64)
    n = rp.size - 1
    P, Q = np.zeros(n, np.int32), np.zeros(n, np.int32)
    nnz = C.c_int64()
    info = abi.XgLuInfo()
    check(lib().xg_lu_analyze_host(n, _ptr(rp), _ptr(ci), _ptr(v), _ptr(P), _ptr(Q), C.byref(nnz),
                                   C.byref(info)))
    return (P, Q, nnz.value, info) if with_info else (P, Q, nnz.value)


def amd_order(rowptr, colidx):
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colidx, dtype=np.int32)
    n = rp.size - 1
    order = np.zeros(n, np.int32)
    nd = C.c_int()
    check(lib().xg_lu_order(n, _ptr(rp), _ptr(ci), _ptr(order), C.byref(nd)))
    return order, nd.value


def transient(circuit, tstop, tstep, out_idx, x0=None, uic=False, precision=abi.LU_FP64,
              n_refine=0, max_points=200000, maxstep=0.0, reltol=1e-3, abstol=1e-6):
    """DC operating point (from the guess x0, or x0 itself with uic) then
    .TRAN tstep tstop, all on the GPU; returns (t, V[len(t), len(out_idx)],
    stats dict)."""
    idx = np.ascontiguousarray(out_idx, np.int32)
    o = abi.XgTranOptions(tstop, tstep, maxstep, reltol, abstol, precision, n_refine, int(bool(uic)))
    x0a = None if x0 is None else np.ascontiguousarray(x0, np.float64)
    t = np.zeros(max_points)
    v = np.zeros((max_points, max(1, idx.size)))
    npts = C.c_int()
    st = abi.XgTranStats()
    check(lib().xg_tran_run(circuit.h, C.byref(o), None if x0a is None else _ptr(x0a), idx.size,
                            _ptr(idx), max_points, _ptr(t), _ptr(v), C.byref(npts), C.byref(st)))
    n = npts.value
    return t[:n], v[:n, : idx.size], st.as_dict()


class Batch:
    """Independent transients stepped together on the GPU (xg_batch_*): each
    request is a netlist, its initial condition x0 (its own unknown
    numbering), tstop and the unknowns to record."""

    def __init__(self, ctx, netlists, x0s, tstops, out_idx, tstep=1e-12, precision=abi.LU_FP64,
                 n_refine=0, max_points=4096, maxstep=0.0, reltol=1e-3, abstol=1e-6):
        self.ctx = ctx
        n = len(netlists)
        self._nl = [nl.to_c() for nl in netlists]
        self._keep = list(netlists)
        nl_arr = (C.c_void_p * n)(*[C.addressof(x) for x in self._nl])
        self._x0 = [np.ascontiguousarray(x, np.float64) for x in x0s]
        x0_arr = (C.c_void_p * n)(*[x.ctypes.data for x in self._x0])
        self._ts = np.ascontiguousarray(tstops, np.float64)
        self.n_out = len(out_idx[0])
        self._out = [np.ascontiguousarray(o, np.int32) for o in out_idx]
        out_arr = (C.c_void_p * n)(*[o.ctypes.data for o in self._out])
        self.max_points = max_points
        o = abi.XgBatchOptions(tstep, maxstep, reltol, abstol, precision, n_refine, self.n_out,
                               max_points)
        h = C.c_void_p()
        check(lib().xg_batch_create(ctx.h, n, nl_arr, x0_arr, _ptr(self._ts), out_arr, C.byref(o),
                                    C.byref(h)))
        self.h = h
        _OPEN["batch"].add(self)
        self.n = n

    def run(self, iterations):
        check(lib().xg_batch_run(self.h, iterations))

    def inflight(self):
        """Runs enqueued and not finished yet."""
        k = C.c_int()
        check(lib().xg_batch_inflight(self.h, C.byref(k)))
        return k.value

    def poll(self, wait=True):
        d = C.c_int()
        check(lib().xg_batch_poll(self.h, int(bool(wait)), C.byref(d)))
        return d.value

    def results(self, i):
        np_ = C.c_int()
        t = np.zeros(self.max_points)
        v = np.zeros((self.max_points, max(1, self.n_out)))
        st = abi.XgTranStats()
        check(lib().xg_batch_results(self.h, i, _ptr(t), _ptr(v), C.byref(np_), C.byref(st)))
        k = np_.value
        return t[:k], v[:k, : self.n_out], st.as_dict()

    def stats(self, i):
        """Request i's counters from the last poll; 'finished' once it is done."""
        np_ = C.c_int()
        st = abi.XgTranStats()
        check(lib().xg_batch_results(self.h, i, None, None, C.byref(np_), C.byref(st)))
        d = st.as_dict()
        d["points"] = np_.value
        d["finished"] = bool(st.status != 0 or st.t_end >= self._ts[i] * (1 - 1e-12))
        return d

    def device_bytes(self):
        nb, b = C.c_int(), C.c_int64()
        check(lib().xg_batch_info(self.h, C.byref(nb), C.byref(b)))
        return b.value

    def close(self):
        if getattr(self, "h", None):
            lib().xg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def slot_need(ctx, netlist, x0, tstop, tstep=1e-12):
    """The slot shape one request needs (its set-up, first Jacobian and
    pivot analysis, as a slotted batch does them)."""
    sh = abi.XgSlotShape()
    cnl = netlist.to_c()
    x = np.ascontiguousarray(x0, np.float64)
    check(lib().xg_slot_need(ctx.h, C.addressof(cnl), _ptr(x), float(tstop), float(tstep), C.byref(sh)))
    return sh


def batch_options(tstep=1e-12, precision=abi.LU_FP64, n_refine=0, n_out=2, max_points=4096, maxstep=0.0,
                  reltol=1e-3, abstol=1e-6):
    return abi.XgBatchOptions(tstep, maxstep, reltol, abstol, precision, n_refine, n_out, max_points)


def slot_bytes(shape, options):
    """Device bytes of one slot of this shape (host arithmetic, no device)."""
    b = C.c_int64()
    check(lib().xg_slot_bytes(C.byref(shape), C.byref(options), C.byref(b)))
    return b.value


def mem_info(ctx):
    f, t = C.c_int64(), C.c_int64()
    check(lib().xg_mem_info(ctx.h, C.byref(f), C.byref(t)))
    return f.value, t.value


class SlotBatch(Batch):
    """A slotted batch (xg_batch_create_slots): n_slots slots of one shape;
    requests are submitted into free slots while it runs and their slots
    released once their results are read."""

    def __init__(self, ctx, n_slots, shape, n_out, tstep=1e-12, precision=abi.LU_FP64, n_refine=0,
                 max_points=4096, maxstep=0.0, reltol=1e-3, abstol=1e-6):
        self.ctx = ctx
        self.shape = shape
        self.n_out, self.max_points = n_out, max_points
        o = batch_options(tstep, precision, n_refine, n_out, max_points, maxstep, reltol, abstol)
        h = C.c_void_p()
        check(lib().xg_batch_create_slots(ctx.h, n_slots, C.byref(shape), C.byref(o), C.byref(h)))
        self.h = h
        _OPEN["batch"].add(self)
        self.n = n_slots
        self._ts = np.zeros(n_slots)
        self._hold = [None] * n_slots

    def submit(self, netlists, x0s, tstops, out_idx):
        """Slots of the requests, -1 for those no free slot took."""
        n = len(netlists)
        if not n:
            return []
        cnl = [nl.to_c() for nl in netlists]
        nl_arr = (C.c_void_p * n)(*[C.addressof(x) for x in cnl])
        xs = [np.ascontiguousarray(x, np.float64) for x in x0s]
        x_arr = (C.c_void_p * n)(*[x.ctypes.data for x in xs])
        ts = np.ascontiguousarray(tstops, np.float64)
        outs = [np.ascontiguousarray(o, np.int32) for o in out_idx]
        o_arr = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
        slots = np.full(n, -1, np.int32)
        check(lib().xg_batch_submit(self.h, n, nl_arr, x_arr, _ptr(ts), o_arr, _ptr(slots)))
        for k, c in enumerate(slots):
            if c >= 0:
                self._ts[c] = ts[k]
        return [int(c) for c in slots]

    def release(self, slot):
        check(lib().xg_batch_release(self.h, int(slot)))

    def finished(self):
        """Slots whose request finished by the last poll, not yet released."""
        buf = np.zeros(self.n, np.int32)
        k = C.c_int()
        check(lib().xg_batch_finished(self.h, self.n, _ptr(buf), C.byref(k)))
        return [int(c) for c in buf[:k.value]]

    def slots(self):
        f, r = C.c_int(), C.c_int()
        check(lib().xg_batch_slots(self.h, C.byref(f), C.byref(r)))
        return f.value, r.value


def run_batch(batch, chunk=64, max_iters=10**7):
    """Step a batch until every request has finished; returns iterations run."""
    it = 0
    while it < max_iters:
        batch.run(chunk)
        it += chunk
        if batch.poll(wait=True) == batch.n:
            break
    return it
