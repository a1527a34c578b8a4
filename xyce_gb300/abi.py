"""ctypes mirror of include/xg.h: the netlist description, option and flag
structs shared by the engine (libxg), and plain-numpy builders for them.

A `Netlist` holds numpy arrays per device type; `Netlist.to_c()` returns an
`XgNetlist` ctypes struct whose pointers stay valid while the Netlist lives.
"""
import ctypes as C

import numpy as np

# device types (enum xg_dev_type)
DEV_RES, DEV_CAP, DEV_VSRC, DEV_ISRC, DEV_DIODE, DEV_MOS1, DEV_BSIM3 = range(7)
NUM_DEV_TYPES = 7
SRC_DC, SRC_PULSE = 0, 1

# vector ids (enum xg_vec_id)
(VEC_SOL_NEXT, VEC_SOL_CURR, VEC_SOL_LAST, VEC_STA_NEXT, VEC_STA_CURR, VEC_STA_LAST,
 VEC_STO_NEXT, VEC_STO_CURR, VEC_STO_LAST, VEC_F, VEC_Q, VEC_DFDXDVP, VEC_DQDXDVP,
 VEC_DFDX, VEC_DQDX) = range(15)

STATUS = {0: "XG_OK", -1: "XG_ERR_ARG", -2: "XG_ERR_CUDA", -3: "XG_ERR_OOM",
          -4: "XG_ERR_SINGULAR", -5: "XG_ERR_NAN", -6: "XG_ERR_TIMEOUT", -7: "XG_ERR_STATE",
          -8: "XG_ERR_UNSUPPORTED", -9: "XG_ERR_NOCONV"}

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class XgModelDesc(C.Structure):
    _fields_ = [("type", C.c_int), ("polarity", C.c_int), ("n_params", C.c_int),
                ("names", C.POINTER(C.c_char_p)), ("values", _dp)]


class XgMosDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("d", _ip), ("g", _ip), ("s", _ip), ("b", _ip), ("model", _ip),
                ("w", _dp), ("l", _dp), ("ad", _dp), ("as_", _dp), ("pd", _dp), ("ps", _dp),
                ("nrd", _dp), ("nrs", _dp), ("m", _dp)]


class XgDiodeDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("a", _ip), ("c", _ip), ("model", _ip), ("area", _dp)]


class XgTwoTermDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("p", _ip), ("m", _ip), ("value", _dp)]


class XgSrcDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("p", _ip), ("m", _ip), ("kind", _ip), ("wave", _dp)]


class XgNetlist(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_models", C.c_int), ("models", C.POINTER(XgModelDesc)),
                ("n_type_order", C.c_int), ("type_order", _ip),
                ("res", XgTwoTermDesc), ("cap", XgTwoTermDesc),
                ("vsrc", XgSrcDesc), ("isrc", XgSrcDesc),
                ("diode", XgDiodeDesc), ("mos1", XgMosDesc), ("bsim3", XgMosDesc)]


class XgDeviceOptions(C.Structure):
    _fields_ = [("gmin", C.c_double), ("temp", C.c_double), ("tnom", C.c_double),
                ("voltlim", C.c_int), ("newmeyer", C.c_int), ("fma", C.c_int)]


class XgLoadFlags(C.Structure):
    _fields_ = [("dcop", C.c_int), ("tranop", C.c_int), ("acop", C.c_int), ("transient", C.c_int),
                ("init_jct", C.c_int), ("init_fix", C.c_int), ("newton_iter", C.c_int),
                ("inputop", C.c_int), ("pdt", C.c_double), ("time", C.c_double),
                ("init_tran", C.c_int)]


class XgCircuitInfo(C.Structure):
    _fields_ = [("n_unknowns", C.c_int), ("n_state", C.c_int), ("n_store", C.c_int),
                ("nnz", C.c_int64), ("n_terms", C.c_int64), ("scratch_bytes", C.c_int64),
                ("n_instances", C.c_int * NUM_DEV_TYPES)]


LU_FP64, LU_FP32 = 0, 1


class XgLuInfo(C.Structure):
    _fields_ = [("n", C.c_int), ("nnz_a", C.c_int64), ("nnz_lu", C.c_int64),
                ("precision", C.c_int), ("levels", C.c_int), ("n_dense", C.c_int),
                ("refactor_flops", C.c_double), ("solve_flops", C.c_double),
                ("min_pivot", C.c_double), ("max_pivot", C.c_double), ("ordering", C.c_int),
                ("solve_chain", C.c_int)]


class XgTranOptions(C.Structure):
    _fields_ = [("tstop", C.c_double), ("tstep", C.c_double), ("maxstep", C.c_double),
                ("reltol", C.c_double), ("abstol", C.c_double), ("lu_precision", C.c_int),
                ("n_refine", C.c_int), ("uic", C.c_int)]


class XgTranStats(C.Structure):
    _fields_ = [("status", C.c_int), ("steps", C.c_int), ("steps_attempted", C.c_int),
                ("rejected", C.c_int), ("newton_iters", C.c_int), ("factorizations", C.c_int),
                ("loads", C.c_int), ("dcop_iters", C.c_int), ("dcop_solves", C.c_int),
                ("analyses", C.c_int), ("t_end", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class XgBatchOptions(C.Structure):
    _fields_ = [("tstep", C.c_double), ("maxstep", C.c_double), ("reltol", C.c_double),
                ("abstol", C.c_double), ("lu_precision", C.c_int), ("n_refine", C.c_int),
                ("n_out", C.c_int), ("max_points", C.c_int)]


class XgSlotShape(C.Structure):
    """The largest request one slot of a slotted batch holds."""
    _fields_ = [("max_unknowns", C.c_int), ("max_instances", C.c_int * NUM_DEV_TYPES),
                ("max_nnz", C.c_int64), ("max_lu_nnz", C.c_int64), ("max_schedule", C.c_int64),
                ("max_breakpoints", C.c_int)]

    def as_dict(self):
        return {"max_unknowns": self.max_unknowns, "max_instances": list(self.max_instances),
                "max_nnz": self.max_nnz, "max_lu_nnz": self.max_lu_nnz,
                "max_schedule": self.max_schedule, "max_breakpoints": self.max_breakpoints}

    @classmethod
    def from_dict(cls, d):
        s = cls()
        s.max_unknowns = int(d["max_unknowns"])
        for t, v in enumerate(d["max_instances"]):
            s.max_instances[t] = int(v)
        s.max_nnz, s.max_lu_nnz = int(d["max_nnz"]), int(d["max_lu_nnz"])
        s.max_schedule, s.max_breakpoints = int(d["max_schedule"]), int(d["max_breakpoints"])
        return s


def device_options(gmin=1e-12, temp=300.15, tnom=300.15, voltlim=1, newmeyer=0, fma=0):
    return XgDeviceOptions(gmin, temp, tnom, voltlim, newmeyer, fma)


def load_flags(dcop=0, tranop=0, acop=0, transient=1, init_jct=0, init_fix=0, newton_iter=1,
               inputop=0, pdt=0.0, time=0.0, init_tran=0):
    return XgLoadFlags(dcop, tranop, acop, transient, init_jct, init_fix, newton_iter, inputop,
                       pdt, time, init_tran)


_NAME_ARRAYS = {}  # parameter-name tuple -> (C array of names, its address); lives with the module
_MODEL_DTYPE = np.dtype([("type", "<i4"), ("polarity", "<i4"), ("n_params", "<i4"), ("pad", "<i4"),
                         ("names", "<u8"), ("values", "<u8")])


def _iarr(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _darr(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


class Model:
    """A .MODEL card: type (DEV_DIODE/DEV_MOS1/DEV_BSIM3), polarity (+1/-1), params."""

    def __init__(self, type_, polarity=1, **params):
        self.type = type_
        self.polarity = polarity
        self.params = {k.upper(): float(v) for k, v in params.items()}


class ModelSet:
    """Many .MODEL cards of one device type that give the same parameters
    (Monte-Carlo variants): polarity per card and a values[card, param]
    array.  A netlist keeps it as one entry that stands for len(self) cards
    with consecutive indices, and hands them to the C ABI without a Python
    loop over the cards."""

    def __init__(self, type_, polarity, **params):
        self.type = type_
        self.names = tuple(k.upper() for k in params)
        cols = [np.asarray(v, np.float64).reshape(-1) for v in params.values()]
        n = len(cols[0]) if cols else len(np.atleast_1d(polarity))
        self.values = np.ascontiguousarray(np.column_stack(cols) if cols else np.zeros((n, 0)))
        self.polarity = np.broadcast_to(np.asarray(polarity, np.int32), (n,)).copy()

    def __len__(self):
        return len(self.polarity)

    def cards(self):
        """The cards as Model objects."""
        for i in range(len(self)):
            m = Model(self.type, int(self.polarity[i]))
            m.params = dict(zip(self.names, (float(v) for v in self.values[i])))
            yield m


class Netlist:
    """Device arrays per type; node -1 is ground."""

    def __init__(self, n_nodes):
        self.n_nodes = int(n_nodes)
        self.models = []
        self.type_order = None
        self.res = None     # dict p, m, value
        self.cap = None
        self.vsrc = None    # dict p, m, kind, wave (n x 7)
        self.isrc = None
        self.diode = None   # dict a, c, model, area
        self.mos1 = None    # dict d, g, s, b, model, w, l, (ad, as, pd, ps, nrd, nrs, m)
        self.bsim3 = None

    def add_model(self, model):
        """Add a Model (returns its index) or a ModelSet (returns the indices
        of its cards)."""
        first = self.n_models
        self.models.append(model)
        if isinstance(model, ModelSet):
            return np.arange(first, first + len(model))
        return first

    @property
    def n_models(self):
        return sum(len(m) if isinstance(m, ModelSet) else 1 for m in self.models)

    def cards(self):
        """Every model card as a Model, in index order."""
        for m in self.models:
            if isinstance(m, ModelSet):
                yield from m.cards()
            else:
                yield m

    _GROUPS = ("res", "cap", "vsrc", "isrc", "diode", "mos1", "bsim3")

    def to_arrays(self):
        """Flat dict of numpy arrays (for np.savez); inverse of from_arrays."""
        out = {"n_nodes": np.array(self.n_nodes)}
        if self.type_order is not None:
            out["type_order"] = np.asarray(self.type_order, np.int32)
        for mi, m in enumerate(self.cards()):
            out[f"model{mi}.meta"] = np.array([m.type, m.polarity])
            out[f"model{mi}.names"] = np.array(list(m.params.keys()), dtype="U16")
            out[f"model{mi}.values"] = np.array(list(m.params.values()), np.float64)
        for g in self._GROUPS:
            d = getattr(self, g)
            if d is None:
                continue
            for k, v in d.items():
                if v is not None:
                    out[f"{g}.{k}"] = np.asarray(v)
        return out

    @classmethod
    def from_arrays(cls, a):
        nl = cls(int(a["n_nodes"]))
        if "type_order" in a:
            nl.type_order = [int(x) for x in a["type_order"]]
        mi = 0
        while f"model{mi}.meta" in a:
            t, pol = (int(x) for x in a[f"model{mi}.meta"])
            m = Model(t, pol)
            m.params = {str(k): float(v) for k, v in zip(a[f"model{mi}.names"], a[f"model{mi}.values"])}
            nl.models.append(m)
            mi += 1
        for g in cls._GROUPS:
            keys = [k for k in a if k.startswith(g + ".")]
            if keys:
                setattr(nl, g, {k[len(g) + 1:]: np.array(a[k]) for k in keys})
        return nl

    def count(self, t):
        d = [self.res, self.cap, self.vsrc, self.isrc, self.diode, self.mos1, self.bsim3][t]
        if d is None:
            return 0
        return len(d[next(iter(d))])

    def to_c(self):
        keep = []
        nl = XgNetlist()
        nl.n_nodes = self.n_nodes
        # the model cards as one array laid out like xg_model_desc, one value
        # buffer for every card, and name arrays shared by cards that give the
        # same parameters (Monte-Carlo variants give many such cards)
        nm = self.n_models
        mods = np.zeros(max(1, nm), dtype=_MODEL_DTYPE)
        allv = np.zeros(1)
        if nm:
            def names_addr(key):
                names = _NAME_ARRAYS.get(key)
                if names is None:
                    arr_ = (C.c_char_p * max(1, len(key)))(*[k.encode() for k in key])
                    names = _NAME_ARRAYS[key] = (arr_, C.addressof(arr_))
                return names[1]
            # per entry (a card or a set of cards): count, type, polarities,
            # parameter names and values
            cnt, typ, pol, lens, addr, vals = [], [], [], [], [], []
            for m in self.models:
                if isinstance(m, ModelSet):
                    n, k = len(m), len(m.names)
                    pol.append(m.polarity)
                    vals.append(m.values.reshape(-1))
                    key = m.names
                else:
                    n, k = 1, len(m.params)
                    pol.append(np.array([m.polarity], np.int32))
                    vals.append(np.fromiter(m.params.values(), np.float64, k))
                    key = tuple(m.params)
                cnt.append(n)
                typ.append(m.type)
                lens.append(k)
                addr.append(names_addr(key))
            cnt = np.asarray(cnt, np.int64)
            per_card = np.repeat(np.asarray(lens, np.int64), cnt)
            allv = _darr(np.concatenate(vals) if sum(len(v) for v in vals) else np.zeros(1))
            offs = np.concatenate(([0], np.cumsum(per_card)[:-1]))
            mods["type"][:nm] = np.repeat(np.asarray(typ, np.int32), cnt)
            mods["polarity"][:nm] = np.concatenate(pol)
            mods["n_params"][:nm] = per_card
            mods["names"][:nm] = np.repeat(np.asarray(addr, np.uint64), cnt)
            mods["values"][:nm] = np.uint64(allv.ctypes.data) + (8 * offs).astype(np.uint64)
        keep += [allv, mods]
        nl.n_models = nm
        nl.models = C.cast(mods.ctypes.data, C.POINTER(XgModelDesc))
        if self.type_order is not None:
            to = _iarr(self.type_order)
            keep.append(to)
            nl.n_type_order = len(to)
            nl.type_order = _p(to, _ip)

        def arr(d, k, f):
            if d is None or d.get(k) is None:
                return None
            a = f(d[k])
            keep.append(a)
            return a

        for field, d in (("res", self.res), ("cap", self.cap)):
            if d is not None:
                p, m, v = arr(d, "p", _iarr), arr(d, "m", _iarr), arr(d, "value", _darr)
                setattr(nl, field, XgTwoTermDesc(len(p), _p(p, _ip), _p(m, _ip), _p(v, _dp)))
        for field, d in (("vsrc", self.vsrc), ("isrc", self.isrc)):
            if d is not None:
                p, m, k = arr(d, "p", _iarr), arr(d, "m", _iarr), arr(d, "kind", _iarr)
                w = arr(d, "wave", lambda x: _darr(np.asarray(x).reshape(-1)))
                setattr(nl, field, XgSrcDesc(len(p), _p(p, _ip), _p(m, _ip), _p(k, _ip),
                                             _p(w, _dp)))
        if self.diode is not None:
            d = self.diode
            a, c_, mo = arr(d, "a", _iarr), arr(d, "c", _iarr), arr(d, "model", _iarr)
            ar = arr(d, "area", _darr)
            nl.diode = XgDiodeDesc(len(a), _p(a, _ip), _p(c_, _ip), _p(mo, _ip), _p(ar, _dp))
        for field, d in (("mos1", self.mos1), ("bsim3", self.bsim3)):
            if d is not None:
                ints = [arr(d, k, _iarr) for k in ("d", "g", "s", "b", "model")]
                dbl = [arr(d, k, _darr) for k in ("w", "l", "ad", "as", "pd", "ps", "nrd", "nrs", "m")]
                setattr(nl, field, XgMosDesc(len(ints[0]), *[_p(a, _ip) for a in ints],
                                             *[_p(a, _dp) for a in dbl]))
        nl._keep = keep
        return nl
