"""ctypes access to the oracle's C restatement (test infrastructure only).

``OracleBulk`` holds a full bulk state in the reference's BulkVarSet layout as
numpy arrays and runs the oracle's loops on it.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from opencaeporox_gb300.fim import ModelDesc  # noqa: E402  (shared description struct of include/ocpx.h)

_libs = {}


def lib(variant="exact"):
    """The oracle library; variant "ulp" is the one-ulp-perturbed build (oracle/ulp_nudge.c)."""
    if variant not in _libs:
        from oracle import build
        path = build.build(variant=variant)
        L = C.CDLL(path)
        P = C.c_void_p
        L.oc_create.argtypes = [C.POINTER(ModelDesc)]
        L.oc_create.restype = P
        L.oc_destroy.argtypes = [P]
        L.oc_check.argtypes = [P, P]
        L.oc_check.restype = C.c_int
        L.oc_flash.argtypes = [P, P, C.c_int, C.c_int]
        L.oc_krpc_rock.argtypes = [P, P, C.c_int, C.c_int]
        L.oc_calres.argtypes = [P, P, P, C.c_double, P, P, P, P]
        L.oc_assemble.argtypes = [P, P, P, C.c_double, P, P, P]
        L.oc_assemble.restype = C.c_long
        L.oc_newton_update.argtypes = [P, P, P, C.c_double]
        if variant == "ulp":
            L.oc_set_nudge_seed.argtypes = [C.c_uint64]
            L.oc_set_nudge_ulps.argtypes = [C.c_int]
        _libs[variant] = L
    return _libs[variant]


D = C.POINTER(C.c_double)
U = C.POINTER(C.c_uint32)
I = C.POINTER(C.c_int32)


class _Bulk(C.Structure):
    _fields_ = [("nb", C.c_int), ("np", C.c_int), ("nc", C.c_int), ("v", D), ("depth", D), ("poroInit", D),
                ("P", D), ("T", D), ("Pb", D), ("Ni", D), ("lNi", D), ("Nt", D), ("vf", D), ("vfP", D), ("vfi", D),
                ("Pj", D), ("Pc", D), ("S", D), ("phaseExist", U), ("xij", D), ("rho", D), ("xi", D), ("mu", D),
                ("rhoP", D), ("xiP", D), ("muP", D), ("rhox", D), ("xix", D), ("mux", D), ("kr", D), ("dKrdS", D),
                ("dPcdS", D), ("dSec_dPri", D), ("poro", D), ("poroP", D), ("rockVp", D), ("skip_flag", U),
                ("skip_minEig", D), ("skip_P", D), ("skip_T", D), ("skip_zi", D), ("ftype", I), ("iters", I)]


class _Conn(C.Structure):
    _fields_ = [("nconn", C.c_int), ("bId", U), ("eId", U), ("trans", D), ("upblock", U), ("dP", D),
                ("flux_vj", D), ("flux_ni", D)]


WIDTH = {"P": 1, "T": 1, "Pb": 1, "Ni": "nc", "lNi": "nc", "Nt": 1, "vf": 1, "vfP": 1, "vfi": "nc", "Pj": "np",
         "Pc": "np", "S": "np", "phaseExist": "np", "xij": "npnc", "rho": "np", "xi": "np", "mu": "np",
         "rhoP": "np", "xiP": "np", "muP": "np", "rhox": "npnc", "xix": "npnc", "mux": "npnc", "kr": "np",
         "dKrdS": "npnp", "dPcdS": "npnp", "dSec_dPri": "lend", "poro": 1, "poroP": 1, "rockVp": 1,
         "skip_flag": 1, "skip_minEig": 1, "skip_P": 1, "skip_T": 1, "skip_zi": "NC", "ftype": 1, "iters": 5}
ALIASES = {"skip_minEigen": "skip_minEig"}


class OracleModel:
    def __init__(self, model, variant="exact"):
        self.model = model
        self.lib = lib(variant)
        self._md, self._keep = model.desc()
        self.h = self.lib.oc_create(C.byref(self._md))

    def __del__(self):
        try:
            self.lib.oc_destroy(self.h)
        except Exception:
            pass


class OracleBulk:
    """Bulk + connections in the reference layout, driven by the oracle."""

    def __init__(self, model, grid, variant="exact"):
        self.om = OracleModel(model, variant)
        self.lib = self.om.lib
        self.nb, self.np, self.nc = grid.nb, 3, model.nc
        self.NC = model.nc - 1 if model.compositional else 0
        dims = {"nc": self.nc, "np": 3, "npnc": 3 * self.nc, "npnp": 9, "lend": 3 * (self.nc + 1) ** 2,
                "NC": max(self.NC, 1)}
        self.a = {}
        for k, w in WIDTH.items():
            n = self.nb * (w if isinstance(w, int) else dims[w])
            dt = np.uint32 if k in ("phaseExist", "skip_flag") else (np.int32 if k in ("ftype", "iters") else np.float64)
            self.a[k] = np.zeros(n, dt)
        self.grid = {"v": np.ascontiguousarray(grid.v, np.float64), "depth": np.ascontiguousarray(grid.depth, np.float64),
                     "poroInit": np.ascontiguousarray(grid.poro_init, np.float64)}
        nconn = grid.nconn
        self.conn = {"bId": np.ascontiguousarray(grid.conn_b, np.uint32), "eId": np.ascontiguousarray(grid.conn_e, np.uint32),
                     "trans": np.ascontiguousarray(grid.conn_trans, np.float64), "upblock": np.zeros(nconn * 3, np.uint32),
                     "dP": np.zeros(nconn * 3), "flux_vj": np.zeros(nconn * 3), "flux_ni": np.zeros(nconn * self.nc)}
        self.nconn = nconn
        self.res = np.zeros(self.nb * (self.nc + 1))
        self.resRelV = np.zeros(self.nb)
        self.resRelN = np.zeros(self.nb)
        self.norms = np.zeros(4)

    def set_nudge_seed(self, seed: int, ulps: int = 1):
        """Seed of the perturbation pattern and the ulps each transcendental
        result moves (variant "ulp" only)."""
        self.lib.oc_set_nudge_seed(seed)
        self.lib.oc_set_nudge_ulps(ulps)

    def load(self, state: dict):
        for k, v in state.items():
            k = ALIASES.get(k, k)
            if k in self.a and np.asarray(v).size == self.a[k].size:
                self.a[k][:] = np.asarray(v).ravel().astype(self.a[k].dtype)

    def _bulk(self):
        b = _Bulk()
        b.nb, b.np, b.nc = self.nb, 3, self.nc
        for k in ("v", "depth", "poroInit"):
            setattr(b, k, self.grid[k].ctypes.data_as(D))
        for k, arr in self.a.items():
            t = U if arr.dtype == np.uint32 else (I if arr.dtype == np.int32 else D)
            setattr(b, k, arr.ctypes.data_as(t))
        return b

    def _conn(self):
        c = _Conn()
        c.nconn = self.nconn
        for k, arr in self.conn.items():
            setattr(c, k, arr.ctypes.data_as(U if arr.dtype == np.uint32 else D))
        return c

    def check(self) -> int:
        b = self._bulk()
        return self.lib.oc_check(self.om.h, C.byref(b))

    def flash(self, n0=0, n1=None):
        b = self._bulk()
        self.lib.oc_flash(self.om.h, C.byref(b), n0, self.nb if n1 is None else n1)

    def krpc_rock(self, n0=0, n1=None):
        b = self._bulk()
        self.lib.oc_krpc_rock(self.om.h, C.byref(b), n0, self.nb if n1 is None else n1)

    def update_property(self) -> int:
        st = self.check()
        self.flash()
        self.krpc_rock()
        return st

    def cal_res(self, dt):
        b, c = self._bulk(), self._conn()
        self.lib.oc_calres(self.om.h, C.byref(b), C.byref(c), float(dt), self.res.ctypes.data_as(D),
                        self.resRelV.ctypes.data_as(D), self.resRelN.ctypes.data_as(D), self.norms.ctypes.data_as(D))
        return self.norms.copy()

    def assemble(self, dt):
        b, c = self._bulk(), self._conn()
        nnz_max = self.nb + 2 * self.nconn
        bs = (self.nc + 1) ** 2
        rp = np.zeros(self.nb + 1, np.uint32)
        col = np.zeros(nnz_max, np.uint32)
        val = np.zeros(nnz_max * bs)
        nnz = self.lib.oc_assemble(self.om.h, C.byref(b), C.byref(c), float(dt), rp.ctypes.data_as(U),
                                col.ctypes.data_as(U), val.ctypes.data_as(D))
        return rp, col[:nnz], val[: nnz * bs]

    def newton_update(self, u, dSmax):
        b = self._bulk()
        u = np.ascontiguousarray(u, np.float64)
        self.lib.oc_newton_update(self.om.h, C.byref(b), u.ctypes.data_as(D), float(dSmax))
