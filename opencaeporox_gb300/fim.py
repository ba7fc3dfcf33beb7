"""Host-side mirror of the reference's FIM method interface over the C ABI.

``FimContext`` exposes the calls IsoT_FIM makes on the bulk each Newton
iteration (src/IsoThermalMethod.cpp):

    ===========================  ==========================================
    reference (IsoT_FIM)          this module
    ===========================  ==========================================
    UpdateProperty (:811-836)     FimContext.update_property()
    CalRes (:1090-1185)           FimContext.cal_res(dt)
    AssembleMatBulks (:1187-1269) FimContext.assemble_mat(dt)
    GetSolution (:1282-1418)      FimContext.get_solution(u, dSmax)
    UpdateLastTimeStep (:1473)    FimContext.update_last_time_step()
    ===========================  ==========================================

State arrays use the reference's BulkVarSet layout (cell-major, then phase,
then component).  All numerical work runs in libocpx_gb300.so on the GPU; the
library must be built (``opencaeporox_gb300.build.build()``) and a CUDA device
must be present, otherwise every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libocpx_gb300.so")

# ---------------------------------------------------------------- C types --
OCPX_OK = 0
STATUS_NAMES = {0: "OK", 1: "NONCONVERGED", 2: "SINGULAR", 3: "NONFINITE", 4: "WATCHDOG", 5: "INVALID_ARG",
                6: "CUDA_ERROR", 7: "NEGATIVE_P", 8: "NEGATIVE_NI", 9: "NO_DEVICE"}

FIELDS = ["P", "T", "PB", "NI", "LNI", "NT", "VF", "VFP", "VFI", "PJ", "PC", "S", "PHASE_EXIST", "XIJ", "RHO",
          "XI", "MU", "RHOP", "XIP", "MUP", "RHOX", "XIX", "MUX", "KR", "DKRDS", "DPCDS", "DSEC_DPRI", "PORO",
          "POROP", "ROCKVP", "SKIP_FLAG", "SKIP_MINEIG", "SKIP_P", "SKIP_T", "SKIP_ZI", "STATUS", "FTYPE",
          "FLASH_ITERS", "UPBLOCK", "CONN_DP", "FLUX_VJ", "FLUX_NI", "RES", "RES_REL_V", "RES_REL_N", "TRANS",
          "PORO_INIT"]
FIELD_ID = {name: i for i, name in enumerate(FIELDS)}
FIELD_DTYPE = {"PHASE_EXIST": np.uint8, "SKIP_FLAG": np.uint8, "STATUS": np.uint32, "FTYPE": np.int8,
               "FLASH_ITERS": np.int32, "UPBLOCK": np.uint32}

# BulkVarSet / BulkConnVarSet names -> field ids (for loading reference dumps)
REF_NAMES = {"P": "P", "T": "T", "Pb": "PB", "Ni": "NI", "lNi": "LNI", "Nt": "NT", "vf": "VF", "vfP": "VFP",
             "vfi": "VFI", "Pj": "PJ", "Pc": "PC", "S": "S", "phaseExist": "PHASE_EXIST", "xij": "XIJ",
             "rho": "RHO", "xi": "XI", "mu": "MU", "rhoP": "RHOP", "xiP": "XIP", "muP": "MUP", "rhox": "RHOX",
             "xix": "XIX", "mux": "MUX", "kr": "KR", "dKrdS": "DKRDS", "dPcdS": "DPCDS",
             "dSec_dPri": "DSEC_DPRI", "poro": "PORO", "poroP": "POROP", "rockVp": "ROCKVP",
             "skip_flag": "SKIP_FLAG", "skip_minEigen": "SKIP_MINEIG", "skip_P": "SKIP_P", "skip_T": "SKIP_T",
             "skip_zi": "SKIP_ZI"}


class Well(C.Structure):
    """ocpx_well (include/ocpx.h)."""
    _fields_ = [("type", C.c_int), ("mode", C.c_int), ("bhp", C.c_double), ("tar_bhp", C.c_double),
                ("tar_rate", C.c_double), ("nperf", C.c_int), ("cell", C.POINTER(C.c_int)),
                ("WI", C.POINTER(C.c_double)), ("dG", C.POINTER(C.c_double)), ("xi_inj", C.POINTER(C.c_double)),
                ("inj_zi", C.POINTER(C.c_double)), ("factor", C.POINTER(C.c_double))]


class Table(C.Structure):
    _fields_ = [("nrow", C.c_int), ("ncol", C.c_int), ("data", C.POINTER(C.c_double))]


class ModelDesc(C.Structure):
    _fields_ = [("mixture", C.c_int), ("nc", C.c_int),
                ("gravity_factor", C.c_double), ("conv_darcy", C.c_double), ("gas_constant", C.c_double),
                ("conv1", C.c_double), ("conv3", C.c_double), ("conv4", C.c_double),
                ("rock_pref", C.c_double), ("rock_cp1", C.c_double), ("rock_cp2", C.c_double),
                ("swof", Table), ("sgof", Table), ("pvtw", Table), ("pvco", Table), ("pvdg", Table),
                ("std_rho_o", C.c_double), ("std_rho_g", C.c_double), ("std_rho_w", C.c_double),
                ("std_vo", C.c_double), ("std_vg", C.c_double), ("std_vw", C.c_double),
                ("Tc", C.POINTER(C.c_double)), ("Pc", C.POINTER(C.c_double)), ("Vc", C.POINTER(C.c_double)),
                ("MW", C.POINTER(C.c_double)), ("OmegaA", C.POINTER(C.c_double)),
                ("OmegaB", C.POINTER(C.c_double)), ("acf", C.POINTER(C.c_double)), ("BIC", C.POINTER(C.c_double)),
                ("Vshift", C.POINTER(C.c_double)), ("Vcvis", C.POINTER(C.c_double)),
                ("lbc_coef", C.POINTER(C.c_double)), ("flash_ctrl", C.POINTER(C.c_double)),
                ("skip_psa", C.c_int)]


class GridDesc(C.Structure):
    _fields_ = [("nb", C.c_int), ("nconn", C.c_int), ("v", C.POINTER(C.c_double)),
                ("depth", C.POINTER(C.c_double)), ("poro_init", C.POINTER(C.c_double)),
                ("conn_b", C.POINTER(C.c_uint32)), ("conn_e", C.POINTER(C.c_uint32)),
                ("conn_trans", C.POINTER(C.c_double)), ("nb_interior", C.c_int)]


class Options(C.Structure):
    """ocpx_options of ocpx_create_ex."""
    _fields_ = [("struct_size", C.c_size_t), ("recompute_flash_der", C.c_int), ("reserved", C.c_int * 7)]


class Report(C.Structure):
    _fields_ = [("status_or", C.c_uint32), ("n_two_phase", C.c_int), ("n_flagged", C.c_int)]


class Norms(C.Structure):
    _fields_ = [("maxRelRes_V", C.c_double), ("maxRelRes_N", C.c_double), ("maxId_V", C.c_int),
                ("maxId_N", C.c_int)]


class ChangeMax(C.Structure):
    """ocpx_change_max: signed maxima of one Newton iteration or time step."""
    _fields_ = [("dP", C.c_double), ("dT", C.c_double), ("dN", C.c_double), ("dS", C.c_double),
                ("eV", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SolveReport(C.Structure):
    """ocpx_solve_report."""
    _fields_ = [("iterations", C.c_int), ("relres", C.c_double), ("converged", C.c_int), ("breakdown", C.c_int)]


class NRControl(C.Structure):
    """ocpx_nr_control: ControlNRParam / ControlTimeParam values, the time step
    that ends, its Newton iterations, and the host-owned (well) terms."""
    _fields_ = [("maxIter", C.c_int), ("tol", C.c_double), ("dPmin", C.c_double), ("dSmin", C.c_double),
                ("maxIncreFac", C.c_double), ("minChopFac", C.c_double), ("dPlim", C.c_double),
                ("dSlim", C.c_double), ("timeMax", C.c_double), ("timeMin", C.c_double), ("end_time", C.c_double),
                ("current_dt", C.c_double), ("current_time", C.c_double), ("iterNR", C.c_int),
                ("maxWellRelRes_mol", C.c_double), ("dPWmaxT", C.c_double), ("res_from_host", C.c_int),
                ("maxRelRes_V", C.c_double), ("maxRelRes0_V", C.c_double), ("maxRelRes_N", C.c_double)]

    @classmethod
    def make(cls, **kw):
        c = cls()
        for k, v in kw.items():
            setattr(c, k, v)
        return c


EXPORTS = ["ocpx_abi_version", "ocpx_last_error", "ocpx_create", "ocpx_destroy", "ocpx_set_field",
           "ocpx_get_field", "ocpx_update_properties", "ocpx_calres", "ocpx_assemble", "ocpx_newton_update",
           "ocpx_update_last_step", "ocpx_synchronize", "ocpx_jacobian_dims", "ocpx_get_jacobian",
           "ocpx_jacobian_device", "ocpx_set_variant", "ocpx_step", "ocpx_enqueue_step", "ocpx_step_report",
           "ocpx_profile_enable", "ocpx_profile_read", "ocpx_checkpoint", "ocpx_measure_fp64_tflops",
           "ocpx_stream", "ocpx_launch_count", "ocpx_set_param", "ocpx_get_param", "ocpx_adjoint",
           "ocpx_nr_init_step", "ocpx_nr_max_change", "ocpx_step_max_change", "ocpx_nr_check_converge",
           "ocpx_next_time_step", "ocpx_linsolve", "ocpx_newton_update_device", "ocpx_wells_eval",
           "ocpx_set_field_range", "ocpx_get_field_range", "ocpx_set_adjoint_seed", "ocpx_get_adjoint",
           "ocpx_get_jacobian_rows", "ocpx_set_wells", "ocpx_get_wells", "ocpx_create_ex", "ocpx_linsolve_async",
           "ocpx_linsolve_report"]

PARAMS = {"flash_budget": 0, "coop_blocks": 1, "block_cell": 2, "deferred": 3, "predefer": 4, "coop_cells": 5,
          "predeferred": 6, "level": 7, "pre_blocks": 8,
          "cell_blocks": 9, "rounds": 10, "round_growth": 11,
          "fused_blocks": 12, "sms": 13, "fused_coop_blocks": 14,
          "fused_excl": 15, "post_block": 16, "recompute_flash_der": 17, "device_bytes": 18,
          "split_refill": 19}

_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load libocpx_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with opencaeporox_gb300.build.build()")
    lib = C.CDLL(path)
    P = C.c_void_p
    lib.ocpx_abi_version.restype = C.c_int
    lib.ocpx_last_error.restype = C.c_char_p
    lib.ocpx_create.argtypes = [C.POINTER(ModelDesc), C.POINTER(GridDesc), C.c_int, C.POINTER(P)]
    lib.ocpx_create_ex.argtypes = [C.POINTER(ModelDesc), C.POINTER(GridDesc), C.c_int, C.POINTER(Options),
                                   C.POINTER(P)]
    lib.ocpx_destroy.argtypes = [P]
    lib.ocpx_set_field.argtypes = [P, C.c_int, P, C.c_size_t]
    lib.ocpx_get_field.argtypes = [P, C.c_int, P, C.c_size_t]
    lib.ocpx_update_properties.argtypes = [P, C.POINTER(Report)]
    lib.ocpx_calres.argtypes = [P, C.c_double, C.POINTER(Norms)]
    lib.ocpx_assemble.argtypes = [P, C.c_double]
    lib.ocpx_newton_update.argtypes = [P, P, C.c_double]
    lib.ocpx_update_last_step.argtypes = [P]
    lib.ocpx_synchronize.argtypes = [P]
    lib.ocpx_jacobian_dims.argtypes = [P, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_int)]
    lib.ocpx_get_jacobian.argtypes = [P, P, P, P]
    lib.ocpx_set_variant.argtypes = [P, C.c_int]
    lib.ocpx_step.argtypes = [P, P, C.c_double, C.c_double, P, P, C.POINTER(Report)]
    lib.ocpx_checkpoint.argtypes = [P, C.c_int, C.c_int]
    lib.ocpx_enqueue_step.argtypes = [P, C.c_double]
    lib.ocpx_step_report.argtypes = [P, C.POINTER(Report)]
    lib.ocpx_profile_enable.argtypes = [P, C.c_int]
    lib.ocpx_profile_read.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
    lib.ocpx_measure_fp64_tflops.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.ocpx_adjoint.argtypes = [P, P, P, P, P]
    lib.ocpx_adjoint.restype = C.c_int
    lib.ocpx_set_param.argtypes = [P, C.c_int, C.c_longlong]
    lib.ocpx_nr_init_step.argtypes = [P]
    lib.ocpx_linsolve.argtypes = [P, C.c_double, C.c_int, P, C.POINTER(SolveReport)]
    lib.ocpx_linsolve_async.argtypes = [P, C.c_double, C.c_int]
    lib.ocpx_linsolve_report.argtypes = [P, C.POINTER(SolveReport)]
    lib.ocpx_newton_update_device.argtypes = [P, C.c_double]
    lib.ocpx_nr_max_change.argtypes = [P, C.POINTER(ChangeMax)]
    lib.ocpx_step_max_change.argtypes = [P, C.POINTER(ChangeMax)]
    lib.ocpx_nr_check_converge.argtypes = [P, C.POINTER(NRControl), C.POINTER(C.c_int)]
    lib.ocpx_next_time_step.argtypes = [P, C.POINTER(NRControl), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.ocpx_wells_eval.argtypes = [P, C.c_int, C.POINTER(Well), C.c_double, P, P, C.POINTER(C.c_double)]
    lib.ocpx_get_param.argtypes = [P, C.c_int, C.POINTER(C.c_longlong)]
    lib.ocpx_set_field_range.argtypes = [P, C.c_int, C.c_size_t, C.c_size_t, P]
    lib.ocpx_get_field_range.argtypes = [P, C.c_int, C.c_size_t, C.c_size_t, P]
    lib.ocpx_set_adjoint_seed.argtypes = [P, P]
    lib.ocpx_get_adjoint.argtypes = [P, P, P, P]
    lib.ocpx_get_jacobian_rows.argtypes = [P, C.c_size_t, C.c_size_t, P, P, P]
    lib.ocpx_set_wells.argtypes = [P, C.c_int, C.POINTER(Well)]
    lib.ocpx_get_wells.argtypes = [P, P, P]
    for fn in ("ocpx_enqueue_step", "ocpx_step_report", "ocpx_profile_enable", "ocpx_profile_read",
               "ocpx_measure_fp64_tflops", "ocpx_checkpoint", "ocpx_set_param", "ocpx_get_param"):
        getattr(lib, fn).restype = C.c_int
    lib.ocpx_stream.argtypes = [P]
    lib.ocpx_stream.restype = P
    lib.ocpx_launch_count.argtypes = [P]
    lib.ocpx_launch_count.restype = C.c_uint64
    for fn in EXPORTS:
        if fn not in ("ocpx_abi_version", "ocpx_last_error", "ocpx_stream", "ocpx_launch_count", "ocpx_destroy"):
            getattr(lib, fn).restype = C.c_int
    lib.ocpx_destroy.restype = None
    _lib = lib
    return lib


class OcpxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def _check(st: int):
    if st != OCPX_OK:
        raise OcpxError(st, load_library().ocpx_last_error().decode())


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


# ---------------------------------------------------------------- models ---
@dataclass
class Model:
    """ParamReservoir-level description: unit constants, rock, saturation and
    PVT tables, and for compositional models the EoS component data."""
    arrays: dict  # name -> np.ndarray, in the reference's storage

    @property
    def compositional(self) -> bool:
        return int(np.asarray(self.arrays["mixture_comp"]).ravel()[0]) == 1

    @property
    def nc(self) -> int:
        return int(np.asarray(self.arrays["nc"]).ravel()[0])

    def desc(self):
        """Build the C model description; returns (ModelDesc, keep-alive list)."""
        a = self.arrays
        keep = []

        def arr(name):
            v = np.ascontiguousarray(np.asarray(a[name], dtype=np.float64).ravel())
            keep.append(v)
            return v

        def table(name, ncol):
            if name not in a:
                return Table(0, 0, None)
            v = arr(name)
            nrow = int(np.asarray(a[name + "_nrow"]).ravel()[0])
            assert v.size == nrow * ncol, name
            return Table(nrow, ncol, _dptr(v))

        def scal(name, default=0.0):
            return float(np.asarray(a[name]).ravel()[0]) if name in a else default

        md = ModelDesc()
        md.mixture = 1 if self.compositional else 0
        md.nc = self.nc
        md.gravity_factor = scal("GRAVITY_FACTOR")
        md.conv_darcy = scal("CONV_DARCY")
        md.gas_constant = scal("GAS_CONSTANT")
        md.conv1 = scal("CONV1")
        md.conv3 = scal("CONV3")
        md.conv4 = scal("CONV4")
        md.rock_pref = scal("rock_Pref")
        md.rock_cp1 = scal("rock_cp1")
        md.rock_cp2 = scal("rock_cp2")
        md.swof = table("SWOF", 4)
        md.sgof = table("SGOF", 4)
        md.pvtw = table("PVTW", 5)
        md.std_rho_w = scal("stdRhoW")
        md.std_vw = scal("stdVw", 1.0)
        if self.compositional:
            for nm in ("Tc", "Pc", "Vc", "OmegaA", "OmegaB", "acf", "BIC", "Vshift", "Vcvis"):
                setattr(md, nm, _dptr(arr(nm)))
            md.MW = _dptr(arr("MWC"))
            md.lbc_coef = _dptr(arr("LBCcoef"))
            md.flash_ctrl = _dptr(arr("flash_ctrl"))
            md.skip_psa = int(scal("skipPSA", 1))
        else:
            md.pvco = table("PVCO", 6)
            md.pvdg = table("PVDG", 3)
            md.std_rho_o = scal("stdRhoO")
            md.std_rho_g = scal("stdRhoG")
            md.std_vo = scal("stdVo", 1.0)
            md.std_vg = scal("stdVg", 1.0)
        return md, keep


@dataclass
class Grid:
    """Bulk geometry and the connection list (bId < eId pairs in the
    reference's order) with transmissibilities.  A subdomain (halo.py) lists
    its interior cells first, nb_interior of them (0: all cells), then its
    ghost cells."""
    v: np.ndarray
    depth: np.ndarray
    poro_init: np.ndarray
    conn_b: np.ndarray
    conn_e: np.ndarray
    conn_trans: np.ndarray
    nb_interior: int = 0

    @property
    def nb(self):
        return len(self.v)

    @property
    def nconn(self):
        return len(self.conn_b)

    def desc(self):
        keep = [np.ascontiguousarray(self.v, np.float64), np.ascontiguousarray(self.depth, np.float64),
                np.ascontiguousarray(self.poro_init, np.float64), np.ascontiguousarray(self.conn_b, np.uint32),
                np.ascontiguousarray(self.conn_e, np.uint32), np.ascontiguousarray(self.conn_trans, np.float64)]
        g = GridDesc(self.nb, self.nconn, _dptr(keep[0]), _dptr(keep[1]), _dptr(keep[2]),
                     keep[3].ctypes.data_as(C.POINTER(C.c_uint32)), keep[4].ctypes.data_as(C.POINTER(C.c_uint32)),
                     _dptr(keep[5]), int(self.nb_interior))
        return g, keep


def model_and_grid_from_dump(arrays: dict, prefix: str = "model/"):
    """Model + Grid from the model dump of the reference (ParamReservoir,
    Bulk and BulkConn after setup), e.g. a golden fixture's ``model/*``."""
    m = {k[len(prefix):]: v for k, v in arrays.items() if k.startswith(prefix)}
    model = Model(m)
    grid = Grid(m["v"], m["depth"], m["poroInit"], m["conn_bId"], m["conn_eId"], m["conn_trans"])
    return model, grid


# --------------------------------------------------------------- context ---
class FimContext:
    """One GPU context holding the bulk state of a grid."""

    def __init__(self, model: Model, grid: Grid, device: int = -1, variant: int = 0, recompute: bool = False):
        """``recompute``: keep no dSec_dPri; the Jacobian, GetSolution and
        the wells recompute it from the flash's results (ocpx_options)."""
        self.lib = load_library()
        self.model = model
        self.grid = grid
        self.nb = grid.nb
        self.nbI = grid.nb_interior or grid.nb
        self.nwell = 0
        self.np = 3
        self.nc = model.nc
        self.nconn = grid.nconn
        self.NC = self.nc - 1 if model.compositional else 0
        md, k1 = model.desc()
        gd, k2 = grid.desc()
        h = C.c_void_p()
        opt = Options(C.sizeof(Options), 1 if recompute else 0)
        _check(self.lib.ocpx_create_ex(C.byref(md), C.byref(gd), device, C.byref(opt), C.byref(h)))
        self.h = h
        self.recompute = bool(recompute)
        if variant:
            self.set_variant(variant)

    def close(self):
        if getattr(self, "h", None):
            self.lib.ocpx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- fields
    def field_size(self, name: str) -> int:
        nb, np_, nc, nconn = self.nb, self.np, self.nc, self.nconn
        w = {"P": 1, "T": 1, "PB": 1, "NI": nc, "LNI": nc, "NT": 1, "VF": 1, "VFP": 1, "VFI": nc, "PJ": np_,
             "PC": np_, "S": np_, "PHASE_EXIST": np_, "XIJ": np_ * nc, "RHO": np_, "XI": np_, "MU": np_,
             "RHOP": np_, "XIP": np_, "MUP": np_, "RHOX": np_ * nc, "XIX": np_ * nc, "MUX": np_ * nc, "KR": np_,
             "DKRDS": np_ * np_, "DPCDS": np_ * np_, "DSEC_DPRI": np_ * (nc + 1) * (nc + 1), "PORO": 1,
             "POROP": 1, "ROCKVP": 1, "SKIP_FLAG": 1, "SKIP_MINEIG": 1, "SKIP_P": 1, "SKIP_T": 1,
             "SKIP_ZI": max(self.NC, 1), "STATUS": 1, "FTYPE": 1, "FLASH_ITERS": 5, "RES": nc + 1,
             "RES_REL_V": 1, "RES_REL_N": 1, "PORO_INIT": 1}
        cw = {"UPBLOCK": np_, "CONN_DP": np_, "FLUX_VJ": np_, "FLUX_NI": nc, "TRANS": 1}
        if name in cw:
            return nconn * cw[name]
        if name == "RES":
            return (nb + self.nwell) * (nc + 1)
        return nb * w[name]

    def set(self, name: str, values):
        dt = FIELD_DTYPE.get(name, np.float64)
        a = np.ascontiguousarray(np.asarray(values).astype(dt, copy=False).ravel())
        _check(self.lib.ocpx_set_field(self.h, FIELD_ID[name], a.ctypes.data_as(C.c_void_p), a.size))

    def get(self, name: str) -> np.ndarray:
        dt = FIELD_DTYPE.get(name, np.float64)
        out = np.empty(self.field_size(name), dtype=dt)
        _check(self.lib.ocpx_get_field(self.h, FIELD_ID[name], out.ctypes.data_as(C.c_void_p), out.size))
        return out

    def field_width(self, name: str) -> int:
        n = self.nconn if name in ("UPBLOCK", "CONN_DP", "FLUX_VJ", "FLUX_NI", "TRANS") else self.nb
        if name == "RES":
            n += self.nwell
        return self.field_size(name) // max(n, 1)

    def get_range(self, name: str, first: int, n: int) -> np.ndarray:
        """Entities [first, first + n) of a field, in the reference layout."""
        dt = FIELD_DTYPE.get(name, np.float64)
        out = np.empty(n * self.field_width(name), dtype=dt)
        _check(self.lib.ocpx_get_field_range(self.h, FIELD_ID[name], first, n, out.ctypes.data_as(C.c_void_p)))
        return out

    def set_range(self, name: str, first: int, values):
        """Write entities [first, first + n) of a field (n from the values)."""
        dt = FIELD_DTYPE.get(name, np.float64)
        a = np.ascontiguousarray(np.asarray(values).astype(dt, copy=False).ravel())
        w = self.field_width(name)
        if a.size % w:
            raise ValueError(f"{name}: {a.size} values are not whole entities of {w}")
        _check(self.lib.ocpx_set_field_range(self.h, FIELD_ID[name], first, a.size // w, a.ctypes.data_as(C.c_void_p)))

    def set_adjoint_seed(self, lam):
        """Adjoint products inside every step from now on (None: off)."""
        if lam is None:
            _check(self.lib.ocpx_set_adjoint_seed(self.h, None))
            return
        self._adj_seed = np.ascontiguousarray(np.asarray(lam, np.float64).ravel())
        if self._adj_seed.size != self.nv:
            raise ValueError(f"lambda must have {self.nv} entries")
        _check(self.lib.ocpx_set_adjoint_seed(self.h, self._adj_seed.ctypes.data_as(C.c_void_p)))

    def get_adjoint(self, out=None):
        """(J^T lam, (dR/dT)^T lam, (dR/dporoInit)^T lam) of the last step,
        into the arrays `out` when given."""
        jt, tr, po = out if out is not None else (np.empty(self.nv), np.empty(self.nconn), np.empty(self.nb))
        _check(self.lib.ocpx_get_adjoint(self.h, jt.ctypes.data_as(C.c_void_p), tr.ctypes.data_as(C.c_void_p),
                                         po.ctypes.data_as(C.c_void_p)))
        return jt, tr, po

    def load_state(self, state: dict, skip_missing: bool = True):
        """Upload arrays named as in BulkVarSet (P, Ni, S, xij, phaseExist, ...)."""
        for ref_name, fid in REF_NAMES.items():
            if ref_name not in state:
                if not skip_missing:
                    raise KeyError(ref_name)
                continue
            v = np.asarray(state[ref_name])
            if fid == "SKIP_ZI" and self.NC == 0:
                continue
            if fid == "DSEC_DPRI" and getattr(self, "recompute", False):
                continue  # not stored: recomputed from the flash's results
            if v.size != self.field_size(fid):
                continue
            self.set(fid, v)

    # ---- Newton step pieces
    def update_property(self) -> Report:
        rep = Report()
        _check(self.lib.ocpx_update_properties(self.h, C.byref(rep)))
        return rep

    def cal_res(self, dt: float) -> Norms:
        n = Norms()
        _check(self.lib.ocpx_calres(self.h, float(dt), C.byref(n)))
        return n

    def assemble_mat(self, dt: float):
        _check(self.lib.ocpx_assemble(self.h, float(dt)))
        _check(self.lib.ocpx_synchronize(self.h))

    @property
    def nv(self) -> int:
        """Entries of the residual, Newton update and adjoint vectors: nc + 1
        per cell and per well."""
        return (self.nb + self.nwell) * (self.nc + 1)

    def get_solution(self, u, dSmax: float):
        """GetSolution with a host Newton update u: its cells' entries, then
        the wells' rows when the context holds wells (nb*(nc+1) entries alone
        leave the wells' bhp unchanged).  Without wells on the context, rows
        past the cells (a host's own wells) are ignored."""
        a = np.ascontiguousarray(np.asarray(u, dtype=np.float64).ravel())
        ncell = self.nb * (self.nc + 1)
        if a.size < ncell:
            raise ValueError(f"u must have at least {ncell} entries")
        if self.nwell == 0:
            a = a[:ncell]
        elif a.size == ncell:
            a = np.concatenate([a, np.zeros(self.nwell * (self.nc + 1))])
        elif a.size != self.nv:
            raise ValueError(f"u must have {self.nv} entries")
        _check(self.lib.ocpx_newton_update(self.h, a.ctypes.data_as(C.c_void_p), float(dSmax)))
        _check(self.lib.ocpx_synchronize(self.h))

    def update_last_time_step(self):
        _check(self.lib.ocpx_update_last_step(self.h))

    def set_variant(self, v: int):
        _check(self.lib.ocpx_set_variant(self.h, int(v)))

    def set_param(self, name: str, value: int):
        """Execution tuning (results do not depend on it): flash_budget,
        coop_blocks, block_cell."""
        _check(self.lib.ocpx_set_param(self.h, PARAMS[name], int(value)))

    def get_param(self, name: str) -> int:
        v = C.c_longlong()
        _check(self.lib.ocpx_get_param(self.h, PARAMS[name], C.byref(v)))
        return int(v.value)

    def checkpoint(self, slot: int = 0, restore: bool = False):
        """Save / restore the whole bulk state on the device (ResetToLastTimeStep)."""
        _check(self.lib.ocpx_checkpoint(self.h, int(slot), 1 if restore else 0))

    def synchronize(self):
        _check(self.lib.ocpx_synchronize(self.h))

    def enqueue_step(self, dt: float):
        """Properties, residual and Jacobian enqueued without waiting."""
        _check(self.lib.ocpx_enqueue_step(self.h, float(dt)))

    def step_report(self) -> Report:
        rep = Report()
        _check(self.lib.ocpx_step_report(self.h, C.byref(rep)))
        return rep

    STAGES = ["check", "flash", "krpc_rock", "report", "flux", "residual", "jac_conn", "jac_rows", "newton_update",
              "flash_order", "flash_budget", "flash_coop", "flash_post", "flash_coop_late", "adjoint"]

    def profile(self, enable: bool = True):
        _check(self.lib.ocpx_profile_enable(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        ms = (C.c_double * len(self.STAGES))()
        n = (C.c_uint64 * len(self.STAGES))()
        _check(self.lib.ocpx_profile_read(self.h, ms, n))
        return {s: (ms[i], int(n[i])) for i, s in enumerate(self.STAGES)}

    def adjoint(self, lam, jt=True, trans=True, poro=True):
        """Vector-Jacobian products of the bulk residual at the last assembled
        state: (J^T lam, (dR/dT)^T lam, (dR/dporoInit)^T lam); None for the ones
        not requested."""
        lam = np.ascontiguousarray(np.asarray(lam, np.float64).ravel())
        if lam.size != self.nv:
            raise ValueError(f"lambda must have {self.nv} entries")
        out_jt = np.empty(lam.size) if jt else None
        out_t = np.empty(self.nconn) if trans else None
        out_p = np.empty(self.nb) if poro else None
        ptr = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
        _check(self.lib.ocpx_adjoint(self.h, ptr(lam), ptr(out_jt), ptr(out_t), ptr(out_p)))
        return out_jt, out_t, out_p

    # --- linear solve of the Newton system (bulk rows, on the device)
    def linsolve(self, tol: float = 1e-10, maxit: int = 2000, copy_out: bool = True):
        """BiCGStab with block-Jacobi preconditioning of J u = rhs (the last
        assembled Jacobian and residual); returns (u or None, report dict)."""
        rep = SolveReport()
        u = np.empty(self.nv) if copy_out else None
        _check(self.lib.ocpx_linsolve(self.h, float(tol), int(maxit),
                                      None if u is None else u.ctypes.data_as(C.c_void_p), C.byref(rep)))
        return u, {k: getattr(rep, k) for k, _ in rep._fields_}

    def linsolve_async(self, tol: float = 1e-10, maxit: int = 2000):
        """The same solve enqueued on the context stream without waiting
        (capturable in a CUDA graph on `stream`); read it with
        linsolve_report."""
        _check(self.lib.ocpx_linsolve_async(self.h, float(tol), int(maxit)))

    def linsolve_report(self):
        """Waits for the context stream; the report of the last solve."""
        rep = SolveReport()
        _check(self.lib.ocpx_linsolve_report(self.h, C.byref(rep)))
        return {k: getattr(rep, k) for k, _ in rep._fields_}

    def newton_update_device(self, dSmax: float):
        """GetSolution with the update the last linsolve left on the device."""
        _check(self.lib.ocpx_newton_update_device(self.h, float(dSmax)))

    # --- Newton-iteration and time-step control (bulk part, on the device)
    def nr_init_step(self):
        """OCPNRsuite::InitStep: the last Newton iterate := the last time step's
        state; the initial residual norm := that of the last cal_res."""
        _check(self.lib.ocpx_nr_init_step(self.h))

    def nr_max_change(self, read: bool = True):
        """OCPNRsuite::CalMaxChangeNR (bulk): signed maxima since the last call
        (left on the device, without a synchronisation, when read is False)."""
        if not read:
            _check(self.lib.ocpx_nr_max_change(self.h, None))
            return None
        out = ChangeMax()
        _check(self.lib.ocpx_nr_max_change(self.h, C.byref(out)))
        return out.as_dict()

    def step_max_change(self) -> dict:
        """OCPNRsuite::CalMaxChangeTime (bulk): signed maxima over the time step."""
        out = ChangeMax()
        _check(self.lib.ocpx_step_max_change(self.h, C.byref(out)))
        return out.as_dict()

    def nr_check_converge(self, ctrl: NRControl) -> int:
        """ControlNR::CheckConverge({"res", "d"}): 0 converged, 1 continue,
        2 not converged within maxIter."""
        st = C.c_int()
        _check(self.lib.ocpx_nr_check_converge(self.h, C.byref(ctrl), C.byref(st)))
        return st.value

    def next_time_step(self, ctrl: NRControl):
        """ControlTime::CalNextTimeStep({"dP", "dS", "iter"}): (next dt, predicted dt)."""
        dt, pdt = C.c_double(), C.c_double()
        _check(self.lib.ocpx_next_time_step(self.h, C.byref(ctrl), C.byref(dt), C.byref(pdt)))
        return dt.value, pdt.value

    def _wells_array(self, wells: list):
        """ocpx_well records of well dicts (and the arrays they point to)."""
        keep, arr = [], (Well * max(len(wells), 1))()
        for k, w in enumerate(wells):
            def dptr(key, n):
                v = w.get(key)
                if v is None:
                    return None
                a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
                assert a.size >= n, key
                keep.append(a)
                return a.ctypes.data_as(C.POINTER(C.c_double))
            cell = np.ascontiguousarray(np.asarray(w["cell"], dtype=np.int32).ravel())
            keep.append(cell)
            n = cell.size
            arr[k] = Well(int(w["type"]), int(w["mode"]), float(w["bhp"]), float(w.get("tar_bhp", 0.0)),
                          float(w.get("tar_rate", 0.0)), n, cell.ctypes.data_as(C.POINTER(C.c_int)),
                          dptr("WI", n), dptr("dG", n), dptr("xi_inj", n), dptr("inj_zi", self.nc),
                          dptr("factor", self.nc))
        return arr, keep

    def set_wells(self, wells: list):
        """Wells inside the Newton step (ocpx_set_wells): dicts with type,
        mode, bhp, tar_bhp, tar_rate, cell, WI (times the multiplier), dG,
        xi_inj, inj_zi, factor; [] removes them."""
        arr, keep = self._wells_array(wells)
        _check(self.lib.ocpx_set_wells(self.h, len(wells), arr))
        self.nwell = len(wells)

    def get_wells(self):
        """(bhp of each well, maxWellRelRes_mol of the last cal_res)."""
        bhp, mrel = np.empty(max(self.nwell, 1)), C.c_double()
        _check(self.lib.ocpx_get_wells(self.h, bhp.ctypes.data_as(C.c_void_p), C.byref(mrel)))
        return bhp[:self.nwell], mrel.value

    def wells_eval(self, wells: list, dt: float, residual: bool = True):
        """The wells' part of the residual and Jacobian (ocpx_wells_eval), for
        a host that keeps its own well code.  wells: dicts as for set_wells.
        Returns the residual with the wells ((nb + nwell) * (nc + 1); None
        without `residual`), the blocks as [nperf][3][nc+1][nc+1] (cell
        diagonal addition, cell-to-well, well-to-cell) and [nwell][nc+1][nc+1]
        (well diagonals), and maxWellRelRes_mol."""
        arr, keep = self._wells_array(wells)
        ncol = self.nc + 1
        nperf = sum(len(np.ravel(w["cell"])) for w in wells)
        res = np.empty((self.nb + len(wells)) * ncol)
        blocks = np.empty((3 * nperf + len(wells)) * ncol * ncol)
        mrel = C.c_double()
        _check(self.lib.ocpx_wells_eval(self.h, len(wells), arr, dt,
                                        res.ctypes.data_as(C.c_void_p) if residual else None,
                                        blocks.ctypes.data_as(C.c_void_p), C.byref(mrel)))
        pb = blocks[:3 * nperf * ncol * ncol].reshape(nperf, 3, ncol, ncol)
        wd = blocks[3 * nperf * ncol * ncol:].reshape(len(wells), ncol, ncol)
        return (res if residual else None), pb, wd, mrel.value

    def jacobian(self):
        nrow, nnz, bd = C.c_size_t(), C.c_size_t(), C.c_int()
        _check(self.lib.ocpx_jacobian_dims(self.h, C.byref(nrow), C.byref(nnz), C.byref(bd)))
        rp = np.empty(nrow.value + 1, np.uint32)   # interior cells' rows, then the wells'
        col = np.empty(nnz.value, np.uint32)
        val = np.empty(nnz.value * bd.value * bd.value, np.float64)
        _check(self.lib.ocpx_get_jacobian(self.h, rp.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
                                          val.ctypes.data_as(C.c_void_p)))
        return rp, col, val

    def jacobian_rows(self, r0: int, r1: int):
        """Rows [r0, r1) of the Jacobian: (rowptr relative to the first row,
        columns, block values)."""
        rp = np.empty(r1 - r0 + 1, np.uint32)
        _check(self.lib.ocpx_get_jacobian_rows(self.h, r0, r1, rp.ctypes.data_as(C.c_void_p), None, None))
        n = int(rp[-1] - rp[0])
        col = np.empty(n, np.uint32)
        val = np.empty(n * (self.nc + 1) ** 2)
        _check(self.lib.ocpx_get_jacobian_rows(self.h, r0, r1, rp.ctypes.data_as(C.c_void_p),
                                               col.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p)))
        return rp - rp[0], col, val

    def step(self, u=None, dSmax=0.2, dt=1.0, res_out=None, jac_out=None):
        rep = Report()
        up = None
        if u is not None:
            u = np.ascontiguousarray(u, dtype=np.float64)
            up = u.ctypes.data_as(C.c_void_p)
        rp = res_out.ctypes.data_as(C.c_void_p) if res_out is not None else None
        jp = jac_out.ctypes.data_as(C.c_void_p) if jac_out is not None else None
        _check(self.lib.ocpx_step(self.h, up, float(dSmax), float(dt), rp, jp, C.byref(rep)))
        return rep

    @property
    def stream(self):
        return self.lib.ocpx_stream(self.h)

    @property
    def launch_count(self) -> int:
        return int(self.lib.ocpx_launch_count(self.h))


def measure_fp64_tflops(device: int = 0, iters: int = 20000) -> float:
    """Measured FP64 FMA throughput of the device in TFLOP/s."""
    v = C.c_double()
    _check(load_library().ocpx_measure_fp64_tflops(device, iters, C.byref(v)))
    return v.value
