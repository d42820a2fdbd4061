"""ctypes binding of libgbsph.so (the C ABI declared in include/gbsph.h).

The library is built in tree by ``dualsphysics_gb300/csrc/Makefile``.  There
is no fallback: if the library is missing or fails to load, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "libgbsph.so")

GBSPH_OK = 0
ERRORS = {
    -1: "GBSPH_EINVAL", -2: "GBSPH_ECUDA", -3: "GBSPH_ENAN_DT", -4: "GBSPH_EBOUND_OUT",
    -5: "GBSPH_ECAPACITY", -6: "GBSPH_ENOMEM", -7: "GBSPH_ESTATE",
}
STEP_VERLET, STEP_SYMPLECTIC = 1, 2
VISCO_ARTIFICIAL, VISCO_LAMINARSPS, VISCO_LAMINAR = 1, 2, 3
DDT_NONE, DDT_DDT, DDT_DDT2, DDT_DDT2FULL = 0, 1, 2, 3
BC_DBC, BC_MDBC = 1, 2
INTERSTEP_VERLET, INTERSTEP_SYMPREDICTOR, INTERSTEP_SYMCORRECTOR = 1, 2, 3


class Params(C.Structure):
    _fields_ = [
        ("tstep", C.c_int), ("tvisco", C.c_int), ("tdensity", C.c_int), ("tboundary", C.c_int),
        ("verletsteps", C.c_int), ("dtallparticles", C.c_int), ("simulate2d", C.c_int), ("cellmode_div", C.c_int),
        ("dp", C.c_double), ("h", C.c_double), ("b", C.c_double), ("rhop0", C.c_double), ("gamma", C.c_double),
        ("massbound", C.c_double), ("massfluid", C.c_double), ("cflnumber", C.c_double),
        ("gravity", C.c_double * 3),
        ("visco", C.c_float), ("viscoboundfactor", C.c_float), ("ddtvalue", C.c_float), ("coefdtmin", C.c_float),
        ("rhopoutmin", C.c_float), ("rhopoutmax", C.c_float),
        ("dtini", C.c_double), ("dtmin", C.c_double),
        ("maprealposmin", C.c_double * 3), ("maprealposmax", C.c_double * 3),
        ("tshift", C.c_int), ("shiftcoef", C.c_float), ("shifttfs", C.c_float),
        ("peri", C.c_int * 3), ("periinc", C.c_double * 9),
    ]


class Consts(C.Structure):
    _fields_ = [
        ("tstep", C.c_int), ("tvisco", C.c_int), ("tdensity", C.c_int), ("tboundary", C.c_int),
        ("verletsteps", C.c_int), ("dtallparticles", C.c_int), ("simulate2d", C.c_int), ("cellmode_div", C.c_int),
        ("kernelh", C.c_float), ("kernelsize", C.c_float), ("kernelsize2", C.c_float), ("cteb", C.c_float),
        ("gamma", C.c_float), ("rhopzero", C.c_float), ("massfluid", C.c_float), ("massbound", C.c_float),
        ("eta2", C.c_float), ("ddtkh", C.c_float), ("ddtgz", C.c_float), ("visco", C.c_float),
        ("viscoboundfactor", C.c_float), ("awen", C.c_float), ("bwenh", C.c_float), ("spssmag", C.c_float),
        ("spsblin", C.c_float), ("scell", C.c_float), ("movlimit", C.c_float), ("rhopoutmin", C.c_float),
        ("rhopoutmax", C.c_float), ("gravity", C.c_float * 3),
        ("dp", C.c_double), ("cs0", C.c_double), ("cflnumber", C.c_double), ("dtmin", C.c_double),
        ("dtini", C.c_double),
        ("mapposmin", C.c_double * 3), ("maprealposmin", C.c_double * 3), ("maprealsize", C.c_double * 3),
        ("maprealposmax", C.c_double * 3),
        ("domposmin", C.c_double * 3), ("domrealposmin", C.c_double * 3), ("domrealposmax", C.c_double * 3),
        ("mapcells", C.c_uint * 3), ("domcells", C.c_uint * 3), ("domcellcode", C.c_uint),
        ("tshift", C.c_int), ("shiftcoef", C.c_float), ("shifttfs", C.c_float),
        ("peri", C.c_int * 3), ("periinc", C.c_double * 9), ("mapposmax", C.c_double * 3),
    ]


class DivInfo(C.Structure):
    _fields_ = [
        ("np", C.c_uint), ("npb", C.c_uint), ("npbok", C.c_uint), ("nout_total", C.c_uint),
        ("cellmin", C.c_uint * 3), ("ncells", C.c_uint * 3), ("nct", C.c_uint), ("nctt", C.c_uint),
        ("dividefull", C.c_uint), ("npfout", C.c_uint), ("npbout", C.c_uint),
    ]


class Mesh(C.Structure):
    """gbsph_mesh: a mesh gauge's grid (jmsh::StMeshBasic)."""
    _fields_ = [
        ("ptref", C.c_double * 3), ("vec1", C.c_double * 3), ("vec2", C.c_double * 3), ("vec3", C.c_double * 3),
        ("dis", C.c_double * 3), ("dispt", C.c_double * 3), ("dirdat", C.c_float * 3),
    ]


class Movement(C.Structure):
    """gbsph_movement: one predefined movement of a moving object."""
    _fields_ = [
        ("type", C.c_int), ("obj", C.c_uint), ("id", C.c_uint), ("nextid", C.c_uint), ("duration", C.c_double),
        ("angdegrees", C.c_int), ("prev", C.c_int), ("v", C.c_double * 3), ("a", C.c_double * 3),
        ("p", C.c_double * 3), ("axisp1", C.c_double * 3), ("axisp2", C.c_double * 3), ("s", C.c_double * 3),
    ]


class MotionEvent(C.Structure):
    _fields_ = [("obj", C.c_uint), ("mov", C.c_uint), ("start", C.c_double), ("finish", C.c_double)]


class MotionObject(C.Structure):
    _fields_ = [("idbegin", C.c_uint), ("count", C.c_uint)]


class MotionData(C.Structure):
    _fields_ = [("type", C.c_int), ("linmov", C.c_double * 3), ("linvel", C.c_double * 3),
                ("mat", C.c_double * 16)]


MOV_TYPES = {"wait": 1, "mvrect": 2, "mvrectace": 3, "mvrot": 4, "mvrotace": 5, "mvrectsinu": 6, "mvrotsinu": 7,
             "mvnull": 8}


TUNE_CANDIDATES = 8


class TuneResult(C.Structure):
    _fields_ = [("best", C.c_int), ("variant", C.c_int * TUNE_CANDIDATES), ("bsize", C.c_int * TUNE_CANDIDATES),
                ("split", C.c_int * TUNE_CANDIDATES), ("ms", C.c_float * TUNE_CANDIDATES),
                ("bound_best", C.c_int), ("bound_lanes", C.c_int * 3), ("bound_ms", C.c_float * 3),
                ("mdbc_best", C.c_int), ("mdbc_split", C.c_int * 3), ("mdbc_ms", C.c_float * 3)]


class Maxes(C.Structure):
    _fields_ = [("acemax", C.c_double), ("velmax", C.c_float), ("viscdtmax", C.c_float)]


# exported symbol -> (restype, argtypes); the same list the header declares
P = C.c_void_p
SIGNATURES = {
    "gbsph_config": (C.c_int, [C.POINTER(Params), C.POINTER(Consts)]),
    "gbsph_create": (C.c_int, [C.POINTER(Consts), C.c_uint, C.c_int, C.POINTER(P)]),
    "gbsph_destroy": (None, [P]),
    "gbsph_last_error": (C.c_char_p, [P]),
    "gbsph_upload": (C.c_int, [P, C.c_uint, C.c_uint, P, P, P, P, P]),
    "gbsph_upload_device": (C.c_int, [P, C.c_uint, C.c_uint, P, P, P, P, P]),
    "gbsph_divide": (C.c_int, [P]),
    "gbsph_mdbc": (C.c_int, [P, C.c_int]),
    "gbsph_forces": (C.c_int, [P, C.c_int, C.POINTER(Maxes)]),
    "gbsph_dtvariable": (C.c_int, [P, C.c_int, C.POINTER(C.c_double)]),
    "gbsph_symplectic_pre": (C.c_int, [P, C.c_double]),
    "gbsph_symplectic_cor": (C.c_int, [P, C.c_double]),
    "gbsph_verlet": (C.c_int, [P, C.c_double]),
    "gbsph_step": (C.c_int, [P]),
    "gbsph_run": (C.c_int, [P, C.c_uint, C.c_int]),
    "gbsph_step_dt": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gbsph_download": (C.c_int, [P, P, P, P, P, P]),
    "gbsph_get_forces": (C.c_int, [P, P, P]),
    "gbsph_get_divinfo": (C.c_int, [P, C.POINTER(DivInfo), P, C.c_uint, P, P]),
    "gbsph_get_maxes": (C.c_int, [P, C.POINTER(Maxes)]),
    "gbsph_sync": (C.c_int, [P]),
    "gbsph_launch_count": (C.c_ulonglong, [P]),
    "gbsph_stream": (P, [P]),
    "gbsph_set_option": (C.c_int, [P, C.c_int, C.c_int]),
    "gbsph_get_option": (C.c_int, [P, C.c_int, C.POINTER(C.c_int)]),
    "gbsph_set_step_state": (C.c_int, [P, C.c_double, C.c_double]),
    "gbsph_tune_forces": (C.c_int, [P, C.c_int, C.POINTER(TuneResult)]),
    "gbsph_tune_sort": (C.c_int, [P, C.c_int, C.POINTER(C.c_int), P]),
    "gbsph_ffma_peak": (C.c_int, [C.c_int, C.POINTER(C.c_float)]),
    "gbsph_ensemble_create": (C.c_int, [C.c_uint, C.POINTER(P), C.POINTER(P)]),
    "gbsph_ensemble_destroy": (None, [P]),
    "gbsph_ensemble_last_error": (C.c_char_p, [P]),
    "gbsph_ensemble_run": (C.c_int, [P, C.c_uint, C.c_int]),
    "gbsph_ensemble_sync": (C.c_int, [P]),
    "gbsph_ensemble_launches_per_step": (C.c_ulonglong, [P]),
    "gbsph_closure_set": (C.c_int, [P, P, C.c_float]),
    "gbsph_closure_features": (C.c_int, [P, P]),
    "gbsph_closure_fallbacks": (C.c_int, [P, C.POINTER(C.c_ulonglong)]),
    "gbsph_mlp_create": (C.c_int, [C.c_int, P, C.POINTER(P)]),
    "gbsph_mlp_destroy": (None, [P]),
    "gbsph_mlp_set_data": (C.c_int, [P, P, P, C.c_uint]),
    "gbsph_mlp_grad": (C.c_int, [P, C.c_uint, C.c_uint, P, P]),
    "gbsph_mlp_train": (C.c_int, [P, C.c_uint, C.c_uint, C.c_float, P]),
    "gbsph_mlp_infer": (C.c_int, [P, P, C.c_uint, P]),
    "gbsph_mlp_params": (C.c_int, [P, P, P]),
    "gbsph_graph_prepare": (C.c_int, [P, C.c_uint]),
    "gbsph_profile": (C.c_int, [P, C.c_uint]),
    "gbsph_profile_read": (C.c_int, [P, P, C.c_uint, C.POINTER(C.c_uint)]),
    "gbsph_mark": (C.c_int, [P, C.c_uint]),
    "gbsph_elapsed": (C.c_int, [P, C.c_uint, C.c_uint, C.POINTER(C.c_float)]),
    "gbsph_pips": (C.c_int, [P, C.POINTER(C.c_ulonglong * 4)]),
    "gbsph_sort_keys_noalloc": (C.c_int, [P, P, C.c_uint, C.c_uint, P, P]),
    "gbsph_gauge_velocity": (C.c_int, [P, C.c_uint, P, P]),
    "gbsph_gauge_swl": (C.c_int, [P, C.c_uint, P, P, P, P]),
    "gbsph_gauge_maxz": (C.c_int, [P, C.c_uint, P, P, P]),
    "gbsph_mesh_points": (C.c_int, [C.POINTER(Mesh), C.POINTER(C.c_uint * 3)]),
    "gbsph_gauge_mesh": (C.c_int, [P, C.POINTER(Mesh), C.c_float, C.c_float, C.c_float, P, P, P, P, P]),
    "gbsph_fluid_front": (C.c_int, [P, P, P, P, C.POINTER(C.c_double), C.POINTER(C.c_uint)]),
    "gbsph_motion_create": (C.c_int, [C.c_uint, P, C.c_uint, P, C.c_uint, P, C.c_int, C.POINTER(P)]),
    "gbsph_motion_destroy": (None, [P]),
    "gbsph_motion_process": (C.c_int, [P, C.c_double, C.c_double, P]),
    "gbsph_set_motion": (C.c_int, [P, P]),
    "gbsph_run_shifting": (C.c_int, [P, C.c_double]),
    "gbsph_get_shiftpos": (C.c_int, [P, P]),
}

SORT_NOALLOC_MAX_KEYS = 262144  # GBSPH_SORT_NOALLOC_MAX_KEYS

_lib = None
_lock = threading.Lock()


class GbsphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Loads libgbsph.so (raises if it is not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIBPATH):
                raise ImportError(f"libgbsph.so is not built ({LIBPATH}); run __graft_entry__.build() "
                                  "or make -C dualsphysics_gb300/csrc")
            L = C.CDLL(LIBPATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to libgbsph must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)


def config(params: Params) -> Consts:
    out = Consts()
    rc = lib().gbsph_config(C.byref(params), C.byref(out))
    if rc:
        raise GbsphError(rc, "gbsph_config failed")
    return out
