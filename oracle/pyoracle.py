"""ctypes binding of the oracle (oracle/liboracle.so, built by oracle/Makefile).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline legs use this module as the checker / timed CPU restatement of the
reference.  The product (dualsphysics_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "liboracle.so")
# the same source built with the reference's optimisation flags and without the
# conditioning sums (timed by bench.py's CPU legs, never used as a checker)
TIMING_LIBPATH = os.path.join(HERE, "liboracle_timing.so")


class OrcParams(C.Structure):
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


class OrcCtes(C.Structure):
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


class OrcDiv(C.Structure):
    _fields_ = [
        ("npb1", C.c_uint), ("npf1", C.c_uint), ("nptot", C.c_uint), ("dividefull", C.c_int),
        ("cellmin", C.c_uint * 3), ("cellmax", C.c_uint * 3),
        ("ncx", C.c_uint), ("ncy", C.c_uint), ("ncz", C.c_uint), ("nsheet", C.c_uint), ("nct", C.c_uint),
        ("nctt", C.c_uint),
        ("boxboundignore", C.c_uint), ("boxfluid", C.c_uint), ("boxboundout", C.c_uint), ("boxfluidout", C.c_uint),
        ("boxboundoutignore", C.c_uint), ("boxfluidoutignore", C.c_uint),
        ("boundlimitok", C.c_int), ("bounddivideok", C.c_int),
        ("boundlimitcellmin", C.c_uint * 3), ("boundlimitcellmax", C.c_uint * 3),
        ("bounddividecellmin", C.c_uint * 3), ("bounddividecellmax", C.c_uint * 3),
        ("npbignore", C.c_uint), ("npbout", C.c_uint), ("npfout", C.c_uint), ("npboutignore", C.c_uint),
        ("npfoutignore", C.c_uint), ("npfinal", C.c_uint), ("npbfinal", C.c_uint),
        ("npb2", C.c_uint), ("npf2", C.c_uint),
    ]


P = C.c_void_p
_SIG = {
    "orc_config": (C.c_int, [C.POINTER(OrcParams), C.POINTER(OrcCtes)]),
    "orc_calc_cellcode": (C.c_uint, [C.c_uint, C.c_uint, C.c_uint]),
    "orc_load_dcell": (None, [C.POINTER(OrcCtes), C.c_uint, P, P, P]),
    "orc_compute_press": (C.c_float, [C.POINTER(OrcCtes), C.c_float]),
    "orc_divide": (C.c_int, [C.POINTER(OrcCtes), C.POINTER(OrcDiv), C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_int, P, P, P, P, P,
                             C.c_uint]),
    "orc_interaction_forces": (None, [C.POINTER(OrcCtes), C.POINTER(OrcDiv), P, C.c_uint, C.c_uint, C.c_uint, P, P,
                                      P, P, P, P, P, P, C.POINTER(C.c_float), C.c_int, P]),
    "orc_interaction_forces_f64": (None, [C.POINTER(OrcCtes), C.POINTER(OrcDiv), P, C.c_uint, C.c_uint, C.c_uint,
                                          P, P, P, P, P, P, P, P, C.POINTER(C.c_double), C.c_int, P, P, P, P]),
    "orc_mdbc_correction": (None, [C.POINTER(OrcCtes), C.POINTER(OrcDiv), P, C.c_uint, P, P, P, P, C.c_int]),
    "orc_pips": (None, [C.POINTER(OrcCtes), C.POINTER(OrcDiv), P, C.c_uint, C.c_uint, C.c_uint, P, P,
                        C.POINTER(C.c_ulonglong * 4), C.c_int]),
    "orc_dtvariable": (C.c_double, [C.POINTER(OrcCtes), C.c_double, C.c_float, C.c_float, C.POINTER(C.c_int)]),
    "orc_sim_create": (P, [C.POINTER(OrcCtes), C.c_uint, C.c_uint, P, P, P, P, P, C.c_int]),
    "orc_sim_destroy": (None, [P]),
    "orc_sim_run_cell_divide": (C.c_int, [P]),
    "orc_sim_mdbc": (C.c_int, [P, C.c_int]),
    "orc_sim_interaction": (C.c_int, [P]),
    "orc_sim_dtvariable": (C.c_double, [P, C.POINTER(C.c_int)]),
    "orc_sim_symplectic_pre": (C.c_int, [P, C.c_double]),
    "orc_sim_symplectic_cor": (C.c_int, [P, C.c_double]),
    "orc_sim_verlet": (C.c_int, [P, C.c_double]),
    "orc_sim_run_shifting": (C.c_int, [P, C.c_double]),
    "orc_sim_get_shiftpos": (None, [P, P]),
    "orc_sim_set_shiftpos": (None, [P, P]),
    "orc_sim_step": (C.c_int, [P, C.POINTER(C.c_double)]),
    "orc_sim_np": (C.c_uint, [P]),
    "orc_sim_npb": (C.c_uint, [P]),
    "orc_sim_npbok": (C.c_uint, [P]),
    "orc_sim_div": (C.POINTER(OrcDiv), [P]),
    "orc_sim_get": (None, [P, P, P, P, P, P]),
    "orc_sim_get_forces": (None, [P, P, P]),
    "orc_sim_get_begincell": (None, [P, P, C.c_uint]),
    "orc_sim_get_sortpart": (None, [P, P, P]),
    "orc_sim_maxes": (None, [P, C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_float),
                             C.POINTER(C.c_double)]),
    "orc_sim_set_dtpre": (None, [P, C.c_double]),
    "orc_sim_set_forces": (None, [P, P, P]),
    "orc_sim_set_state": (None, [P, P, P]),
    "orc_sim_nout": (C.c_uint, [P]),
    "orc_sim_time": (C.c_double, [P]),
    "orc_sim_times": (None, [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "orc_set_sampling": (None, [C.c_int, C.c_int]),
    "orc_sim_mdbc_f64": (None, [C.c_void_p, C.c_void_p]),
}

_L = None
_PATH = LIBPATH


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def use_timing_build() -> None:
    """Makes this process load the timing build (call before the first use)."""
    global _PATH
    if _L is not None and _PATH != TIMING_LIBPATH:
        raise RuntimeError("the checker build of the oracle is already loaded")
    _PATH = TIMING_LIBPATH


def lib() -> C.CDLL:
    global _L
    if _L is None:
        if not os.path.exists(_PATH):
            build()
        L = C.CDLL(_PATH)
        for k, (r, a) in _SIG.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _L = L
    return _L


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def params_from(prm) -> OrcParams:
    """Copies a product Params (same field layout) into the oracle's struct."""
    o = OrcParams()
    C.memmove(C.byref(o), C.byref(prm), C.sizeof(OrcParams))
    return o


def config(prm: OrcParams) -> OrcCtes:
    c = OrcCtes()
    rc = lib().orc_config(C.byref(prm), C.byref(c))
    if rc:
        raise ValueError("orc_config failed")
    return c


class Sim:
    """Oracle solver state (JSphCpuSingle arrays and step driver)."""

    def __init__(self, ctes: OrcCtes, pos, velrho, idp, code, npb, boundnor=None, nthreads=0):
        self.ctes = ctes
        self._keep = [np.ascontiguousarray(pos, np.float64), np.ascontiguousarray(velrho, np.float32),
                      np.ascontiguousarray(idp, np.uint32), np.ascontiguousarray(code, np.uint16),
                      None if boundnor is None else np.ascontiguousarray(boundnor, np.float32)]
        n = len(idp)
        self.h = lib().orc_sim_create(C.byref(ctes), n, npb, *[_p(a) for a in self._keep], nthreads)
        if not self.h:
            raise RuntimeError("orc_sim_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sim_destroy(self.h)
            self.h = None

    @property
    def np(self):
        return lib().orc_sim_np(self.h)

    @property
    def npb(self):
        return lib().orc_sim_npb(self.h)

    @property
    def npbok(self):
        return lib().orc_sim_npbok(self.h)

    def div(self) -> OrcDiv:
        return lib().orc_sim_div(self.h).contents

    def state(self):
        n = self.np
        pos = np.empty((n, 3), np.float64)
        vr = np.empty((n, 4), np.float32)
        idp = np.empty(n, np.uint32)
        code = np.empty(n, np.uint16)
        dcell = np.empty(n, np.uint32)
        lib().orc_sim_get(self.h, _p(pos), _p(vr), _p(idp), _p(code), _p(dcell))
        return {"pos": pos, "velrho": vr, "idp": idp, "code": code, "dcell": dcell}

    def forces(self):
        n = self.np
        ace = np.empty((n, 3), np.float32)
        ar = np.empty(n, np.float32)
        lib().orc_sim_get_forces(self.h, _p(ace), _p(ar))
        return ace, ar

    def begincell(self):
        d = self.div()
        out = np.empty(d.nctt, np.uint32)
        lib().orc_sim_get_begincell(self.h, _p(out), d.nctt)
        return out

    def sortpart(self):
        d = self.div()
        sp = np.empty(d.nptot, np.uint32)
        cp = np.empty(d.nptot, np.uint32)
        lib().orc_sim_get_sortpart(self.h, _p(sp), _p(cp))
        return sp, cp

    def maxes(self):
        a, v, vi, d = C.c_double(), C.c_float(), C.c_float(), C.c_double()
        lib().orc_sim_maxes(self.h, C.byref(a), C.byref(v), C.byref(vi), C.byref(d))
        return {"acemax": a.value, "velmax": v.value, "viscdtmax": vi.value, "dtpre": d.value}

    def divide(self):
        rc = lib().orc_sim_run_cell_divide(self.h)
        if rc:
            raise RuntimeError(f"oracle divide failed rc={rc}")

    def mdbc(self, corrector=False):
        lib().orc_sim_mdbc(self.h, int(corrector))

    def interaction(self):
        lib().orc_sim_interaction(self.h)

    def dtvariable(self):
        e = C.c_int()
        dt = lib().orc_sim_dtvariable(self.h, C.byref(e))
        if e.value:
            raise FloatingPointError("dt is NaN/inf")
        return dt

    def symplectic_pre(self, dt):
        lib().orc_sim_symplectic_pre(self.h, dt)

    def symplectic_cor(self, dt):
        lib().orc_sim_symplectic_cor(self.h, dt)

    def verlet(self, dt):
        lib().orc_sim_verlet(self.h, dt)

    def run_shifting(self, dt):
        lib().orc_sim_run_shifting(self.h, dt)

    def shiftpos(self):
        out = np.empty((self.np, 4), np.float32)
        lib().orc_sim_get_shiftpos(self.h, _p(out))
        return out

    def set_shiftpos(self, sh):
        lib().orc_sim_set_shiftpos(self.h, _p(np.ascontiguousarray(sh, np.float32)))

    def step(self):
        dt = C.c_double()
        rc = lib().orc_sim_step(self.h, C.byref(dt))
        if rc:
            raise RuntimeError(f"oracle step failed rc={rc}")
        return dt.value

    def set_dtpre(self, dt):
        lib().orc_sim_set_dtpre(self.h, dt)

    def set_state(self, pos=None, velrho=None):
        self._s = (None if pos is None else np.ascontiguousarray(pos, np.float64),
                   None if velrho is None else np.ascontiguousarray(velrho, np.float32))
        lib().orc_sim_set_state(self.h, _p(self._s[0]), _p(self._s[1]))

    def set_forces(self, ace, ar):
        self._f = (np.ascontiguousarray(ace, np.float32), np.ascontiguousarray(ar, np.float32))
        lib().orc_sim_set_forces(self.h, _p(self._f[0]), _p(self._f[1]))

    def time(self):
        return lib().orc_sim_time(self.h)

    def times(self):
        a, b = C.c_double(), C.c_double()
        lib().orc_sim_times(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def nout(self):
        return lib().orc_sim_nout(self.h)


def forces_f64(sim: Sim):
    """FP64 evaluation of Interaction_Forces on the oracle's current state."""
    st = sim.state()
    d = sim.div()
    bc = sim.begincell()
    n = sim.np
    ace = np.zeros((n, 3), np.float64)
    ar = np.zeros(n, np.float64)
    strain = np.zeros((n, 6), np.float64)
    tau = np.zeros((n, 6), np.float64)
    visc = C.c_double()
    absace = np.zeros(n, np.float64)
    absar = np.zeros(n, np.float64)
    shift = np.zeros((n, 4), np.float64)
    absshift = np.zeros(n, np.float64)
    lib().orc_interaction_forces_f64(C.byref(sim.ctes), C.byref(d), _p(bc), n, sim.npb, sim.npbok,
                                     _p(st["dcell"]), _p(st["pos"]), _p(st["velrho"]), _p(st["code"]), _p(tau),
                                     _p(ace), _p(ar), _p(strain), C.byref(visc), 0, _p(absace), _p(absar),
                                     _p(shift), _p(absshift))
    return {"ace": ace, "ar": ar, "viscdt": visc.value, "absace": absace, "absar": absar, "shiftpos": shift,
            "absshift": absshift}


def mdbc_f64(sim: Sim) -> np.ndarray:
    """FP64 evaluation of the mDBC corrected densities of the boundary rows
    (npbok) on the oracle's current state; the state is not changed."""
    out = np.empty(sim.npbok, np.float64)
    lib().orc_sim_mdbc_f64(sim.h, _p(out))
    return out


def pips(sim: Sim):
    st = sim.state()
    d = sim.div()
    bc = sim.begincell()
    out = (C.c_ulonglong * 4)()
    lib().orc_pips(C.byref(sim.ctes), C.byref(d), _p(bc), sim.np, sim.npb, sim.npbok, _p(st["dcell"]),
                   _p(st["pos"]), C.byref(out), 0)
    return {"checked_bound": out[0], "real_bound": out[1], "checked_fluid": out[2], "real_fluid": out[3]}
