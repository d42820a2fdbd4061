"""Host-side driver mirroring the reference's JSphGpuSingle (Run/ComputeStep).

``GbSphSingle`` exposes the reference's step surface (JSphGpuSingle.cpp:372-1010,
JSphGpu.cpp:846-1150) over the C ABI of libgbsph.so:

* ``LoadCase`` = LoadConfig + LoadCaseParticles + ConfigDomain (constants,
  particles, first cell division),
* ``RunCellDivide``, ``MdbcBoundCorrection``, ``Interaction_Forces``,
  ``DtVariable``, ``ComputeSymplecticPre``/``ComputeSymplecticCorr``,
  ``ComputeVerlet`` and ``ComputeStep_Sym`` for step-by-step use,
* ``ComputeStep`` / ``RunSteps``: the device-resident step (dt never leaves the
  GPU; optionally replayed from a captured CUDA graph),
* ``Run``: the main loop with ``data/Part_%04u.bi4`` output every TimeOut
  (JSph::SaveData, JSph.cpp:3062-3110, 3209).

All compute runs in libgbsph's CUDA kernels; a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import bi4
from ._lib import (DivInfo, GbsphError, INTERSTEP_SYMCORRECTOR, INTERSTEP_SYMPREDICTOR, Maxes, STEP_SYMPLECTIC,
                   config, lib, ptr)
from .case import CaseData, load_case


CODE_MASKSPECIAL = 0xE000


def default_capacity(cd: CaseData) -> int:
    """Particles to allocate for a case: its particles, plus room for the
    periodic copies.  A particle has at most 2^k - 1 copies over k periodic
    axes (one per axis and per combination of axes, the period being longer
    than twice the kernel size), and while RunPeriodic appends the new copies
    the copies of the last divide are still in the arrays: np * (1 + 2 (2^k - 1))."""
    nperi = sum(1 for k in cd.params.peri if k)
    return int(cd.np * (1 + 2 * ((1 << nperi) - 1)))


def normal_rows(code: np.ndarray) -> np.ndarray:
    """Rows whose code is normal (CODE_IsNormal): particles of the case, not
    their periodic copies."""
    return (code & CODE_MASKSPECIAL) == 0


class GbSphSingle:
    def __init__(self, device: int = 0):
        self.device = device
        self.ctx = C.c_void_p()
        self.consts = None
        self.case: CaseData | None = None
        self.timestep = 0.0
        self.nstep = 0
        self.part = 0
        self.dirout = None
        self.motion = C.c_void_p()   # gbsph_motion of a case with moving boundaries

    # ---- lifetime -------------------------------------------------------
    def _check(self, rc: int, what: str):
        if rc:
            msg = lib().gbsph_last_error(self.ctx).decode() if self.ctx else what
            raise GbsphError(rc, f"{what}: {msg}")

    def close(self):
        if self.ctx:
            lib().gbsph_destroy(self.ctx)
            self.ctx = C.c_void_p()
        if self.motion:
            lib().gbsph_motion_destroy(self.motion)
            self.motion = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def LoadCase(self, casedir: str, casename: str, capacity: int | None = None, cellmode: str = "full") -> None:
        """LoadConfig + LoadCaseParticles + ConfigDomain (JSphGpuSingle.cpp:151-240)."""
        self.case = cd = load_case(casedir, casename, cellmode)
        self.setup(cd, capacity)

    def setup(self, cd: CaseData, capacity: int | None = None) -> None:
        self.case = cd
        self.consts = config(cd.params)
        self.close()
        cap = int(capacity or default_capacity(cd))
        self._check(lib().gbsph_create(C.byref(self.consts), cap, self.device, C.byref(self.ctx)), "gbsph_create")
        self._check(lib().gbsph_upload(self.ctx, cd.np, cd.npb, ptr(cd.pos), ptr(cd.velrho), ptr(cd.idp),
                                       ptr(cd.code), ptr(cd.boundnor)), "gbsph_upload")
        if cd.motion:  # JSph::LoadCaseConfig -> JDsMotion::Init (JSph.cpp:1064-1067)
            from .case import motion_structs
            objs, movs, nmov, evts, nevt = motion_structs(cd.motion)
            self._check(lib().gbsph_motion_create(len(cd.motion["objects"]), objs, nmov, movs, nevt, evts,
                                                  int(cd.params.simulate2d), C.byref(self.motion)),
                        "gbsph_motion_create")
            self._check(lib().gbsph_set_motion(self.ctx, self.motion), "gbsph_set_motion")
        self.timestep = 0.0
        self.nstep = 0

    # ---- step pieces (JSphGpuSingle protected surface) -------------------
    def RunCellDivide(self) -> None:
        self._check(lib().gbsph_divide(self.ctx), "RunCellDivide")

    def MdbcBoundCorrection(self, interstep: int) -> None:
        self._check(lib().gbsph_mdbc(self.ctx, interstep), "MdbcBoundCorrection")

    def Interaction_Forces(self, interstep: int) -> dict:
        m = Maxes()
        self._check(lib().gbsph_forces(self.ctx, interstep, C.byref(m)), "Interaction_Forces")
        return {"acemax": m.acemax, "velmax": m.velmax, "viscdtmax": m.viscdtmax}

    def DtVariable(self, final: bool) -> float:
        dt = C.c_double()
        self._check(lib().gbsph_dtvariable(self.ctx, int(final), C.byref(dt)), "DtVariable")
        return dt.value

    def ComputeSymplecticPre(self, dt: float) -> None:
        self._check(lib().gbsph_symplectic_pre(self.ctx, dt), "ComputeSymplecticPre")

    def ComputeSymplecticCorr(self, dt: float) -> None:
        self._check(lib().gbsph_symplectic_cor(self.ctx, dt), "ComputeSymplecticCorr")

    def ComputeVerlet(self, dt: float) -> None:
        self._check(lib().gbsph_verlet(self.ctx, dt), "ComputeVerlet")

    def RunShifting(self, dt: float) -> None:
        """JSphCpu::RunShifting: shifting sums -> displacements (no-op without shifting)."""
        self._check(lib().gbsph_run_shifting(self.ctx, dt), "RunShifting")

    def shiftpos(self) -> np.ndarray:
        """The shifting sums after an interaction, or the displacements after RunShifting."""
        n = self.divinfo()["np"]
        out = np.empty((n, 4), np.float32)
        self._check(lib().gbsph_get_shiftpos(self.ctx, ptr(out)), "shiftpos")
        return out

    def ComputeStep_Sym(self, dtpre: float) -> tuple[float, float]:
        """Host-sequenced Symplectic step (JSphGpuSingle.cpp:785-826); returns (dt, next dt)."""
        dt = dtpre
        self.MdbcBoundCorrection(INTERSTEP_SYMPREDICTOR)
        self.Interaction_Forces(INTERSTEP_SYMPREDICTOR)
        dt_p = self.DtVariable(False)
        self.ComputeSymplecticPre(dt)
        self.RunCellDivide()
        self.MdbcBoundCorrection(INTERSTEP_SYMCORRECTOR)
        self.Interaction_Forces(INTERSTEP_SYMCORRECTOR)
        dt_c = self.DtVariable(True)
        self.RunShifting(dt)  # the predictor's RunShifting(dt/2) is not applied by the reference
        self.ComputeSymplecticCorr(dt)
        return dt, min(dt_p, dt_c)

    # ---- device-resident stepping ---------------------------------------
    def ComputeStep(self) -> None:
        """ComputeStep + RunCellDivide with dt kept on the device."""
        self._check(lib().gbsph_step(self.ctx), "ComputeStep")

    def RunSteps(self, nsteps: int, use_graph: bool = True) -> None:
        self._check(lib().gbsph_run(self.ctx, nsteps, int(use_graph)), "RunSteps")

    def sync(self) -> None:
        self._check(lib().gbsph_sync(self.ctx), "sync")

    def step_dt(self) -> tuple[float, float, float]:
        a, b, t = C.c_double(), C.c_double(), C.c_double()
        self._check(lib().gbsph_step_dt(self.ctx, C.byref(a), C.byref(b), C.byref(t)), "step_dt")
        return a.value, b.value, t.value

    # ---- read-back --------------------------------------------------------
    def divinfo(self, with_arrays: bool = False) -> dict:
        info = DivInfo()
        self._check(lib().gbsph_get_divinfo(self.ctx, C.byref(info), None, 0, None, None), "divinfo")
        out = {k: (list(getattr(info, k)) if hasattr(getattr(info, k), "__len__") else getattr(info, k))
               for k, _ in DivInfo._fields_}
        if with_arrays:
            bc = np.empty(info.nctt, np.uint32)
            self._check(lib().gbsph_get_divinfo(self.ctx, C.byref(info), ptr(bc), info.nctt, None, None), "divinfo")
            out["begincell"] = bc
        return out

    def download(self) -> dict:
        n = self.divinfo()["np"]
        pos = np.empty((n, 3), np.float64)
        vr = np.empty((n, 4), np.float32)
        idp = np.empty(n, np.uint32)
        code = np.empty(n, np.uint16)
        dcell = np.empty(n, np.uint32)
        self._check(lib().gbsph_download(self.ctx, ptr(pos), ptr(vr), ptr(idp), ptr(code), ptr(dcell)), "download")
        return {"pos": pos, "velrho": vr, "idp": idp, "code": code, "dcell": dcell}

    def download_into(self, out: dict) -> dict:
        """download() into caller-provided arrays (e.g. page-locked ones) of at
        least np rows; returns the views holding the np current particles."""
        n = self.divinfo()["np"]
        for k, w in (("pos", 3), ("velrho", 4), ("idp", 1), ("code", 1), ("dcell", 1)):
            a = out[k]
            assert a.shape[0] >= n and a.flags["C_CONTIGUOUS"] and (a.ndim == 1 or a.shape[1] == w), k
        self._check(lib().gbsph_download(self.ctx, ptr(out["pos"]), ptr(out["velrho"]), ptr(out["idp"]),
                                         ptr(out["code"]), ptr(out["dcell"])), "download")
        return {k: v[:n] for k, v in out.items()}

    def forces(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.divinfo()["np"]
        ace = np.empty((n, 3), np.float32)
        ar = np.empty(n, np.float32)
        self._check(lib().gbsph_get_forces(self.ctx, ptr(ace), ptr(ar)), "forces")
        return ace, ar

    def pips(self) -> dict:
        """Particle interactions of the current state (JDsPips definition)."""
        out = (C.c_ulonglong * 4)()
        self._check(lib().gbsph_pips(self.ctx, C.byref(out)), "pips")
        return {"checked_bound": out[0], "real_bound": out[1], "checked_fluid": out[2], "real_fluid": out[3]}

    def fluid_front(self, direction=(1.0, 0.0, 0.0), bmin=None, bmax=None) -> tuple[float, int]:
        """Surge front: the largest pos.direction over the fluid particles in
        the box [bmin, bmax] (default: everywhere) and how many fluid particles
        the box holds; -inf when it holds none."""
        big = 1e300
        d = np.ascontiguousarray(direction, np.float64)
        lo = np.ascontiguousarray(bmin if bmin is not None else (-big,) * 3, np.float64)
        hi = np.ascontiguousarray(bmax if bmax is not None else (big,) * 3, np.float64)
        front, n = C.c_double(), C.c_uint()
        self._check(lib().gbsph_fluid_front(self.ctx, ptr(d), ptr(lo), ptr(hi), C.byref(front), C.byref(n)),
                    "fluid_front")
        return front.value, n.value

    def profile(self, max_launches: int) -> None:
        self._check(lib().gbsph_profile(self.ctx, max_launches), "profile")

    def profile_read(self, cap: int = 4096) -> np.ndarray:
        ms = np.zeros(cap, np.float32)
        n = C.c_uint()
        self._check(lib().gbsph_profile_read(self.ctx, ptr(ms), cap, C.byref(n)), "profile_read")
        return ms[: n.value].copy()

    def mark(self, slot: int) -> None:
        self._check(lib().gbsph_mark(self.ctx, slot), "mark")

    def elapsed(self, a: int, b: int) -> float:
        ms = C.c_float()
        self._check(lib().gbsph_elapsed(self.ctx, a, b, C.byref(ms)), "elapsed")
        return ms.value

    def set_option(self, key: int, value: int) -> None:
        """Kernel options: key 1 = fluid-row kernel (2 cell-tiled with a ring of
        8 chunks, the default; 3 the same with 4; 0 queued rounds; 1 one thread
        per particle), key 0 = block size of kernel 1, key 2 = sort digit bits,
        key 3 = mDBC kernel (0 cell-tiled, 1 one thread per row), key 4 =
        warps per group of 32 fluid rows in the cell-tiled kernel (1, 2, 4; 0
        automatic; get_option(5) reads the value in effect), key 6 = lanes a
        boundary row in the bound-row pass (1, 4, 32; 0 automatic;
        get_option(7) reads the value in effect), key 8 = warps per group of
        32 boundary rows in the cell-tiled mDBC kernel (1, 2, 4; 0 automatic;
        get_option(9) reads the value in effect), key 10 = the bound-row pass
        beside the fluid-row pass on a second stream (1) or before it (0)."""
        self._check(lib().gbsph_set_option(self.ctx, key, value), "set_option")

    def get_option(self, key: int) -> int:
        v = C.c_int()
        self._check(lib().gbsph_get_option(self.ctx, key, C.byref(v)), "get_option")
        return v.value

    def graph_prepare(self, nsteps: int) -> None:
        self._check(lib().gbsph_graph_prepare(self.ctx, nsteps), "graph_prepare")

    def launch_count(self) -> int:
        return int(lib().gbsph_launch_count(self.ctx))

    # ---- output -----------------------------------------------------------
    def SaveData(self) -> str:
        """Writes data/Part_%04u.bi4 (JSph::SaveData / JPartDataBi4, JSph.cpp:3062-3110)."""
        cd = self.case
        st = self.download()
        # only the particles of the case are saved, not their periodic copies
        # (GetParticlesData with onlynormal, JSphCpu.cpp:366-424)
        keep = normal_rows(st["code"])
        st = {k: v[keep] for k, v in st.items()}
        order = np.argsort(st["idp"], kind="stable")
        dtl, dtn, t = self.step_dt()
        nmov = sum(c for _, c in cd.motion["objects"]) if cd.motion else 0
        root = bi4.make_partdata_root(
            casename=cd.name, appname="dualsphysics_gb300", data2d=False, casenp=cd.np, casenfixed=cd.npb - nmov,
            casenmoving=nmov, casenfloat=0, casenfluid=cd.nfluid, caseposmin=cd.pos.min(axis=0),
            caseposmax=cd.pos.max(axis=0), dp=cd.params.dp, h=cd.params.h, b=cd.params.b, rhop0=cd.params.rhop0,
            gamma=cd.params.gamma, massbound=cd.params.massbound, massfluid=cd.params.massfluid,
            mapposmin=tuple(cd.params.maprealposmin), mapposmax=tuple(cd.params.maprealposmax))
        npok = len(order)
        extra = {"SymplecticDtPre": (bi4.DAT_DOUBLE, float(dtn)), "DemDtForce": (bi4.DAT_DOUBLE, 0.0)}
        part = bi4.make_part(self.part, t, npok, cd.np - npok, self.nstep, st["pos"].min(axis=0) if npok else (0, 0, 0),
                             st["pos"].max(axis=0) if npok else (0, 0, 0), st["idp"][order], st["pos"][order],
                             st["velrho"][order, :3], st["velrho"][order, 3], posdouble=cd.savepos_double,
                             extra=extra)
        root.items.append(part)
        os.makedirs(os.path.join(self.dirout, "data"), exist_ok=True)
        path = os.path.join(self.dirout, "data", "Part_%04u.bi4" % self.part)
        bi4.write(path, root)
        return path

    def Run(self, casedir: str, casename: str, dirout: str, time_max: float | None = None,
            nsteps: int | None = None, use_graph: bool = True, save: bool = True, cellmode: str = "full") -> dict:
        """Main loop (JSphGpuSingle::Run, JSphGpuSingle.cpp:950-1010)."""
        self.LoadCase(casedir, casename, cellmode=cellmode)
        self.dirout = dirout
        os.makedirs(dirout, exist_ok=True)
        cd = self.case
        tmax = cd.time_max if time_max is None else time_max
        tout = cd.time_out if cd.time_out > 0 else tmax
        self.part = 0
        if save:
            self.SaveData()
        self.part = 1
        tnext = tout
        t0 = time.perf_counter()
        steps = 0
        while True:
            # run a chunk of steps on the device, then check the clock
            chunk = 1 if nsteps is None else max(1, min(50, nsteps - steps))
            if nsteps is not None and steps >= nsteps:
                break
            if cd.params.tstep == STEP_SYMPLECTIC:
                self.RunSteps(chunk, use_graph)
            else:
                for _ in range(chunk):
                    self.ComputeStep()
            steps += chunk
            self.nstep = steps
            _, _, t = self.step_dt()
            self.timestep = t
            if save and (t >= tnext):
                self.SaveData()
                self.part += 1
                tnext += tout
            if nsteps is None and t >= tmax:
                break
        self.sync()
        wall = time.perf_counter() - t0
        return {"steps": steps, "time": self.timestep, "wall_s": wall, "parts": self.part,
                "np": self.divinfo()["np"]}
