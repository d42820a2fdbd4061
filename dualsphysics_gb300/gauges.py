"""Gauge system on the GPU state: the host side of the reference's JGaugeSystem
(JDsGaugeSystem.cpp:383-468) for the velocity, SWL, max-z and mesh gauges.

Gauges are added by name (AddGaugeVel / AddGaugeSwl / AddGaugeMaxZ /
AddGaugeMesh), computed together on the current divided state by CalculeGpu
(one gbsph_gauge_* call per gauge type, one per mesh gauge) and read with
GetResult: a velocity or surface point (3 floats), a zmax, or for a mesh gauge
a dict of vel, veldir, rhop, mass (per point) and zsurf (per column).
Pressure() turns a mesh gauge's density into pressure probes.  SaveResults
writes the per-gauge CSV files the reference writes for the point gauges
(Gauges<Type>_<name>.csv with the same columns, JDsGaugeItem.cpp:385-398,
679-693, 966-979).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from ._lib import lib

VEL, SWL, MAXZ, MESH = "Vel", "SWL", "MaxZ", "Mesh"
FLT_MAX = float(np.finfo(np.float32).max)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class Gauge:
    name: str
    kind: str
    point0: tuple
    point2: tuple = (0.0, 0.0, 0.0)
    pointdp: float = 0.0
    masslimit: float = 0.0
    height: float = 0.0
    distlimit: float = 0.0
    mesh: object = None            # _lib.Mesh of a mesh gauge
    kclimit: float = 0.5
    kcdummy: float = 0.0
    results: list = field(default_factory=list)   # (timestep, value) per CalculeGpu


class GaugeSystem:
    """JGaugeSystem counterpart bound to one GbSphSingle."""

    def __init__(self, sph):
        self.sph = sph
        self.gauges: list[Gauge] = []

    def _add(self, g: Gauge) -> Gauge:
        if any(x.name == g.name for x in self.gauges):
            raise ValueError(f"The name '{g.name}' already exists.")
        self.gauges.append(g)
        return g

    def AddGaugeVel(self, name: str, point) -> Gauge:
        return self._add(Gauge(name, VEL, tuple(float(v) for v in point)))

    def AddGaugeSwl(self, name: str, point0, point2, pointdp: float, masslimit: float = 0.0) -> Gauge:
        """masslimit <= 0 takes the reference's default (massfluid*0.5, 0.4 in 2-D)."""
        return self._add(Gauge(name, SWL, tuple(float(v) for v in point0), tuple(float(v) for v in point2),
                               float(pointdp), float(masslimit)))

    def AddGaugeMaxZ(self, name: str, point0, height: float, distlimit: float) -> Gauge:
        return self._add(Gauge(name, MAXZ, tuple(float(v) for v in point0), height=float(height),
                               distlimit=float(distlimit)))

    def AddGaugeMesh(self, name: str, ptref, vec1, vec2, vec3, dis, dispt, dirdat=(0.0, 0.0, 0.0),
                     kclimit: float = 0.5, kcdummy: float = 0.0, masslimit: float = 0.0) -> Gauge:
        """Mesh gauge (JGaugeSystem::AddGaugeMesh): a grid of npt1 x npt2 x npt3
        points; kclimit / kcdummy None disable the kernel correction / the dummy
        value (the reference's "none"); dirdat is made unitary as the
        reference's XML loader does."""
        from ._lib import Mesh
        m = Mesh()
        for f, v in (("ptref", ptref), ("vec1", vec1), ("vec2", vec2), ("vec3", vec3), ("dis", dis),
                     ("dispt", dispt)):
            getattr(m, f)[:] = [float(x) for x in v]
        d = np.asarray(dirdat, np.float32)
        n = np.float32(np.sqrt(np.float32(np.float32(d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])))
        m.dirdat[:] = [float(x) for x in ((d / n).astype(np.float32) if n else d)]
        return self._add(Gauge(name, MESH, tuple(float(v) for v in ptref), mesh=m, masslimit=float(masslimit),
                               kclimit=FLT_MAX if kclimit is None else float(kclimit),
                               kcdummy=FLT_MAX if kcdummy is None else float(kcdummy)))

    @staticmethod
    def MeshPoints(g: Gauge) -> tuple[int, int, int]:
        out = (C.c_uint * 3)()
        if lib().gbsph_mesh_points(C.byref(g.mesh), C.byref(out)) != 0:
            raise ValueError(f"invalid mesh of gauge '{g.name}'")
        return tuple(int(x) for x in out)

    def GetGauge(self, key) -> Gauge:
        if isinstance(key, int):
            return self.gauges[key]
        for g in self.gauges:
            if g.name == key:
                return g
        raise KeyError(key)

    # ---- computation ------------------------------------------------------
    def CalculeGpu(self, timestep: float) -> None:
        """Computes every gauge on the current state of the context."""
        ctx = self.sph.ctx
        L = lib()
        vel = [g for g in self.gauges if g.kind == VEL]
        if vel:
            pts = np.ascontiguousarray([g.point0 for g in vel], np.float64)
            out = np.empty((len(vel), 3), np.float32)
            self.sph._check(L.gbsph_gauge_velocity(ctx, len(vel), _ptr(pts), _ptr(out)), "gauge velocity")
            for g, v in zip(vel, out):
                g.results.append((timestep, v.copy()))
        swl = [g for g in self.gauges if g.kind == SWL]
        if swl:
            p = np.ascontiguousarray([g.point0 + g.point2 for g in swl], np.float64)
            dp = np.ascontiguousarray([g.pointdp for g in swl], np.float64)
            ml = np.ascontiguousarray([g.masslimit for g in swl], np.float32)
            out = np.empty((len(swl), 3), np.float32)
            self.sph._check(L.gbsph_gauge_swl(ctx, len(swl), _ptr(p), _ptr(dp), _ptr(ml), _ptr(out)), "gauge swl")
            for g, v in zip(swl, out):
                g.results.append((timestep, v.copy()))
        mz = [g for g in self.gauges if g.kind == MAXZ]
        if mz:
            p = np.ascontiguousarray([g.point0 + (g.height,) for g in mz], np.float64)
            dl = np.ascontiguousarray([g.distlimit for g in mz], np.float32)
            out = np.empty(len(mz), np.float32)
            self.sph._check(L.gbsph_gauge_maxz(ctx, len(mz), _ptr(p), _ptr(dl), _ptr(out)), "gauge maxz")
            for g, v in zip(mz, out):
                g.results.append((timestep, np.float32(v)))
        for g in (x for x in self.gauges if x.kind == MESH):
            n1, n2, n3 = self.MeshPoints(g)
            n = n1 * n2 * n3
            r = {"npt": (n1, n2, n3), "vel": np.empty((n, 3), np.float32), "veldir": np.empty(n, np.float32),
                 "rhop": np.empty(n, np.float32), "mass": np.empty(n, np.float32),
                 "zsurf": np.empty(n1 * n2, np.float32)}
            self.sph._check(L.gbsph_gauge_mesh(ctx, C.byref(g.mesh), g.kclimit, g.kcdummy, g.masslimit,
                                               _ptr(r["vel"]), _ptr(r["veldir"]), _ptr(r["rhop"]), _ptr(r["mass"]),
                                               _ptr(r["zsurf"])), "gauge mesh")
            g.results.append((timestep, r))

    def Pressure(self, rhop) -> np.ndarray:
        """Pressure probes from a mesh gauge's kernel-corrected density, with the
        case's Tait equation of state p = B((rho/rho0)^gamma - 1)
        (FunSphEos.h:38-40)."""
        c = self.sph.consts
        r = np.asarray(rhop, np.float64)
        return c.cteb * ((r / c.rhopzero) ** c.gamma - 1.0)

    def GetResult(self, key):
        """Last result of a gauge: velocity (3 floats), surface point (3 floats) or zmax."""
        g = self.GetGauge(key)
        if not g.results:
            raise RuntimeError(f"gauge '{g.name}' has no result yet")
        return g.results[-1][1]

    # ---- output -----------------------------------------------------------
    def SaveResults(self, dirout: str) -> list[str]:
        """Writes dirout/Gauges<Type>_<name>.csv for every gauge (all results so far)."""
        files = []
        for g in self.gauges:
            if g.kind == MESH:  # the reference writes mesh data through its own mesh-data files
                continue
            path = os.path.join(dirout, f"Gauges{g.kind}_{g.name}.csv")
            p0 = ";".join("%g" % np.float32(v) for v in g.point0)
            with open(path, "w") as f:
                if g.kind == VEL:
                    f.write("time [s];velx [m/s];vely [m/s];velz [m/s];posx [m];posy [m];posz [m]\n")
                    for t, v in g.results:
                        f.write("%g;%g;%g;%g;%s\n" % (t, v[0], v[1], v[2], p0))
                elif g.kind == SWL:
                    p2 = ";".join("%g" % np.float32(v) for v in g.point2)
                    f.write("time [s];swlx [m];swly [m];swlz [m];pos0x [m];pos0y [m];pos0z [m];"
                            "pos2x [m];pos2y [m];pos2z [m]\n")
                    for t, v in g.results:
                        f.write("%g;%g;%g;%g;%s;%s\n" % (t, v[0], v[1], v[2], p0, p2))
                else:
                    f.write("time [s];zmax [m];posx [m];posy [m];posz [m]\n")
                    for t, v in g.results:
                        f.write("%g;%g;%s\n" % (t, v, p0))
            files.append(path)
        return files
