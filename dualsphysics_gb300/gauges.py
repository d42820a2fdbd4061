"""Gauge system on the GPU state: the host side of the reference's JGaugeSystem
(JDsGaugeSystem.cpp:383-441) for the velocity, SWL and max-z gauges.

Gauges are added by name (AddGaugeVel / AddGaugeSwl / AddGaugeMaxZ), computed
together on the current divided state by CalculeGpu (one gbsph_gauge_* call per
gauge type, each one kernel launch) and read with GetResult; SaveResults writes
the per-gauge CSV files the reference writes (Gauges<Type>_<name>.csv with the
same columns, JDsGaugeItem.cpp:385-398, 679-693, 966-979).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from ._lib import lib

VEL, SWL, MAXZ = "Vel", "SWL", "MaxZ"


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
