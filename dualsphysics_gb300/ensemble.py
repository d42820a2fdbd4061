"""Batched ensembles: many independent dam-break / sloshing cases advanced
together on one GPU (``gbsph_ensemble_*``), with the fluid-row kernel of each
case chosen by the autotuner (``gbsph_tune_forces``).

The reference has no counterpart: it runs one case per process
(JSphGpuSingle::Run, JSphGpuSingle.cpp:950-1010).  Each case here is a full
``GbSphSingle`` (its own arrays, stream, adaptive dt and motion); the ensemble
captures one step of all of them as one CUDA graph with a branch per case.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import tempfile
from dataclasses import dataclass

import numpy as np

from . import casegen as cg
from ._lib import GbsphError, TuneResult, lib
from .case import load_case
from .sph import GbSphSingle


@dataclass
class EnsembleCase:
    spec: cg.CaseSpec
    target: int          # drawn particle count (fluid)
    sloshing: bool


def ensemble_specs(n: int = 64, seed: int = 0, count_range=(20_000, 2_000_000), scale: float = 1.0,
                   time_max: float = 1.0) -> list[EnsembleCase]:
    """The seeded draw of n cases: tank dims uniform in 0.5-2.0 m, fill
    fraction (fluid volume / tank volume) uniform in 0.2-0.6, fluid count
    log-uniform in count_range (times `scale`) setting dp, and half of the
    cases a sinusoidal x sloshing motion of the walls, amplitude 0-0.05 m,
    frequency 0.5-2 Hz."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        lx, ly, lz = (float(v) for v in rng.uniform(0.5, 2.0, 3))
        fill = float(rng.uniform(0.2, 0.6))
        target = int(math.exp(rng.uniform(math.log(count_range[0]), math.log(count_range[1]))) * scale)
        slosh = bool(rng.uniform() < 0.5)
        ampl, freq = float(rng.uniform(0.0, 0.05)), float(rng.uniform(0.5, 2.0))
        # column against the x=0 wall: full width, sqrt(fill) of length and height
        cx, cz = lx * math.sqrt(fill), lz * math.sqrt(fill)
        dp = (cx * ly * cz / max(target, 1000)) ** (1.0 / 3.0)
        dp = float(np.float32(dp))
        kw = dict(name=f"Ens{k:02d}", tank=(lx, ly, lz), column=(cx, ly, cz), dp=dp, seed=seed * 1000 + k,
                  time_max=time_max)
        if slosh:
            margin = ampl + 4 * dp
            kw.update(motion=[dict(type="mvrectsinu", id=1, duration=1000.0, anglesunits="radians",
                                   freq=(freq, 0.0, 0.0), ampl=(ampl, 0.0, 0.0), phase=(0.0, 0.0, 0.0))],
                      posmin_x=f"default - {margin:.6f}", posmax_x=f"default + {margin:.6f}")
        out.append(EnsembleCase(cg.CaseSpec(**kw), target, slosh))
    return out


def load_ensemble_case(ec: EnsembleCase, workdir: str | None = None):
    """Generates and loads one case through the product loader."""
    tmp = workdir or tempfile.mkdtemp(prefix="gbens_")
    cg.write_case(cg.make_dam_break(ec.spec), tmp)
    return load_case(tmp, ec.spec.name)


class Ensemble:
    """A set of GbSphSingle cases advanced together (gbsph_ensemble)."""

    def __init__(self, sims: list[GbSphSingle]):
        self.sims = sims
        self.e = C.c_void_p()
        arr = (C.c_void_p * len(sims))(*[s.ctx.value for s in sims])
        rc = lib().gbsph_ensemble_create(len(sims), arr, C.byref(self.e))
        if rc:
            raise GbsphError(rc, "gbsph_ensemble_create")

    def _check(self, rc: int, what: str):
        if rc:
            raise GbsphError(rc, f"{what}: {lib().gbsph_ensemble_last_error(self.e).decode()}")

    def run(self, nsteps: int, use_graph: bool = True) -> None:
        self._check(lib().gbsph_ensemble_run(self.e, nsteps, int(use_graph)), "gbsph_ensemble_run")

    def sync(self) -> None:
        self._check(lib().gbsph_ensemble_sync(self.e), "gbsph_ensemble_sync")

    def launches_per_step(self) -> int:
        return int(lib().gbsph_ensemble_launches_per_step(self.e))

    def close(self) -> None:
        if self.e:
            lib().gbsph_ensemble_destroy(self.e)
            self.e = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune(sim: GbSphSingle, reps: int = 3) -> dict:
    """Runs the autotuners on one case (fluid-row kernel, then the sort's
    digit width); returns the timings and the choices."""
    r = TuneResult()
    sim._check(lib().gbsph_tune_forces(sim.ctx, reps, C.byref(r)), "gbsph_tune_forces")
    bits = C.c_int()
    ms = (C.c_float * 2)()
    sim._check(lib().gbsph_tune_sort(sim.ctx, reps, C.byref(bits), ms), "gbsph_tune_sort")
    return {"best": r.best, "variant": list(r.variant), "bsize": list(r.bsize), "split": list(r.split), "ms": list(r.ms),
            "bound_best": r.bound_best, "bound_lanes": list(r.bound_lanes), "bound_ms": list(r.bound_ms),
            "mdbc_best": r.mdbc_best, "mdbc_split": list(r.mdbc_split), "mdbc_ms": list(r.mdbc_ms),
            "sort_bits": bits.value, "sort_ms": list(ms)}


# Options of a case that shape its kernels' launches (gbsph_set_option keys):
# fluid-row kernel, its block size, warps per fluid row group, lanes a
# boundary row, warps per mDBC row group.
SHAPE_KEYS = (1, 0, 4, 6, 8)

# Ensemble-level policies, each a function (case options as tuned alone) ->
# the options the case runs with in the ensemble graph.
MIX_POLICIES = {
    "as tuned alone": lambda o: dict(o),
    "one thread a boundary row": lambda o: {**o, 6: 1},
    "one warp or thread a row": lambda o: {**o, 4: 1, 6: 1, 8: 1},
}


def case_options(sim: GbSphSingle) -> dict:
    return {k: sim.get_option(k) for k in SHAPE_KEYS}


def set_case_options(sim: GbSphSingle, opts: dict) -> None:
    for k in SHAPE_KEYS:
        if sim.get_option(k) != opts[k]:
            sim.set_option(k, opts[k])


def tune_mix(ens: "Ensemble", sims: list, reps: int = 3) -> dict:
    """The ensemble-level autotuner: each case's autotuner times it alone,
    where launches that spread a small case over more warps pay off; in the
    ensemble graph the cases' branches already share the SMs.  This times
    replays of the whole ensemble under each policy of MIX_POLICIES (one
    warm-up replay, which captures the graph, then `reps`), applied to the
    options the cases were tuned to, and keeps the fastest.  The cases step
    while it runs.  Returns the mean ms of a replay per policy and the
    policy kept."""
    import time
    alone = [case_options(s) for s in sims]
    ms = {}
    for name, pol in MIX_POLICIES.items():
        for s, o in zip(sims, alone):
            set_case_options(s, pol(o))
        ens.run(1, use_graph=True)
        ens.sync()
        t0 = time.perf_counter()
        ens.run(reps, use_graph=True)
        ens.sync()
        ms[name] = 1e3 * (time.perf_counter() - t0) / reps
    best = min(ms, key=ms.get)
    for s, o in zip(sims, alone):
        set_case_options(s, MIX_POLICIES[best](o))
    return {"ms_per_replay": ms, "kept": best, "alone": alone}
