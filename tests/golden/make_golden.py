"""Generates the golden fixtures in tests/golden/ from the REFERENCE solver.

Each case is generated with dualsphysics_gb300.casegen (deterministic, seeded),
run through oracle/_ref/ref_harness -- a step-level harness linked against the
reference DualSPHysics CPU solver compiled from its own sources (see
oracle/Makefile.ref) -- and the arrays it dumps are packed into <case>.npz.

Run from the repository root, with the reference source tree available:
    make -f oracle/Makefile.ref -j8 REFSRC=<reference>/src/source
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from dualsphysics_gb300 import casegen as cg  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
OUT = os.path.dirname(os.path.abspath(__file__))

# name -> (spec factory, steps after the detailed first step)
CASES = {
    "dbc_d04": (lambda: cg.spec_c1(dp=0.04, name="dbc_d04"), 20),
    "mdbc_d04": (lambda: cg.spec_c2(dp=0.04, name="mdbc_d04"), 20),
    "jit_d04": (lambda: cg.spec_c1(dp=0.04, name="jit_d04", jitter=0.01, seed=7), 20),
    "vel_d04": (lambda: cg.spec_c1(dp=0.04, name="vel_d04", init_vel=0.05, seed=11), 10),
    "verlet_d04": (lambda: cg.spec_c1(dp=0.04, name="verlet_d04", step_algorithm=1, verlet_steps=5,
                                      init_vel=0.05, seed=3), 12),
    "sps_d04": (lambda: cg.spec_c1(dp=0.04, name="sps_d04", visco_treatment=2, visco=1e-6, density_dt=1,
                                   init_vel=0.05, seed=5), 10),
    "lam_d04": (lambda: cg.spec_c1(dp=0.04, name="lam_d04", visco_treatment=3, visco=1e-6, density_dt=0,
                                   init_vel=0.05, seed=13), 10),
    "ddt2f_d04": (lambda: cg.spec_c2(dp=0.04, name="ddt2f_d04", density_dt=3, init_vel=0.02, seed=17), 10),
    "half_d04": (lambda: cg.spec_c1(dp=0.04, name="half_d04", init_vel=0.02, seed=19), 10, ["-cellmode:half"]),
    "mov_d04": (lambda: spec_moving(), 20),
    "movv_d04": (lambda: spec_moving(name="movv_d04", step_algorithm=1, verlet_steps=5, seed=41), 20),
    # standard shifting: Full with the free-surface threshold (Symplectic), and
    # NoBound without it (Verlet)
    "shift_d04": (lambda: cg.spec_c1(dp=0.04, name="shift_d04", init_vel=0.05, seed=29,
                                     extra_params={"Shifting": 3, "ShiftCoef": -2, "ShiftTFS": 2.75}), 12),
    "shiftnb_d04": (lambda: cg.spec_c1(dp=0.04, name="shiftnb_d04", step_algorithm=1, verlet_steps=5,
                                       init_vel=0.05, seed=31, extra_params={"Shifting": 1}), 12),
    # periodic in x: a channel whose fluid moves at 2 m/s across the periodic faces
    "peri_d04": (lambda: cg.spec_c1(dp=0.04, name="peri_d04", tank=(0.8, 0.4, 0.3), column=(0.8, 0.4, 0.2),
                                    periodic_x=True, init_vel_x=2.0, init_vel=0.02, seed=37), 30),
    # periodic in x and y: a floor only, the fluid moving diagonally across both
    # pairs of faces; copies made for x are copied again for y
    # the channel with Verlet (periodic copies are moved by the update), and with mDBC (copies carry their normals)
    "periv_d04": (lambda: cg.spec_c1(dp=0.04, name="periv_d04", tank=(0.8, 0.4, 0.3), column=(0.8, 0.4, 0.2),
                                     periodic_x=True, init_vel_x=2.0, init_vel=0.02, seed=47, step_algorithm=1,
                                     verlet_steps=5), 30),
    "perim_d04": (lambda: cg.spec_c1(dp=0.04, name="perim_d04", tank=(0.8, 0.4, 0.3), column=(0.8, 0.4, 0.2),
                                     periodic_x=True, init_vel_x=2.0, init_vel=0.02, seed=53, boundary="mdbc"), 30),
    # the channel with standard shifting (sums over copies near the faces)
    "peris_d04": (lambda: cg.spec_c1(dp=0.04, name="peris_d04", tank=(0.8, 0.4, 0.3), column=(0.8, 0.4, 0.2),
                                     periodic_x=True, init_vel_x=2.0, init_vel=0.02, seed=59,
                                     extra_params={"Shifting": 3, "ShiftCoef": -2, "ShiftTFS": 2.75}), 30),
    # the channel with a cross increment: copies and wrapped particles shift by 0.08 m in y
    "perishear_d04": (lambda: cg.spec_c1(dp=0.04, name="perishear_d04", tank=(0.8, 0.4, 0.3),
                                         column=(0.8, 0.4, 0.2), periodic_x=True, peri_inc_y=0.08, init_vel_x=2.0,
                                         init_vel=0.02, seed=61), 30),
    # periodic in z: side walls only, the fluid falls through the bottom face and comes back at the top
    "periz_d04": (lambda: cg.spec_c1(dp=0.04, name="periz_d04", tank=(0.4, 0.4, 0.4), column=(0.4, 0.4, 0.4),
                                     periodic_z=True, init_vel_z=-2.0, init_vel=0.02, seed=67), 30),
    "perixy_d04": (lambda: cg.spec_c1(dp=0.04, name="perixy_d04", tank=(0.6, 0.4, 0.3), column=(0.6, 0.4, 0.2),
                                      periodic_x=True, periodic_y=True, init_vel_x=1.5, init_vel_y=-1.0,
                                      init_vel=0.02, seed=43), 30),
}

# A sloshing tank: the walls move through a chain of movements -- sinusoidal
# translation, sinusoidal pitch about a y axis (phase carried over), uniform
# translation, uniform acceleration (velocity carried over) -- with durations
# that end inside steps, so the handover of the rest of a step is exercised.
MOVING_TANK = [
    dict(type="mvrectsinu", id=1, duration=0.004, next=2, anglesunits="radians", freq=(1.5, 0.0, 0.0),
         ampl=(0.03, 0.0, 0.0), phase=(0.3, 0.0, 0.0)),
    dict(type="mvrotsinu", id=2, duration=0.003, next=3, anglesunits="degrees", axisp1=(0.8, -1.0, 0.2),
         axisp2=(0.8, 1.0, 0.2), freq=2.0, ampl=3.0),
    dict(type="mvrect", id=3, duration=0.002, next=4, vel=(0.05, 0.0, 0.01)),
    dict(type="mvrectace", id=4, duration=1.0, ace=(0.5, 0.0, 0.0)),
]


def spec_moving(name: str = "mov_d04", seed: int = 23, **kw):
    return cg.spec_c1(dp=0.04, name=name, motion=MOVING_TANK, posmin_x="default - 0.1",
                      posmax_x="default + 0.1", init_vel=0.02, seed=seed, **kw)


GAUGE_CASES = ("dbc_d04", "mdbc_d04")
GAUGE_KINDS = {"vel": 0, "swl": 1, "maxz": 2}


def gauges_for(spec) -> list:
    """Gauges of a dam-break case, as (kind, 8 parameters): vel (x,y,z), swl
    (x0,y0,z0,x2,y2,z2,pointdp,masslimit), maxz (x,y,z,height,distlimit) --
    inside the column, near its front and surface, where there is no fluid and
    outside the map."""
    tx, ty, tz = spec.tank
    cx, cy, cz = spec.column
    dp = spec.dp
    h2 = 2.0 * spec.coefh * (3.0 ** 0.5) * dp
    ym = cy / 2
    g = [("vel", (cx * 0.5, ym, cz * 0.5)), ("vel", (cx * 0.95, ym * 0.9, cz * 0.2)),
         ("vel", (cx * 0.5, ym, cz * 0.98)), ("vel", (tx * 0.8, ym, tz * 0.5)), ("vel", (-1.0, ym, 0.1)),
         ("swl", (cx * 0.5, ym, dp, cx * 0.5, ym, tz - dp, dp / 2, 0.0)),
         ("swl", (cx * 0.9, ym * 0.7, dp, cx * 0.9, ym * 0.7, tz - dp, dp / 2, 0.0)),
         ("swl", (tx * 0.8, ym, dp, tx * 0.8, ym, tz - dp, dp / 2, 0.0)),
         ("maxz", (cx * 0.5, ym, 0.0, tz, h2)), ("maxz", (cx * 0.9, ym, 0.0, tz, h2)),
         ("maxz", (tx * 0.8, ym, 0.0, tz, h2))]
    return [(k, tuple(float(v) for v in p) + (0.0,) * (8 - len(p))) for k, p in g]


FLT_MAX = float(np.finfo(np.float32).max)


def mesh_gauges_for(spec) -> list:
    """Mesh gauges of a dam-break case, 24 parameters each: ptref (3), vec1..3
    (9), dis1..3, dispt1..3, dirdat (3), kclimit, kcdummy, masslimit -- a
    vertical x-z grid through the column and the flow (density for pressure
    probes, surface z), and a y-z plane across the column without kernel
    correction."""
    tx, ty, tz = spec.tank
    cx, cy, cz = spec.column
    dp = spec.dp
    ym = cy / 2
    a = (0.05, ym, 0.02, 1, 0, 0, 0, 1, 0, 0, 0, 1, cx * 1.5, 0.0, tz - 0.04, dp, dp, dp / 2, 1, 0, 0,
         0.5, 0.0, 0.0)
    b = (cx * 0.5, 0.02, 0.02, 0, 1, 0, 0, 0, 1, 0, 0, 0, cy * 0.8, cz, 0.0, 2 * dp, dp, 0.0, 0, 0, 1,
         FLT_MAX, FLT_MAX, 0.0)
    return [tuple(float(v) for v in g) for g in (a, b)]


def _write_gauges(casedir: str, gauges: list, meshes: list = ()) -> None:
    nargs = {"vel": 3, "swl": 8, "maxz": 5}
    with open(os.path.join(casedir, "gauges.txt"), "w") as f:
        for k, p in gauges:
            f.write(k + " " + " ".join(repr(v) for v in p[:nargs[k]]) + "\n")
        for p in meshes:
            f.write("mesh " + " ".join(repr(v) for v in p) + "\n")


def run_options(name: str) -> list:
    """Run options of a case beyond the run XML (the reference takes the cell
    mode from the command line)."""
    v = CASES[name]
    return list(v[2]) if len(v) > 2 else []

STATE = (("idp", np.uint32, 1), ("code", np.uint16, 1), ("dcell", np.uint32, 1), ("pos", np.float64, 3),
         ("velrho", np.float32, 4))


def _raw(d, tag, nm, dt, w=1):
    a = np.fromfile(os.path.join(d, f"{tag}_{nm}.bin"), dtype=dt)
    return a.reshape(-1, w) if w > 1 else a


def _meta(d, tag):
    out = {}
    with open(os.path.join(d, f"{tag}_meta.txt")) as f:
        for line in f:
            k, v = line.strip().split("=", 1)
            out[k] = v
    return out


def make(name: str, threads: int = 8) -> str:
    spec_fn, nsteps = CASES[name][:2]
    with tempfile.TemporaryDirectory() as tmp:
        casedir = os.path.join(tmp, "case")
        outdir = os.path.join(tmp, "out")
        os.makedirs(outdir)
        spec = spec_fn()
        cg.write_case(cg.make_dam_break(spec), casedir)
        gauges = gauges_for(spec) if name in GAUGE_CASES else []
        meshes = mesh_gauges_for(spec) if name in GAUGE_CASES else []
        if gauges:
            _write_gauges(casedir, gauges, meshes)
        subprocess.run([HARNESS, casedir, name, outdir, str(nsteps), str(threads)] + run_options(name), check=True,
                       stdout=subprocess.DEVNULL)
        arr = {}
        for tag in ("s0", "s0pre", "s1", "end") + (("s0div", "s0corr") if os.path.exists(
                os.path.join(outdir, "s0div_meta.txt")) else ()):
            for nm, dt, w in STATE:
                if tag in ("s0div", "s1") and nm in ("pos", "velrho"):
                    continue
                arr[f"{tag}_{nm}"] = _raw(outdir, tag, nm, dt, w)
        for tag in ("s0", "s0div", "s1", "end"):
            if os.path.exists(os.path.join(outdir, f"{tag}_begincell.bin")):
                arr[f"{tag}_begincell"] = _raw(outdir, tag, "begincell", np.uint32)
        for tag in ("s0pred", "s0cor"):
            if os.path.exists(os.path.join(outdir, f"{tag}_ace.bin")):
                arr[f"{tag}_ace"] = _raw(outdir, tag, "ace", np.float32, 3)
                arr[f"{tag}_ar"] = _raw(outdir, tag, "ar", np.float32)
        for tag in ("s0pred", "s0cor", "s0predsh", "s0corsh"):  # shifting sums, then displacements
            if os.path.exists(os.path.join(outdir, f"{tag}_shiftpos.bin")):
                arr[f"{tag}_shiftpos"] = _raw(outdir, tag, "shiftpos", np.float32, 4)
        arr["s0mdbc_rho"] = _raw(outdir, "s0mdbc", "velrho", np.float32, 4)[:, 3].copy()
        arr["dtlist"] = np.fromfile(os.path.join(outdir, "end_dtlist.bin"), dtype=np.float64)
        if os.path.exists(os.path.join(outdir, "motion.txt")):  # per-step motion data of the moving objects
            arr["motion"] = np.loadtxt(os.path.join(outdir, "motion.txt"), dtype=np.float64, ndmin=2)
        meta = {tag: _meta(outdir, tag) for tag in ("s0", "s0pred", "s0cor", "s0div", "s1", "end")
                if os.path.exists(os.path.join(outdir, f"{tag}_meta.txt"))}
        if gauges:  # gauges of the final state, computed by the reference's gauge classes
            out, mnpt, mpt, mzs = [], [], [], []
            with open(os.path.join(outdir, "gauges_out.txt")) as f:
                for line in f:
                    t = line.split()
                    v = [float(x) for x in t[1:]]
                    if t[0] == "mesh":
                        mnpt.append([int(x) for x in t[1:]])
                    elif t[0] == "pt":
                        mpt.append(v)
                    elif t[0] == "zs":
                        mzs.append(v[0])
                    else:
                        out.append(v + [0.0] * (3 - len(v)))
            arr["gauge_kind"] = np.array([GAUGE_KINDS[k] for k, _ in gauges], np.uint8)
            arr["gauge_par"] = np.array([p for _, p in gauges], np.float64)
            arr["gauge_out"] = np.array(out, np.float64)
            arr["mesh_par"] = np.array(meshes, np.float64)
            arr["mesh_npt"] = np.array(mnpt, np.uint32)
            arr["mesh_pt"] = np.array(mpt, np.float64)
            arr["mesh_zs"] = np.array(mzs, np.float64)
        arr["meta_json"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, **arr)
        return path


SERIES = {"dbc_d04": (1800, 30)}   # case -> (steps, sample interval)


def series_probes(spec) -> tuple:
    """Pressure probes of a series: a mesh gauge of 7 heights x 2 columns at
    mid-width, 1.5h off the wall behind the water column (x = 0) and at
    x = 2 column lengths, where the surge passes."""
    h = spec.coefh * (3.0 ** 0.5) * spec.dp
    dz = 0.04
    dx = 2 * spec.column[0] - 1.5 * h
    return (1.5 * h, spec.column[1] / 2, spec.dp / 2, 0, 0, 1, 1, 0, 0, 0, 0, 0,
            6 * dz, dx, 0.0, dz, dx, 0.0, 0, 0, 0, 0.5, 0.0, 0.0)


def make_series(name: str, threads: int = 8) -> str:
    """Runs the reference for SERIES[name] steps from the case's initial state
    and records, every interval: step, time, particle and fluid counts, the
    surge front (largest fluid x) and the probes' kernel-corrected density."""
    nsteps, every = SERIES[name]
    spec_fn = CASES[name][0]
    with tempfile.TemporaryDirectory() as tmp:
        casedir = os.path.join(tmp, "case")
        outdir = os.path.join(tmp, "out")
        os.makedirs(outdir)
        spec = spec_fn()
        cg.write_case(cg.make_dam_break(spec), casedir)
        probes = series_probes(spec)
        with open(os.path.join(casedir, "series.txt"), "w") as f:
            f.write(f"{nsteps} {every}\n")
            f.write("mesh " + " ".join(repr(float(v)) for v in probes) + "\n")
        subprocess.run([HARNESS, casedir, name, outdir, "0", str(threads)] + run_options(name), check=True,
                       stdout=subprocess.DEVNULL)
        smp, rho = [], []
        with open(os.path.join(outdir, "series_out.txt")) as f:
            for line in f:
                t = line.split()
                if t[0] == "sample":
                    smp.append([float(x) for x in t[1:]])
                    rho.append([])
                elif t[0] == "pt":
                    rho[-1].append(float(t[5]))
        smp = np.array(smp)
        arr = {"step": smp[:, 0].astype(np.uint32), "time": smp[:, 1], "np": smp[:, 2].astype(np.uint32),
               "nfluid": smp[:, 3].astype(np.uint32), "xfront": smp[:, 4], "probe_rhop": np.array(rho, np.float64),
               "probe_par": np.array(probes, np.float64)}
        path = os.path.join(OUT, f"series_{name}.npz")
        np.savez_compressed(path, **arr)
        return path


# restart cases: steps the reference runs before its state is written as a
# Part file, and steps after the restart
RESTART = {"dbc_d04": (10, 6)}


def _part_writer(tmp: str) -> str:
    """Builds part_write (tests/golden/part_write.cpp with gbsph_run's Part
    writer, gbsph_io.cpp: host code only)."""
    exe = os.path.join(tmp, "part_write")
    csrc = os.path.join(ROOT, "dualsphysics_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + csrc,
                    os.path.join(OUT, "part_write.cpp"), os.path.join(csrc, "gbsph_io.cpp"), "-o", exe], check=True)
    return exe


def make_restart(name: str, threads: int = 8) -> str:
    """The reference runs n1 steps; its state is written as Part_0001.bi4 by
    this library's Part writer; the reference restarts from that file
    (-partbegin:1:1, its own JPartsLoad4 reader) for n2 steps, and also runs
    n1 + n2 steps without a restart.  Keeps the Part file, the restarted run's
    first and last states and dts, and the continuous run's last state."""
    n1, n2 = RESTART[name]
    spec_fn = CASES[name][0]
    with tempfile.TemporaryDirectory() as tmp:
        casedir = os.path.join(tmp, "case")
        cg.write_case(cg.make_dam_break(spec_fn()), casedir)
        outs = {k: os.path.join(tmp, k) for k in ("first", "part", "restart", "cont")}
        for d in outs.values():
            os.makedirs(d)
        # the harness runs a detailed first step, then <nsteps> more
        run = lambda out, n, extra=(): subprocess.run(
            [HARNESS, casedir, name, out, str(n - 1), str(threads)] + run_options(name) + list(extra), check=True,
            stdout=subprocess.DEVNULL)
        run(outs["first"], n1)
        subprocess.run([_part_writer(tmp), casedir, name, outs["first"], "end", "1", outs["part"]], check=True)
        partfile = os.path.join(outs["part"], "data", "Part_0001.bi4")
        run(outs["restart"], n2, ("-partbegin:1:1", os.path.join(outs["part"], "data")))
        run(outs["cont"], n1 + n2)
        arr = {"part_bytes": np.frombuffer(open(partfile, "rb").read(), np.uint8),
               "first_meta_json": np.frombuffer(json.dumps(_meta(outs["first"], "end")).encode(), np.uint8),
               "restart_meta_json": np.frombuffer(json.dumps(_meta(outs["restart"], "end")).encode(), np.uint8),
               "restart_s0_meta_json": np.frombuffer(json.dumps(_meta(outs["restart"], "s0")).encode(), np.uint8),
               "n1": np.uint32(n1), "n2": np.uint32(n2)}
        for tag, d, t in (("first", outs["first"], "end"), ("restart_s0", outs["restart"], "s0"),
                          ("restart", outs["restart"], "end"), ("cont", outs["cont"], "end")):
            for nm, dt, w in STATE:
                arr[f"{tag}_{nm}"] = _raw(d, t, nm, dt, w)
        arr["restart_dtlist"] = np.fromfile(os.path.join(outs["restart"], "end_dtlist.bin"), np.float64)
        arr["cont_dtlist"] = np.fromfile(os.path.join(outs["cont"], "end_dtlist.bin"), np.float64)
        path = os.path.join(OUT, f"restart_{name}.npz")
        np.savez_compressed(path, **arr)
        return path


if __name__ == "__main__":
    if not os.path.exists(HARNESS):
        sys.exit(f"reference harness not built: {HARNESS} (make -f oracle/Makefile.ref)")
    for nm in (sys.argv[1:] or list(CASES) + ["series", "restart"]):
        if nm == "restart":
            for rn in RESTART:
                p = make_restart(rn)
                print("restart", rn, os.path.getsize(p), "bytes")
            continue
        if nm == "series":
            for sn in SERIES:
                p = make_series(sn)
                print("series", sn, os.path.getsize(p), "bytes")
            continue
        p = make(nm)
        print(nm, os.path.getsize(p), "bytes")
