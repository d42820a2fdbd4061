"""Benchmark of the GB300 WCSPH step on the 3-D dam break with mDBC and the box
obstacle at dp=0.0025 m (~5.2M fluid + ~1.5M boundary particles).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb|reference] [--dp DP]
    python bench.py --workload c3|c3err|ensemble|closure|closure-judge   (the other measured workloads)

A step is one Symplectic step (predictor + corrector interaction passes, two
cell divisions, mDBC correction, dt reduction) of the whole particle set.

* ``value``: steps/s with the state resident in HBM, timed with CUDA events on
  the context stream around K steps replayed from one captured CUDA graph.
* ``e2e``: steps/s through the C ABI as a caller drives it (gbsph_upload from
  host arrays, K x (gbsph_step + dt read-back, as the reference's Run loop
  reads TimeStep every step), gbsph_download of the final state), wall clock.
* ``roofline``: the fluid Interaction_Forces kernel (the dominant one), each
  launch bracketed by CUDA events inside the timed region.  Algorithmic bytes
  per launch: 52 B per fluid row (pscell, velrho, dcell read; acear written)
  plus 32 B per boundary particle (read once as a neighbour); ``traffic`` is
  the DRAM bytes per launch that ncu measured for that kernel on this
  workload (DRAM_TRAFFIC below, with the capture it comes from).  The kernel is issue-bound, so its HBM
  fraction is small by construction; ``roofline_fp32`` states the same
  launches against the FP32 FLOP model (80 FLOP per real fluid-row pair) and
  the FFMA rate measured in the same run (gbsph_ffma_peak; the nominal rate
  at the sampled SM clock beside it), and ``gather_gbs`` the neighbour bytes
  the checks read from the staged copies (32 B per checked neighbour).
* ``cpu_baseline``: the oracle (CPU restatement of the reference step, OpenMP
  on all host cores), in its timing build, timed over full steps of the same
  state.
* ``--impl reference``: the same timed oracle on the host cores as the
  reference arm (the reference's sources are not on the GPU host, and its
  x86 build here does not run on the host's Arm cores).
Inputs (~1.5 GB of particle arrays) are larger than L2 (129 MB).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s & particle-interactions/s on 1 GB300"
FLOP_PER_FLUID_PAIR = 80.0  # Wendland + artificial visc + DDT2 + precomputed EOS
BYTES_PER_CHECKED = 32.0    # pscell (16 B) + velrho (16 B) per checked neighbour
BYTES_PER_FLUID_ROW = 52.0  # pscell 16 + velrho 16 + dcell 4 read, acear 16 written
BYTES_PER_BOUND_NEIGHBOUR = 32.0  # pscell + velrho of a boundary particle, read once
FP32_LANES_PER_SM = 128     # FFMA lanes per SM (2 FLOP each per clock)


# DRAM bytes per launch of the fluid-row kernels on the C2 workload (dp =
# 0.0025 m), from one ncu capture each (dram__bytes_read.sum +
# dram__bytes_write.sum, --clock-control none), summarised in profiles/:
# variant -> (kernel, bytes per launch, dp of the capture)
DRAM_TRAFFIC = {0: ("k_forces_fluid_q", 269218560.0, 0.0025),   # k_forces_fluid_q_c2_dram.md
                2: ("k_forces_fluid_t", 271390000.0, 0.0025)}   # k_forces_fluid_t_c2_dram.md
# the fluid-row kernel of each variant (gbsph_set_option key 1)
KERNEL_NAME = {0: "k_forces_fluid_q", 1: "k_forces_fluid", 2: "k_forces_fluid_t (ring of 8 chunks)",
               3: "k_forces_fluid_t (ring of 4 chunks)"}


def _dram_traffic(variant: int, dp: float):
    v = DRAM_TRAFFIC.get(variant)
    return v[1] if v and abs(v[2] - dp) < 1e-12 else None


def _pinned(shape, dtype):
    """A numpy array in page-locked host memory (torch is used for the allocation only)."""
    import torch
    t = torch.empty(shape, dtype={np.float64: torch.float64, np.float32: torch.float32, np.uint32: torch.int32,
                                  np.uint16: torch.int16}[dtype], pin_memory=True)
    return t.numpy().view(dtype)


def _pinned_case(cd):
    """A copy of the case whose particle arrays live in page-locked host memory."""
    import copy
    pc = copy.copy(cd)
    for k in ("pos", "velrho", "idp", "code", "boundnor"):
        v = getattr(cd, k)
        if v is not None:
            pv = _pinned(v.shape, v.dtype.type)
            pv[...] = v
            setattr(pc, k, pv)
    return pc


def _sm_count(dev: int) -> int:
    try:
        import torch
        return int(torch.cuda.get_device_properties(dev).multi_processor_count)
    except Exception:
        return 152


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                         timeout=5).stdout.strip()
                    if out:
                        self.rows.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)

        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and "Active" in r[3 + i]
                          and "Not" not in r[3 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def replica_throughput(ms: float, K: int, dist=None, world: int = 1) -> tuple[float, float]:
    """N independent replicas (one per rank, no data-path collective): each
    rank timed its own K steps in `ms`; the job took as long as the slowest
    rank (a MAX all-reduce over the ranks), and the whole-job value is
    world * K steps over that time.  Returns (t_max in ms, steps/s)."""
    t_max = ms
    if dist is not None and world > 1:
        import torch
        tt = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    return t_max, world * K / (t_max / 1e3)


def make_case(dp: float, cellmode: str = "full", workload: str = "c2"):
    """c2: the dam break with the box obstacle and mDBC (tank 1.6x0.67x0.4 m);
    c3: the large plain run, the geometry scaled x4 (tank 6.4x2.68x1.6 m, a
    1.6x2.68x0.6 m column, DBC walls)."""
    from dualsphysics_gb300 import casegen as cg
    from dualsphysics_gb300.case import load_case
    tmp = tempfile.mkdtemp(prefix="gbbench_")
    name = "DamC3" if workload == "c3" else "DamC2"
    spec = cg.spec_c3(dp=dp, name=name) if workload == "c3" else cg.spec_c2(dp=dp, name=name)
    cg.write_case(cg.make_dam_break(spec), tmp)
    return load_case(tmp, name, cellmode)


def workload_text(args) -> str:
    if args.workload in ("c3", "c3err"):
        return (f"large plain dam break (tank 6.4x2.68x1.6 m, column 1.6x2.68x0.6 m), DBC walls, dp={args.dp}, "
                f"Symplectic, Wendland, artificial visc 0.01, DDT2 0.1")
    return (f"3-D dam break (tank 1.6x0.67x0.4 m, column 0.4x0.67x0.3 m), mDBC + 0.12x0.12x0.45 m box obstacle, "
            f"dp={args.dp}, Symplectic, Wendland, artificial visc 0.01, DDT2 0.1")


def cpu_baseline(cd, steps: int, warmup: int = 0):
    """The oracle's timing build (OpenMP on all host cores) over `steps` full,
    unsampled steps of the state `cd` after `warmup` untimed steps; returns
    (mean seconds per step, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    po.use_timing_build()
    ct = po.config(po.params_from(cd.params))
    sim = po.Sim(ct, cd.pos, cd.velrho, cd.idp, cd.code, cd.npb, cd.boundnor)
    for _ in range(warmup):
        sim.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.step()
    t = (time.perf_counter() - t0) / max(steps, 1)
    return t, int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))


def run_reference(args, cd, rank):
    """The reference arm: full oracle steps (timing build) on the host cores,
    one untimed warm-up step (a CPU step needs no more), then K timed steps."""
    warm = min(args.warmup, 1)
    t, cores = cpu_baseline(cd, args.steps, warm)
    v = 1.0 / t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": warm, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 positions)", "data": "synthetic",
            "config": {"workload": workload_text(args), "particles": cd.np,
                       "fluid": cd.nfluid, "boundary": cd.npb, "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full oracle steps of the workload (timing build: the "
                                       f"reference's -O3 -ffast-math), after {warm} warm-up step"},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if rank == 0:
        print(json.dumps(line))


def _dt_from(c, acemax, velmax, viscdt):
    """DtVariable (JSphCpu.cpp:2035-2078) in double from the three maxima."""
    h = float(c.kernelh)
    dt1 = np.sqrt(h / acemax) if acemax else np.finfo(np.float64).max
    dt2 = h / (max(float(c.cs0), velmax * 10.0) + h * viscdt)
    return max(float(c.cflnumber) * min(dt1, dt2), float(c.dtmin))


def run_c3err(args, local: int = 0):
    """C3 error statement (--workload c3err): the large plain run (49.4 M
    particles) stepped `--steps` times on the GPU; at the first, middle and
    last step the state is read back, and the interaction the next step starts
    with (the predictor's Interaction_Forces and DtVariable) is evaluated both
    on the GPU and by the oracle in FP64 (and, for comparison, in FP32, the
    reference's own algorithm and evaluation order) on that same state.
    Reports, per sample, the scaled errors (|x - x_f64| / conditioning scale)
    of ace (fluid rows) and ar (all rows) -- maximum, 99.9th percentile and
    median -- and the relative error of AceMax and of the dt."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    from dualsphysics_gb300 import _lib
    from dualsphysics_gb300.sph import GbSphSingle
    po.build()
    cd = make_case(args.dp, args.cellmode, "c3")
    s = GbSphSingle(local)
    s.setup(cd)
    ct = po.config(po.params_from(cd.params))
    K = args.steps
    samples = sorted({0, K // 2, K})
    out = []

    def errs(x, ref, scale):
        e = np.abs(np.asarray(x, np.float64) - ref)
        e = (e.max(axis=1) if e.ndim == 2 else e) / np.maximum(scale, 1e-30)
        return {"max": float(e.max()), "p99.9": float(np.percentile(e, 99.9)), "median": float(np.median(e))}

    t0 = time.perf_counter()
    for k in range(K + 1):
        if k in samples:
            mx = s.Interaction_Forces(_lib.INTERSTEP_SYMPREDICTOR)
            dt_gpu = s.DtVariable(False)
            ace, ar = s.forces()
            gs = s.download()
            o = po.Sim(ct, gs["pos"], gs["velrho"], gs["idp"], gs["code"], cd.npb, None)
            assert np.array_equal(o.state()["idp"], gs["idp"]), "the oracle's divide of the GPU state differs"
            f64 = po.forces_f64(o)
            o.interaction()
            a32, r32 = o.forces()
            om = o.maxes()
            npb = o.npb
            acemax64 = float(np.sqrt((f64["ace"][npb:] ** 2).sum(axis=1).max()))
            dt64 = _dt_from(ct, acemax64, om["velmax"], f64["viscdt"])
            out.append({"step": k, "particles": int(o.np),
                        "ace_gpu": errs(ace[npb:], f64["ace"][npb:], f64["absace"][npb:]),
                        "ace_oracle_fp32": errs(a32[npb:], f64["ace"][npb:], f64["absace"][npb:]),
                        "ar_gpu": errs(ar, f64["ar"], f64["absar"]),
                        "ar_oracle_fp32": errs(r32, f64["ar"], f64["absar"]),
                        "acemax_rel": abs(mx["acemax"] - acemax64) / acemax64,
                        "viscdtmax_rel": abs(mx["viscdtmax"] - f64["viscdt"]) / max(f64["viscdt"], 1e-30),
                        "dt_rel": abs(dt_gpu - dt64) / dt64})
            del o, f64
            print(json.dumps(out[-1]), flush=True)
        if k < K:
            s.RunSteps(1, use_graph=True)
    s.close()
    worst = {q: max(r[q]["max"] for r in out) for q in ("ace_gpu", "ace_oracle_fp32", "ar_gpu", "ar_oracle_fp32")}
    line = {"metric": "FP32 error against the FP64 oracle, C3 (max over the samples)", "value": worst["ace_gpu"],
            "unit": "scaled error of ace", "steps": K, "samples": out, "worst": worst,
            "dt_rel_max": max(r["dt_rel"] for r in out), "wall_s": time.perf_counter() - t0,
            "config": {"workload": workload_text(args), "particles": cd.np}}
    print(json.dumps(line))


def run_ensemble(args, local: int = 0):
    """Batched ensemble (--workload ensemble): n seeded dam-break / sloshing
    cases (tank 0.5-2 m per side, fill 0.2-0.6, 20k-2M fluid particles
    log-uniform, half of them sloshing) advanced together, each case's
    fluid-row kernel chosen by the autotuner.  Reports aggregate
    particle-steps/s of the ensemble graph (one replay = one step of every
    case), of the same cases on concurrent streams without a graph, and of the
    cases run one after the other through the plain path (gbsph_run per case),
    wall clock around K steps with the device synchronised on both sides."""
    from dualsphysics_gb300.ensemble import Ensemble, ensemble_specs, load_ensemble_case, set_case_options, tune, \
        tune_mix
    from dualsphysics_gb300.sph import GbSphSingle
    specs = ensemble_specs(args.ens_cases, seed=args.ens_seed, scale=args.ens_scale)
    sims, tuned = [], []
    t_load = time.perf_counter()
    for ec in specs:
        s = GbSphSingle(local)
        s.setup(load_ensemble_case(ec))
        sims.append(s)
    t_load = time.perf_counter() - t_load
    for s in sims:
        tuned.append(tune(s, reps=3))
    nps = np.array([s.divinfo()["np"] for s in sims], dtype=np.float64)
    ens = Ensemble(sims)
    K, W = args.steps, args.warmup
    mix = tune_mix(ens, sims, reps=3)       # the ensemble-level policy (cases step meanwhile)
    ens.run(W, use_graph=True)
    ens.sync()

    def timed(fn):
        ens.sync()
        t0 = time.perf_counter()
        fn()
        ens.sync()
        return time.perf_counter() - t0

    with ClockSampler(local) as clk:
        t_graph = timed(lambda: ens.run(K, use_graph=True))
        t_streams = timed(lambda: ens.run(K, use_graph=False))

        def sequential():
            for s in sims:
                s.RunSteps(K, use_graph=True)
                s.sync()
        mixed = [{k: s.get_option(k) for k in (1, 0, 4, 6, 8)} for s in sims]
        for s, o in zip(sims, mix["alone"]):   # the plain path runs each case as tuned alone
            set_case_options(s, o)
        for s in sims:
            s.RunSteps(1, use_graph=True)       # graph capture outside the clock
        t_seq = timed(sequential)
        for s, o in zip(sims, mixed):
            set_case_options(s, o)
    pst = float(nps.sum()) * K
    line = {"metric": "aggregate particle-steps/s, batched ensemble", "value": pst / t_graph,
            "unit": "particle-steps/s", "n_gpus": 1, "steps": K, "warmup": W, "higher_is_better": True,
            "dtype": "f32 (f64 positions and integration)", "data": "synthetic",
            "config": {"workload": f"{len(sims)} dam-break/sloshing cases, seed {args.ens_seed}",
                       "particles_total": int(nps.sum()), "particles_min": int(nps.min()),
                       "particles_max": int(nps.max()), "sloshing": int(sum(ec.sloshing for ec in specs)),
                       "setup_s": t_load},
            "streams_no_graph": pst / t_streams, "sequential_plain": pst / t_seq,
            "speedup_vs_sequential": t_seq / t_graph,
            "launches_per_replay": ens.launches_per_step(),
            "mix_tuner": {"ms_per_replay": {k: round(v, 4) for k, v in mix["ms_per_replay"].items()},
                          "kept": mix["kept"]},
            "tuner": {"choices": [[t["variant"][t["best"]], t["bsize"][t["best"]], t["split"][t["best"]]]
                                  for t in tuned],
                      "sort_bits": [t["sort_bits"] for t in tuned],
                      "sort_ms_8_11": [[round(x, 4) for x in t["sort_ms"]] for t in tuned],
                      "candidates": [[v, b, sp] for v, b, sp in zip(tuned[0]["variant"], tuned[0]["bsize"],
                                                                     tuned[0]["split"])],
                      "ms": [[round(x, 4) for x in t["ms"]] for t in tuned]},
            "clocks": clk.summary()}
    ens.close()
    for s in sims:
        s.close()
    print(json.dumps(line))


def run_closure(args, local: int = 0):
    """Learned closure (--workload closure): paired fine (dp 0.005) / coarse
    (dp 0.02) data over seeded column heights, training on the GPU, then on a
    held-out height the probe pressures on the obstacle face and the surge
    front of the coarse run with and without the closure and of a plain run
    at dp 0.01, each against the plain fine run (dp 0.005, the judge), with
    the wall time of each run.  The target: the learned coarse run as
    accurate as the plain dp 0.01 run, in a fifth of its time."""
    from dualsphysics_gb300 import closure as cl
    rng = np.random.default_rng(args.clos_seed)
    heights = [float(h) for h in np.sort(rng.uniform(0.2, 0.5, args.clos_heights))]
    held, t_end, dtp = args.clos_held, args.clos_tend, 0.005
    dpf, ratio = args.clos_dpfine, args.clos_ratio
    dpc, dpm = dpf * ratio, dpf * ratio / 2
    val = heights[3::8]                                   # 4 of 32 heights validate (early stopping)
    train = [h for h in heights if h not in val]
    t0 = time.perf_counter()
    kw = dict(dp_fine=dpf, ratio=ratio, t_end=t_end, n_snap=args.clos_snaps, device=local,
              smooth=bool(args.clos_smooth), avg_steps=args.clos_avg)
    xs, ts, meta = cl.paired_samples(train, **kw)
    xv, tv, _ = cl.paired_samples(val, **kw)
    t_data = time.perf_counter() - t0
    t1 = time.perf_counter()
    p, w, loss = cl.train_closure(xs, ts, epochs=args.clos_epochs, seed=args.clos_seed, device=local, xv=xv, tv=tv)
    t_train = time.perf_counter() - t1
    xh, th, mh = cl.paired_samples([held], **kw)
    ev = cl.Trainer(cl.from_bf16(w), local)     # the deployed BF16 weights
    yh = ev.infer(xh)
    ev.close()
    coarse = cl._load(cl.spec(dpc, held, "HeldC"))
    hc = coarse.params.h
    judge = cl.run_with_probes(cl._load(cl.spec(dpf, held, "HeldJ")), t_end, dtp, device=local, mesh_h=hc)
    mid = cl.run_with_probes(cl._load(cl.spec(dpm, held, "HeldM")), t_end, dtp, device=local, mesh_h=hc)
    plain = cl.run_with_probes(coarse, t_end, dtp, device=local, mesh_h=hc)
    learned = cl.run_with_probes(coarse, t_end, dtp, w_bf16=w, limit=0.2, device=local, mesh_h=hc)
    km, kp, kl = f"plain_dp{dpm:g}", f"coarse_plain_dp{dpc:g}", f"coarse_learned_dp{dpc:g}"
    runs = {km: mid, kp: plain, kl: learned}
    err = {k: cl.errors(r, judge) for k, r in runs.items()}
    head = cl.HEADLINE_ERROR
    # more trainings on the same data with other seeds: the spread of the
    # learned run's errors (the data generation is the costly part)
    seeds = []
    for sd in range(1, max(1, args.clos_seeds)):
        _, w2, _ = cl.train_closure(xs, ts, epochs=args.clos_epochs, seed=args.clos_seed + sd, device=local,
                                    xv=xv, tv=tv)
        ev2 = cl.Trainer(cl.from_bf16(w2), local)
        yh2 = ev2.infer(xh)
        ev2.close()
        l2 = cl.run_with_probes(coarse, t_end, dtp, w_bf16=w2, limit=0.2, device=local, mesh_h=hc)
        seeds.append({"seed": args.clos_seed + sd, "errors": cl.errors(l2, judge),
                      "apriori_mse_raw": float(np.mean((mh["raw"] - yh2) ** 2))})
    speed = mid["wall_s"] / learned["wall_s"]
    converges = bool(err[km][head] < err[kp][head] and err[km]["front_rmse_m"] < err[kp]["front_rmse_m"])
    line = {"metric": f"learned vs plain time-to-accuracy ({head}, probes on the obstacle face)",
            "value": speed, "unit": f"x (plain dp={dpm:g} wall time / learned coarse wall time)", "n_gpus": 1,
            "higher_is_better": True, "data": "synthetic", "dtype": "bf16 weights, f32 accumulate",
            "config": {"workload": f"dam break with box obstacle, mDBC, tank height {cl.TANK_HEIGHT} m; held-out "
                                   f"column {held} m; {t_end} s; fine/judge dp={dpf:g}, coarse dp={dpc:g}",
                       "train_heights": len(train), "validation_heights": len(val),
                       "snapshots_per_height": args.clos_snaps,
                       "samples": int(len(xs)), "epochs": args.clos_epochs,
                       "targets": ("kernel-smoothed" if args.clos_smooth else "raw") +
                                  f", fine accelerations averaged over {args.clos_avg} fine steps"},
            "errors": err, "judge_converges": converges,
            "wall_s": {f"judge_dp{dpf:g}": judge["wall_s"], **{k: r["wall_s"] for k, r in runs.items()}},
            "ms_per_step": {f"judge_dp{dpf:g}": judge["ms_per_step"], **{k: r["ms_per_step"] for k, r in runs.items()}},
            "steps": {f"judge_dp{dpf:g}": judge["steps"], **{k: r["steps"] for k, r in runs.items()}},
            "particles": {"judge": judge["np"], "mid": mid["np"], "coarse": plain["np"]},
            "target_met": bool(converges and err[kl][head] <= err[km][head] and speed >= 5.0),
            "learned_vs_plain_error": err[kl][head] / err[kp][head],
            "apriori_heldout_mse": {"plain": float(np.mean(th ** 2)), "learned": float(np.mean((th - yh) ** 2)),
                                    "targets": "smoothed" if args.clos_smooth else "raw",
                                    "raw_plain": float(np.mean(mh["raw"] ** 2)),
                                    "raw_learned": float(np.mean((mh["raw"] - yh) ** 2))},
            "train": {"loss_first": float(loss[0]), "loss_last": float(loss[-1]), "data_s": t_data,
                      "train_s": t_train, "fine_steps": meta["fine_steps"]},
            "fallback_rows": learned["fallbacks"]}
    if seeds:
        allh = [err[kl][head]] + [sd["errors"][head] for sd in seeds]
        line["other_seeds"] = seeds
        line["learned_error_over_seeds"] = {"n": len(allh), "min": min(allh), "max": max(allh),
                                            "mean": float(np.mean(allh)), "plain": err[kp][head]}
    print(json.dumps(line))


def run_closure_judge(args, local: int = 0):
    """Convergence of the closure's error measures (--workload closure-judge):
    plain runs of the held-out column at the spacings --clos-judge-dps, each
    judged against the finest."""
    from dualsphysics_gb300 import closure as cl
    dps = [float(v) for v in args.clos_judge_dps.split(",")]
    t0 = time.perf_counter()
    res = cl.judge_study(args.clos_held, dps, t_end=args.clos_tend, device=local,
                         log=lambda m: print(m, file=sys.stderr, flush=True))
    print(json.dumps({"workload": "closure-judge", "column": args.clos_held, "t_end": args.clos_tend,
                      "reference_dp": min(dps), "by_dp": {f"{k:g}": v for k, v in res.items()},
                      "total_s": time.perf_counter() - t0}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb", choices=["gb", "reference"])
    ap.add_argument("--dp", type=float, default=0.0025)
    ap.add_argument("--cpu-steps", type=int, default=None,
                    help="full oracle steps timed for cpu_baseline (default 2; 1 for c3)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cellmode", default="full", choices=["full", "half"],
                    help="the reference's -cellmode run option: cells of 2h (default) or h")
    ap.add_argument("--variant", type=int, default=None,
                    help="fluid-row kernel: 0 queued rounds, 1 one thread per particle, 2/3 cell-tiled staged "
                         "(ring of 8/4 chunks); default: the library's")
    ap.add_argument("--split", type=int, default=None, choices=[0, 1, 2, 4],
                    help="warps per group of 32 fluid rows in the cell-tiled kernel (0 automatic); default: the "
                         "library's")
    ap.add_argument("--bound-lanes", type=int, default=None, choices=[0, 1, 4, 32],
                    help="lanes a boundary row in the bound-row pass (0 automatic); default: the library's")
    ap.add_argument("--mdbc-split", type=int, default=None, choices=[0, 1, 2, 4],
                    help="warps per group of 32 boundary rows in the cell-tiled mDBC kernel (0 automatic); "
                         "default: the library's")
    ap.add_argument("--bound-beside", type=int, default=None, choices=[0, 1],
                    help="the bound-row pass on a side stream beside the fluid-row pass; default: the library's")
    ap.add_argument("--no-tune", action="store_true", help="keep the 8-bit sort digits (no sort autotuning)")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c3err", "ensemble", "closure",
                                                         "closure-judge"],
                    help="c2: the dam break with obstacle (default); c3: the large plain run (dp 0.004, "
                         "~49 M particles); ensemble: the batched cases; closure: the learned closure against "
                         "fine runs")
    ap.add_argument("--clos-heights", type=int, default=32)
    ap.add_argument("--clos-snaps", type=int, default=8)
    ap.add_argument("--clos-epochs", type=int, default=40)
    ap.add_argument("--clos-held", type=float, default=0.3)
    ap.add_argument("--clos-tend", type=float, default=0.3)
    ap.add_argument("--clos-seed", type=int, default=5)
    ap.add_argument("--clos-dpfine", type=float, default=0.005)
    ap.add_argument("--clos-ratio", type=int, default=4, choices=[2, 4])
    ap.add_argument("--clos-smooth", type=int, default=1, choices=[0, 1],
                    help="train on kernel-smoothed targets (closure.smooth_targets)")
    ap.add_argument("--clos-seeds", type=int, default=1,
                    help="trainings (seeds) on the same data; the spread of the learned run's errors")
    ap.add_argument("--clos-avg", type=int, default=8,
                    help="fine steps the fine block-mean acceleration is averaged over (about one coarse step)")
    ap.add_argument("--clos-judge-dps", default="0.02,0.01,0.005,0.0025")
    ap.add_argument("--ens-cases", type=int, default=64)
    ap.add_argument("--ens-seed", type=int, default=1)
    ap.add_argument("--ens-scale", type=float, default=1.0, help="scales every case's particle count")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.workload in ("c3", "c3err") and args.dp == 0.0025:
        args.dp = 0.004
    if args.workload == "c3err" and args.steps == 20:
        args.steps = 200
    if args.cpu_steps is None:
        args.cpu_steps = 1 if args.workload == "c3" else 2

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo", init_method="env://")
        dist = dist_mod

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, make_case(args.dp, args.cellmode, args.workload), rank)
        if dist:
            dist.destroy_process_group()
        return

    if args.workload in ("ensemble", "closure", "c3err", "closure-judge"):
        if rank == 0:
            {"ensemble": run_ensemble, "closure": run_closure, "c3err": run_c3err,
             "closure-judge": run_closure_judge}[args.workload](args, local)
        if dist:
            dist.destroy_process_group()
        return

    from dualsphysics_gb300 import _lib
    from dualsphysics_gb300.sph import GbSphSingle

    cd = make_case(args.dp, args.cellmode, args.workload)
    K, W = args.steps, args.warmup
    s = GbSphSingle(local)
    s.setup(cd)
    # the sort autotuner (outside the timed region; both digit widths give the
    # same particle order, so the run is unchanged)
    import ctypes as C
    sort_bits, sort_ms = C.c_int(8), (C.c_float * 2)()
    if not args.no_tune:
        s._check(_lib.lib().gbsph_tune_sort(s.ctx, 3, C.byref(sort_bits), sort_ms), "gbsph_tune_sort")
    if args.variant is not None:
        s.set_option(1, args.variant)
    if args.split is not None:
        s.set_option(4, args.split)
    if args.bound_lanes is not None:
        s.set_option(6, args.bound_lanes)
    if args.mdbc_split is not None:
        s.set_option(8, args.mdbc_split)
    if args.bound_beside is not None:
        s.set_option(10, args.bound_beside)
    variant, split, blanes, msplit = s.get_option(1), s.get_option(5), s.get_option(7), s.get_option(9)
    beside = s.get_option(10)
    pi = s.pips()
    s.RunSteps(W, use_graph=True)
    s.sync()
    # timed region: K steps from one captured graph, fluid forces bracketed by events
    s.profile(2 * K)
    s.graph_prepare(K)
    l0 = s.launch_count()
    if dist:
        dist.barrier()
    s.sync()
    with ClockSampler(local) as clk:
        s.mark(0)
        s.RunSteps(K, use_graph=2)
        s.mark(1)
        ms = s.elapsed(0, 1)
    s.sync()
    launches = s.launch_count() - l0
    kms = s.profile_read()
    s.profile(0)
    t_max, steps_per_s = replica_throughput(ms, K, dist, world)
    pis_per_step = 2.0 * (pi["real_fluid"] + pi["real_bound"])
    info = s.divinfo()
    # roofline of the fluid Interaction_Forces kernel
    peaks, src = _peaks()
    kavg = float(np.mean(kms)) if len(kms) else float("nan")
    bytes_launch = BYTES_PER_FLUID_ROW * cd.nfluid + BYTES_PER_BOUND_NEIGHBOUR * cd.npb
    ach = bytes_launch / (kavg / 1e3) / 1e9
    gather_gbs = BYTES_PER_CHECKED * pi["checked_fluid"] / (kavg / 1e3) / 1e9
    flops_launch = FLOP_PER_FLUID_PAIR * pi["real_fluid"]
    # e2e through the C ABI with host buffers
    s.close()
    e2e = None
    if rank == 0 or world > 1:
        # inputs and outputs in pinned host memory (prepared outside the timed region)
        pcd = _pinned_case(cd)
        n = cd.np
        out = {"pos": _pinned((n, 3), np.float64), "velrho": _pinned((n, 4), np.float32),
               "idp": _pinned((n,), np.uint32), "code": _pinned((n,), np.uint16), "dcell": _pinned((n,), np.uint32)}
        t0 = time.perf_counter()
        e = GbSphSingle(local)
        e.setup(pcd)
        e.set_option(2, sort_bits.value)   # the tuned sort width, set as a caller would
        if args.variant is not None:
            e.set_option(1, args.variant)
        if args.split is not None:
            e.set_option(4, args.split)
        if args.bound_lanes is not None:
            e.set_option(6, args.bound_lanes)
        if args.mdbc_split is not None:
            e.set_option(8, args.mdbc_split)
        if args.bound_beside is not None:
            e.set_option(10, args.bound_beside)
        for _ in range(K):
            e.RunSteps(1, use_graph=True)  # one step, replayed from its captured graph
            e.step_dt()                    # the Run loop reads the step's dt and time back
        e.download_into(out)
        te = time.perf_counter() - t0
        h2d = cd.pos.nbytes + cd.velrho.nbytes + cd.idp.nbytes + cd.code.nbytes + \
            (cd.boundnor.nbytes if cd.boundnor is not None else 0)
        d2h = sum(v.nbytes for v in out.values()) + K * 24
        e2e = {"value": world * K / te, "unit": "steps/s", "h2d_bytes_per_step": int(h2d / K),
               "d2h_bytes_per_step": int(d2h / K)}
        e.close()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        t_cpu, cores = cpu_baseline(cd, args.cpu_steps)
        cpu = {"value": 1.0 / t_cpu, "unit": "steps/s", "cores": cores, "kind": "port",
               "sample": f"{args.cpu_steps} full oracle steps of the same state (timing build: the reference's "
                         f"-O3 -ffast-math; within 4% of the reference's own solver on C1, same threads)"}
    clks = clk.summary()
    traffic = _dram_traffic(variant, args.dp)
    fp32_nominal = None
    if clks.get("sm_mhz"):
        fp32_nominal = _sm_count(local) * FP32_LANES_PER_SM * 2 * clks["sm_mhz"] * 1e6 / 1e12
    # the measured FP32 rate: FFMA microbenchmark on this device, after the timed region
    import ctypes as C
    ff = C.c_float()
    fp32_peak = float(ff.value) if _lib.lib().gbsph_ffma_peak(local, C.byref(ff)) == 0 and ff.value > 0 else None
    fp32_src = "measured: FFMA microbenchmark (gbsph_ffma_peak), best of 5 launches"
    if fp32_peak is None:
        fp32_peak, fp32_src = fp32_nominal, "nominal FFMA rate (SMs x 128 lanes x 2 FLOP) at the sampled SM clock"
    if rank == 0:
        line = {
            "metric": METRIC, "value": steps_per_s, "unit": "steps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": t_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 positions and integration)", "data": "synthetic",
            "config": {"workload": workload_text(args),
                       "particles": cd.np, "fluid": cd.nfluid, "boundary": cd.npb, "cellmode": args.cellmode,
                       "sort_digit_bits": sort_bits.value, "fluid_kernel_variant": variant,
                       "warps_per_row_group": split, "lanes_per_bound_row": blanes,
                       "warps_per_mdbc_row_group": msplit, "bound_rows_beside_fluid_rows": beside,
                       "sort_divide_ms_8_11": [round(float(x), 4) for x in sort_ms] if not args.no_tune else None,
                       "parallelism": "replicas only" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (no flush)"},
            "particle_interactions_per_s": steps_per_s * pis_per_step,
            "particle_interactions_per_step": pis_per_step,
            "np_after": info["np"],
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": ach / peaks["hbm_gbs"], "traffic": traffic,
                         "kernel": KERNEL_NAME.get(variant, str(variant)),
                         "model": "52 B per fluid row + 32 B per boundary neighbour per launch",
                         "peak_source": src, "launch_ms": kavg, "launches_timed": int(len(kms)),
                         "gather_gbs": gather_gbs},
            "roofline_fp32": {"achieved_tflops": flops_launch / (kavg / 1e3) / 1e12, "peak_tflops": fp32_peak,
                              "frac": flops_launch / (kavg / 1e3) / 1e12 / fp32_peak if fp32_peak else None,
                              "model": "80 FLOP per real fluid-row pair",
                              "peak_source": fp32_src, "nominal_tflops": fp32_nominal},
            "clocks": clks,
            "gpu_launches": int(launches),
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
