"""Cross-timing of the oracle (the CPU restatement of the reference step) against
the reference's own CPU solver, on the same case, the same number of steps and
the same number of threads, in this container.

TEST INFRASTRUCTURE: it states how fast the timed CPU baseline (the oracle,
which is what runs on the GPU machine's host cores, where the reference's sources
are absent) is next to the reference's own code.

    python oracle/crosstime.py [--dp 0.01] [--steps 10] [--threads 8]

The reference side is oracle/_ref/ref_harness (make -f oracle/Makefile.ref
REFSRC=<reference>/src/source) in its timing mode: the case is loaded and
divided, then <steps> steps of its Run loop (ComputeStep + RunCellDivide,
JSphCpuSingle.cpp:1183-1196) are timed.  The oracle side times the same steps
of orc_sim_step after its initial divide.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dp", type=float, default=0.01)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--workload", default="c1", choices=["c1", "c2"])
    ap.add_argument("--build", default="timing", choices=["timing", "checker"],
                    help="the oracle build timed: the timing build (bench.py's CPU legs) or the checker")
    args = ap.parse_args()
    from dualsphysics_gb300 import casegen as cg
    from dualsphysics_gb300.case import load_case
    harness = os.path.join(HERE, "_ref", "ref_harness")
    if not os.path.exists(harness):
        sys.exit(f"reference harness not built: {harness}")
    spec = (cg.spec_c1 if args.workload == "c1" else cg.spec_c2)(dp=args.dp, name="Cross")
    with tempfile.TemporaryDirectory() as tmp:
        casedir, outdir = os.path.join(tmp, "case"), os.path.join(tmp, "out")
        os.makedirs(outdir)
        cg.write_case(cg.make_dam_break(spec), casedir)
        with open(os.path.join(casedir, "timing.txt"), "w") as f:
            f.write(f"{args.steps}\n")
        subprocess.run([harness, casedir, "Cross", outdir, "0", str(args.threads)], check=True,
                       stdout=subprocess.DEVNULL)
        with open(os.path.join(outdir, "timing_out.txt")) as f:
            tok = f.read().split()
        ref_s, ref_np = float(tok[3]), int(tok[5])
        os.environ["OMP_NUM_THREADS"] = str(args.threads)
        import pyoracle as po
        po.build()
        if args.build == "timing":
            po.use_timing_build()
        cd = load_case(casedir, "Cross")
        sim = po.Sim(po.config(po.params_from(cd.params)), cd.pos, cd.velrho, cd.idp, cd.code, cd.npb, cd.boundnor,
                     nthreads=args.threads)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            sim.step()
        orc_s = time.perf_counter() - t0
    out = {"workload": args.workload, "dp": args.dp, "particles": ref_np, "steps": args.steps, "build": args.build,
           "threads": args.threads, "reference_steps_per_s": args.steps / ref_s,
           "oracle_steps_per_s": args.steps / orc_s, "oracle_over_reference_time": orc_s / ref_s}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
