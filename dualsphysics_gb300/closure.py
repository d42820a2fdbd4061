"""Learned closure for coarse runs (no reference counterpart).

A 16-64-64-64-3 tanh MLP (BF16 weights, FP32 accumulation) adds a per-particle
correction to the fluid accelerations of a coarse run.  It is trained on data
the method generates itself:

* a fine run (spacing dp) of the dam break with the box obstacle;
* every fine fluid particle belongs to the coarse particle of its initial
  lattice block (fine indices ri..ri+r-1 per axis for a spacing ratio r of 2
  or 4; the fine particle at the block's corner starts where the coarse
  particle starts).  At snapshot
  times the fine state restricted to the blocks -- the corner particle's
  position, the block's mean velocity and density -- with the coarse case's
  own walls is a coarse state;
* the target of each coarse particle is (the block's mean fine acceleration
  - the coarse acceleration of the restricted state) / |g| (the block mean is
  the force on the block's mass, which removes most of the particle-scale
  noise of single fine accelerations); the inputs are the closure features
  of the restricted state (``gbsph_closure_features``).

Training, inference and the correction inside the step run in the library's
own kernels (``gbsph_mlp_*``, ``gbsph_closure_set``); the plain method is the
fallback (per particle, when the correction exceeds ``limit`` x |ace|) and the
judge (the plain fine run's probe pressures and surge front).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import tempfile
import time

import numpy as np

from . import casegen as cg
from ._lib import GbsphError, INTERSTEP_SYMPREDICTOR, lib, ptr
from .case import load_case
from .sph import GbSphSingle

NFEAT = 16
NHID = 64
NOUT = 3
NPARAMS = NHID * NFEAT + NHID + 2 * (NHID * NHID + NHID) + NOUT * NHID + NOUT
TANK_HEIGHT = 0.6   # room for columns up to 0.5 m
# the error measure the closure is judged by (a key of errors())
HEADLINE_ERROR = "probe_rmse_pa_20ms_means"


def layer_slices():
    """(W, b) slices of the flat parameter vector, layers 0..3."""
    out, o = [], 0
    for nin, nout in ((NFEAT, NHID), (NHID, NHID), (NHID, NHID), (NHID, NOUT)):
        w = slice(o, o + nin * nout)
        o += nin * nout
        b = slice(o, o + nout)
        o += nout
        out.append((w, b, nout, nin))
    assert o == NPARAMS
    return out


def init_params(seed: int = 0, out_scale: float = 0.1) -> np.ndarray:
    """Glorot-uniform weights, zero biases; the output layer scaled down so the
    untrained correction is small."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float32)
    for k, (w, b, nout, nin) in enumerate(layer_slices()):
        lim = math.sqrt(6.0 / (nin + nout)) * (out_scale if k == 3 else 1.0)
        p[w] = rng.uniform(-lim, lim, nout * nin).astype(np.float32)
    return p


def to_bf16(p: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even BF16 bit patterns of float32 values."""
    u = np.ascontiguousarray(p, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def from_bf16(b: np.ndarray) -> np.ndarray:
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


class Trainer:
    """gbsph_mlp: data on the device, FP32 master weights + BF16 copy, Adam."""

    def __init__(self, params: np.ndarray, device: int = 0):
        self.m = C.c_void_p()
        p = np.ascontiguousarray(params, np.float32)
        rc = lib().gbsph_mlp_create(device, ptr(p), C.byref(self.m))
        if rc:
            raise GbsphError(rc, "gbsph_mlp_create")

    def _check(self, rc, what):
        if rc:
            raise GbsphError(rc, what)

    def set_data(self, x: np.ndarray, t: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        assert x.shape[1] == NFEAT and t.shape == (x.shape[0], NOUT)
        self._check(lib().gbsph_mlp_set_data(self.m, ptr(x), ptr(t), x.shape[0]), "gbsph_mlp_set_data")
        self.n = x.shape[0]

    def grad(self, first: int = 0, n: int | None = None) -> tuple[np.ndarray, float]:
        n = self.n - first if n is None else n
        g = np.empty(NPARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        self._check(lib().gbsph_mlp_grad(self.m, first, n, ptr(g), ptr(loss)), "gbsph_mlp_grad")
        return g, float(loss[0])

    def train(self, epochs: int, batch: int, lr: float) -> np.ndarray:
        loss = np.empty(epochs, np.float32)
        self._check(lib().gbsph_mlp_train(self.m, epochs, batch, lr, ptr(loss)), "gbsph_mlp_train")
        return loss

    def infer(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty((x.shape[0], NOUT), np.float32)
        self._check(lib().gbsph_mlp_infer(self.m, ptr(x), x.shape[0], ptr(y)), "gbsph_mlp_infer")
        return y

    def params(self) -> tuple[np.ndarray, np.ndarray]:
        master = np.empty(NPARAMS, np.float32)
        w = np.empty(NPARAMS, np.uint16)
        self._check(lib().gbsph_mlp_params(self.m, ptr(master), ptr(w)), "gbsph_mlp_params")
        return master, w

    def close(self):
        if self.m:
            lib().gbsph_mlp_destroy(self.m)
            self.m = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fold_standardisation(p: np.ndarray, mu_x, sd_x, sd_t) -> np.ndarray:
    """Parameters of a network trained on standardised data ((x - mu_x)/sd_x
    in, t/sd_t out) rewritten to take raw features and give raw targets: the
    input scaling goes into W0 and b0, the output scaling into W3 and b3."""
    q = np.array(p, np.float64)
    (w0, b0, _, _), _, _, (w3, b3, _, _) = layer_slices()
    W0 = q[w0].reshape(NHID, NFEAT) / sd_x[None, :]
    q[b0] = q[b0] - W0 @ mu_x
    q[w0] = W0.ravel()
    q[w3] = (q[w3].reshape(NOUT, NHID) * sd_t[:, None]).ravel()
    q[b3] = q[b3] * sd_t
    return q.astype(np.float32)


def train_closure(x: np.ndarray, t: np.ndarray, epochs: int = 40, batch: int = 1024, lr: float = 1e-3,
                  seed: int = 0, device: int = 0, xv: np.ndarray | None = None, tv: np.ndarray | None = None,
                  check_every: int = 5) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Trains on standardised features and targets (zero mean and unit
    variance per column; constant columns left as they are), in a seeded
    shuffled order, and returns the folded FP32 parameters, their BF16 bits
    and the per-epoch losses (in standardised units).  With validation data
    (xv, tv: runs not trained on), the weights kept are those of the
    `check_every`-epoch checkpoint with the lowest validation error (early
    stopping), the untrained network's included."""
    x = np.asarray(x, np.float32)
    t = np.asarray(t, np.float32)
    mu = x.mean(axis=0).astype(np.float64)
    sd = x.std(axis=0).astype(np.float64)
    const = sd < 1e-6
    mu[const], sd[const] = 0.0, 1.0
    st = np.maximum(t.std(axis=0).astype(np.float64), 1e-6)
    order = np.random.default_rng(seed).permutation(len(x))
    xs = ((x[order] - mu) / sd).astype(np.float32)
    ts = (t[order] / st).astype(np.float32)
    tr = Trainer(init_params(seed), device)
    try:
        tr.set_data(xs, ts)
        if xv is None:
            loss = tr.train(epochs, batch, lr)
            master, _ = tr.params()
        else:
            xvs = ((np.asarray(xv, np.float32) - mu) / sd).astype(np.float32)
            tvs = (np.asarray(tv, np.float32) / st).astype(np.float32)
            master, _ = tr.params()
            best = float(np.mean((tr.infer(xvs) - tvs) ** 2))
            losses = []
            for _ in range(max(1, epochs // check_every)):
                losses.append(tr.train(check_every, batch, lr))
                v = float(np.mean((tr.infer(xvs) - tvs) ** 2))
                if v < best:
                    best, (master, _) = v, tr.params()
            loss = np.concatenate(losses)
    finally:
        tr.close()
    p = fold_standardisation(master, mu, sd, st)
    return p, to_bf16(p), loss


def attach(sim: GbSphSingle, w_bf16: np.ndarray | None, limit: float = 0.2) -> None:
    """Turns the closure on (or off with None) for every later step of `sim`."""
    w = None if w_bf16 is None else np.ascontiguousarray(w_bf16, np.uint16)
    sim._check(lib().gbsph_closure_set(sim.ctx, ptr(w), float(limit)), "gbsph_closure_set")


def fallbacks(sim: GbSphSingle) -> int:
    n = C.c_ulonglong()
    sim._check(lib().gbsph_closure_fallbacks(sim.ctx, C.byref(n)), "gbsph_closure_fallbacks")
    return int(n.value)


def features(sim: GbSphSingle) -> np.ndarray:
    """Closure features of the fluid rows (after Interaction_Forces)."""
    info = sim.divinfo()
    out = np.empty((info["np"] - info["npb"], NFEAT), np.float32)
    sim._check(lib().gbsph_closure_features(sim.ctx, ptr(out)), "gbsph_closure_features")
    return out


# ---- the paired fine / coarse data --------------------------------------------
def spec(dp: float, height: float, name: str) -> cg.CaseSpec:
    """The dam break with the box obstacle and mDBC (the C2 geometry), a
    column of the given height, in a tank raised to TANK_HEIGHT."""
    return cg.spec_c2(dp=dp, name=name, tank=(1.6, 0.67, TANK_HEIGHT), column=(0.4, 0.67, height), hswl=height)


def _load(s: cg.CaseSpec):
    tmp = tempfile.mkdtemp(prefix="gbclos_")
    cg.write_case(cg.make_dam_break(s), tmp)
    return load_case(tmp, s.name)


def lattice_key(pos: np.ndarray, dp: float) -> np.ndarray:
    """(k, j, i) lattice indices of initial fluid positions, as one sortable key."""
    idx = np.rint(pos / dp).astype(np.int64)
    return (idx[:, 2] * 100000 + idx[:, 1]) * 100000 + idx[:, 0], idx


class Pair:
    """A fine case and its coarse twin (spacing x ratio, ratio 2 or 4); maps
    fine fluid ids to coarse fluid rows: the fine lattice point ratio*i of
    every axis is the coarse lattice point i, and each fine particle belongs
    to the coarse block floor(i/ratio)."""

    def __init__(self, height: float, dp_fine: float = 0.01, tag: str = "P", ratio: int = 2):
        self.height = height
        self.ratio = r = int(ratio)
        self.fine = _load(spec(dp_fine, height, f"{tag}F"))
        self.coarse = _load(spec(r * dp_fine, height, f"{tag}C"))
        f, c = self.fine, self.coarse
        fpos = f.pos[f.npb:]
        _, idx = lattice_key(fpos, dp_fine)
        corner = np.all(idx % r == 0, axis=1)
        fkey, _ = lattice_key(fpos[corner] / float(r), dp_fine)
        ckey, _ = lattice_key(c.pos[c.npb:], r * dp_fine)
        # coarse fluid row r <- the fine fluid particle with the same lattice point
        order_f = np.argsort(fkey)
        order_c = np.argsort(ckey)
        if len(fkey) != len(ckey) or not np.array_equal(fkey[order_f], ckey[order_c]):
            raise ValueError("fine and coarse lattices do not nest")
        fine_ids = f.idp[f.npb:][np.nonzero(corner)[0]]
        self.coarse_row_fine_id = np.empty(len(ckey), np.int64)
        self.coarse_row_fine_id[order_c] = fine_ids[order_f]
        # block of every fine fluid particle: the coarse row of lattice point floor(idx/ratio)
        bkey, _ = lattice_key((idx // r).astype(np.float64), 1.0)
        pos_c = np.searchsorted(ckey[order_c], bkey)
        if (pos_c >= len(ckey)).any() or not np.array_equal(ckey[order_c][pos_c], bkey):
            raise ValueError("a fine particle has no coarse block")
        self.fine_id = f.idp[f.npb:].astype(np.int64)
        self.fine_block = order_c[pos_c]                     # coarse fluid row of each fine fluid particle

    def block_mean(self, fst: dict, values: np.ndarray) -> np.ndarray:
        """Mean of per-row `values` of the fine state over each coarse block
        (the fine particles still present)."""
        where = np.full(int(fst["idp"].max()) + 1, -1, np.int64)
        where[fst["idp"]] = np.arange(len(fst["idp"]))
        rows = where[np.minimum(self.fine_id, len(where) - 1)]
        ok = (self.fine_id < len(where)) & (rows >= 0)
        nc = self.coarse.np - self.coarse.npb
        v = np.asarray(values, np.float64)[rows[ok]]
        blk = self.fine_block[ok]
        cnt = np.bincount(blk, minlength=nc).astype(np.float64)
        if v.ndim == 1:
            sums = np.bincount(blk, weights=v, minlength=nc)
        else:
            sums = np.stack([np.bincount(blk, weights=v[:, k], minlength=nc) for k in range(v.shape[1])], axis=1)
        return sums / np.maximum(cnt, 1.0).reshape((nc,) + (1,) * (v.ndim - 1)), cnt

    def coarse_state(self, fst: dict):
        """The coarse case with its fluid rows taken from the fine state
        `fst` (download of the fine run): corner particle positions, block
        mean velocity and density; None if a corner particle left the domain."""
        c = self.coarse
        where = np.full(int(fst["idp"].max()) + 1, -1, np.int64)
        where[fst["idp"]] = np.arange(len(fst["idp"]))
        rows = where[self.coarse_row_fine_id]
        if (rows < 0).any():
            return None
        import copy
        cd = copy.copy(c)
        cd.pos = c.pos.copy()
        cd.velrho = c.velrho.copy()
        cd.pos[c.npb:] = fst["pos"][rows]
        vr, _ = self.block_mean(fst, fst["velrho"])
        cd.velrho[c.npb:] = vr.astype(np.float32)
        return cd, rows


def smooth_targets(pos: np.ndarray, t: np.ndarray, h: float) -> np.ndarray:
    """Kernel-weighted (Wendland, support 2h) Shepard mean of the targets of
    each particle's neighbours, itself included: the part of the fine-minus-
    coarse acceleration that varies over the kernel's scale, without the
    particle-scale noise no local feature can predict."""
    from scipy.spatial import cKDTree
    tree = cKDTree(pos)
    pairs = tree.query_pairs(2.0 * h, output_type="ndarray")
    i, j = pairs[:, 0], pairs[:, 1]
    q = np.linalg.norm(pos[i] - pos[j], axis=1) / h
    w = (1.0 - 0.5 * q) ** 4 * (2.0 * q + 1.0)
    n = len(pos)
    num = np.array(t, np.float64)          # the particle itself, W(0) = 1
    den = np.ones(n)
    for k in range(t.shape[1]):
        num[:, k] += np.bincount(i, weights=w * t[j, k], minlength=n) + np.bincount(j, weights=w * t[i, k], minlength=n)
    den += np.bincount(i, weights=w, minlength=n) + np.bincount(j, weights=w, minlength=n)
    return (num / den[:, None]).astype(np.float32)


def paired_samples(heights, dp_fine: float = 0.01, t_end: float = 0.3, n_snap: int = 10,
                   device: int = 0, log=None, ratio: int = 2, smooth: bool = False,
                   avg_steps: int = 1) -> tuple[np.ndarray, np.ndarray, dict]:
    """Features and targets over fine runs of the given column heights,
    restricted to the coarse particles (spacing ratio*dp_fine) at n_snap
    times in (0, t_end].  With avg_steps > 1, the fine block-mean
    acceleration is averaged over that many consecutive fine steps from the
    snapshot (about one coarse step for avg_steps = 2 * ratio: the mean fine
    acceleration over the coarse step's interval, without the fine run's
    acoustic oscillations); the coarse state and features are those of the
    snapshot.  With smooth, the targets are replaced by their kernel-weighted
    neighbourhood means (smooth_targets); meta["raw"] keeps the raw ones."""
    xs, ts, raw, meta = [], [], [], {"snapshots": 0, "fine_steps": 0, "fine_s": 0.0}
    g = 9.81
    for hk, h in enumerate(heights):
        pair = Pair(h, dp_fine, tag=f"H{hk}", ratio=ratio)
        fine = GbSphSingle(device)
        fine.setup(pair.fine)
        tnext = t_end / n_snap
        t0 = time.perf_counter()
        while True:
            fine.RunSteps(1, use_graph=True)
            meta["fine_steps"] += 1
            t = fine.step_dt()[2]
            if t < tnext:
                continue
            tnext += t_end / n_snap
            # fine accelerations of this state
            fine.MdbcBoundCorrection(INTERSTEP_SYMPREDICTOR)
            fine.Interaction_Forces(INTERSTEP_SYMPREDICTOR)
            fst = fine.download()
            face, _ = fine.forces()
            got = pair.coarse_state(fst)
            if got is not None:
                cd, rows = got
                cs = GbSphSingle(device)
                cs.setup(cd)
                cs.MdbcBoundCorrection(INTERSTEP_SYMPREDICTOR)
                cs.Interaction_Forces(INTERSTEP_SYMPREDICTOR)
                cst = cs.download()
                cace, _ = cs.forces()
                x = features(cs)
                cs.close()
                crow = cst["idp"][cst["idp"] >= cd.npb] - cd.npb    # coarse fluid row of each feature row
                fmean, _ = pair.block_mean(fst, face)               # block mean of the fine accelerations
                for _ in range(1, max(1, avg_steps)):               # averaged over the next fine steps
                    fine.RunSteps(1, use_graph=True)
                    meta["fine_steps"] += 1
                    fine.MdbcBoundCorrection(INTERSTEP_SYMPREDICTOR)
                    fine.Interaction_Forces(INTERSTEP_SYMPREDICTOR)
                    fm, _ = pair.block_mean(fine.download(), fine.forces()[0])
                    fmean = fmean + fm
                fmean = fmean / max(1, avg_steps)
                t = fine.step_dt()[2]
                tgt = (fmean[crow] - cace[cd.npb:cd.npb + len(crow)]) / g
                ok = np.isfinite(x).all(axis=1) & np.isfinite(tgt).all(axis=1)
                xs.append(x[ok])
                raw.append(tgt[ok].astype(np.float32))
                if smooth:
                    fpos = cst["pos"][cd.npb:cd.npb + len(crow)].astype(np.float64)
                    ts.append(smooth_targets(fpos[ok], tgt[ok], float(cd.params.h)))
                else:
                    ts.append(tgt[ok].astype(np.float32))
                meta["snapshots"] += 1
            if t >= t_end - 1e-12:
                break
        meta["fine_s"] += time.perf_counter() - t0
        fine.close()
        if log:
            log(f"height {h:.3f}: {sum(len(x) for x in xs)} samples")
    meta["raw"] = np.concatenate(raw)
    return np.concatenate(xs), np.concatenate(ts), meta


# ---- evaluation against the fine run ---------------------------------------------
def probe_mesh(h: float):
    """Pressure probes on the obstacle's upstream face, 1.5 h off it: a grid
    of 10 heights (z = 0.02 to 0.20 m) by 5 positions across the face (from
    0.01 m inside either edge)."""
    x0, y0, sx, sy, sz = cg.OBSTACLE_C2
    return dict(ptref=(x0 - 1.5 * h, y0 + 0.01, 0.02), vec1=(0.0, 0.0, 1.0), vec2=(0.0, 1.0, 0.0),
                vec3=(1.0, 0.0, 0.0), dis=(0.18, sy - 0.02, 0.0), dispt=(0.02, (sy - 0.02) / 4, 0.0))


def probe_pressure(gs, rhop) -> np.ndarray:
    """Probe pressures (Pa) from a mesh gauge's densities: the Tait pressure
    where the probe is wet, 0 (the atmosphere) where it is dry.  A dry probe
    (kernel sum below the gauge's limit) reads the dummy density 0, whose Tait
    pressure -B would turn a few ms of difference in the arrival of the front
    into errors of the order of B."""
    r = np.asarray(rhop, np.float64)
    return np.where(r > 0, gs.Pressure(r), 0.0)


def run_with_probes(cd, t_end: float, dt_probe: float, w_bf16=None, limit: float = 0.2, device: int = 0,
                    mesh_h: float | None = None, chunk: int = 10) -> dict:
    """Runs a case to t_end in replays of one graph holding `chunk` steps,
    sampling the probes and the surge front after the first chunk that passes
    each multiple of dt_probe; returns them with their times, the wall time of
    the stepping alone and its steps."""
    from .gauges import GaugeSystem
    s = GbSphSingle(device)
    s.setup(cd)
    if w_bf16 is not None:
        attach(s, w_bf16, limit)
    gs = GaugeSystem(s)
    m = probe_mesh(mesh_h if mesh_h is not None else cd.params.h)
    gs.AddGaugeMesh("probes", **m)
    times, press, fronts = [], [], []
    tnext, t, wall, nsteps = dt_probe, 0.0, 0.0, 0
    s.graph_prepare(chunk)                  # one graph of `chunk` steps, captured outside the clock
    while t < t_end:
        s.sync()
        t0 = time.perf_counter()
        s.RunSteps(chunk, use_graph=2)
        t = s.step_dt()[2]
        wall += time.perf_counter() - t0
        nsteps += chunk
        if t >= tnext:
            tnext += dt_probe
            gs.CalculeGpu(t)
            times.append(t)
            press.append(probe_pressure(gs, gs.GetResult("probes")["rhop"]))
            fronts.append(s.fluid_front((1.0, 0.0, 0.0))[0])
    out = {"t": np.array(times), "p": np.array(press), "front": np.array(fronts), "wall_s": wall, "steps": nsteps,
           "ms_per_step": 1e3 * wall / max(nsteps, 1), "np": cd.np,
           "fallbacks": fallbacks(s) if w_bf16 is not None else 0}
    s.close()
    return out


def front_error(run: dict, ref: dict) -> float:
    """RMS difference of the surge front (largest fluid x) against the reference run (m)."""
    n = min(len(run["t"]), len(ref["t"]))
    if n == 0:
        return float("nan")
    return float(np.sqrt(np.mean((run["front"][:n] - np.interp(run["t"][:n], ref["t"], ref["front"])) ** 2)))


def _window_means(run: dict, ref: dict, window: float):
    tmax = min(run["t"][-1], ref["t"][-1])
    edges = np.arange(0.0, tmax + 1e-12, window)
    a, b = [], []
    for lo, hi in zip(edges[:-1], edges[1:]):
        ma = (run["t"] > lo) & (run["t"] <= hi)
        mb = (ref["t"] > lo) & (ref["t"] <= hi)
        if ma.any() and mb.any():
            a.append(run["p"][ma].mean(axis=0))
            b.append(ref["p"][mb].mean(axis=0))
    return np.array(a), np.array(b)


def probe_error(run: dict, ref: dict, window: float = 0.0) -> float:
    """RMS difference of the probe pressures against the reference run (Pa).
    window 0: sample by sample, the reference interpolated to the run's
    times; window > 0: of the means over consecutive windows of that length
    (impact peaks last a few ms, so sample-wise differences are dominated by
    their timing)."""
    n = min(len(run["t"]), len(ref["t"]))
    if n == 0:
        return float("nan")
    if window <= 0:
        pr = np.stack([np.interp(run["t"][:n], ref["t"], ref["p"][:, k]) for k in range(ref["p"].shape[1])], axis=1)
        return float(np.sqrt(np.mean((run["p"][:n] - pr) ** 2)))
    a, b = _window_means(run, ref, window)
    return float(np.sqrt(np.mean(np.square(a - b)))) if len(a) else float("nan")


def face_error(run: dict, ref: dict, window: float = 0.02) -> float:
    """RMS difference (Pa) of the mean pressure over the face's probes, in
    window means, against the reference run."""
    if min(len(run["t"]), len(ref["t"])) == 0:
        return float("nan")
    a, b = _window_means(run, ref, window)
    return float(np.sqrt(np.mean(np.square(a.mean(axis=1) - b.mean(axis=1))))) if len(a) else float("nan")


def errors(run: dict, ref: dict) -> dict:
    """Every error measure of a run against the reference run."""
    return {"probe_rmse_pa": probe_error(run, ref), "probe_rmse_pa_20ms_means": probe_error(run, ref, 0.02),
            "face_rmse_pa_20ms_means": face_error(run, ref, 0.02), "front_rmse_m": front_error(run, ref)}


def judge_study(height: float, dps, t_end: float = 0.3, dt_probe: float = 0.005, device: int = 0,
                mesh_h: float | None = None, log=None) -> dict:
    """Plain runs of one column height at the spacings `dps`, each judged
    against the finest: a measure judges the closure only if its error
    falls as the spacing does."""
    dps = sorted(dps, reverse=True)
    mesh_h = mesh_h if mesh_h is not None else _load(spec(dps[0], height, "JS0")).params.h
    runs = {}
    for k, dp in enumerate(dps):
        runs[dp] = run_with_probes(_load(spec(dp, height, f"JS{k}")), t_end, dt_probe, device=device, mesh_h=mesh_h)
        if log:
            log(f"dp {dp}: {runs[dp]['np']} particles, {runs[dp]['steps']} steps, {runs[dp]['wall_s']:.1f} s")
    ref = runs[dps[-1]]
    out = {}
    for dp in dps[:-1]:
        e = errors(runs[dp], ref)
        e.update(particles=int(runs[dp]["np"]), steps=int(runs[dp]["steps"]), wall_s=runs[dp]["wall_s"],
                 ms_per_step=runs[dp]["ms_per_step"])
        out[dp] = e
    out[dps[-1]] = {"particles": int(ref["np"]), "steps": int(ref["steps"]), "wall_s": ref["wall_s"],
                    "ms_per_step": ref["ms_per_step"]}
    return out
