"""The learned closure (no reference counterpart): its MLP kernels against the
FP64 oracle (oracle/closure_oracle.py), its features against a brute-force
restatement, its use inside the step, and what a trained network gains.

* CPU: the oracle's gradient against central finite differences; BF16
  rounding against torch's; the parameter count against the header; the
  fine/coarse lattices nest.
* GPU: forward (BF16 weights, FP32 accumulation) and gradient against the
  oracle evaluated with the same BF16 weights; Adam training of a smooth
  target; the features of a case against the oracle; a zero correction and
  an always-rejected correction leave the run bit-identical to the plain one
  (the second counted as fallbacks); a network trained on paired runs of
  three column heights lowers the acceleration error of a fourth, held-out
  height against its fine run.
"""
import os
import re
import sys

import numpy as np
import pytest

import goldens as G
from dualsphysics_gb300 import closure as cl

sys.path.insert(0, os.path.join(G.ROOT, "oracle"))
import closure_oracle as co  # noqa: E402


def _rand_data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (n, cl.NFEAT)).astype(np.float32)
    x[:, 13:] = 0
    t = np.stack([np.sin(x[:, 0]) * 0.5, x[:, 1] * x[:, 2] * 0.3, np.tanh(x[:, 3] - x[:, 4])], 1).astype(np.float32)
    return x, t


def test_parameter_count_matches_header():
    h = open(os.path.join(G.ROOT, "include", "gbsph.h")).read()
    assert int(re.search(r"#define GBSPH_CLOSURE_PARAMS (\d+)", h).group(1)) == cl.NPARAMS == 9603
    assert int(re.search(r"#define GBSPH_CLOSURE_FEATURES (\d+)", h).group(1)) == cl.NFEAT


def test_oracle_gradient_against_finite_differences():
    x, t = _rand_data(7, 1)
    p = cl.init_params(3, out_scale=1.0).astype(np.float64)
    _, g = co.loss_and_grad(p, x, t)
    rng = np.random.default_rng(2)
    for i in rng.choice(cl.NPARAMS, 40, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (co.loss_and_grad(p + e, x, t)[0] - co.loss_and_grad(p - e, x, t)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i]), i


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    v = np.random.default_rng(0).normal(0, 3, 5000).astype(np.float32)
    v[:4] = [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8]   # ties to even
    ours = cl.to_bf16(v)
    ref = torch.from_numpy(v).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    np.testing.assert_array_equal(ours, ref)


def test_standardisation_folds_into_the_first_and_last_layers():
    rng = np.random.default_rng(3)
    x = rng.normal(2.0, 5.0, (50, cl.NFEAT))
    mu, sd = x.mean(0), x.std(0) + 0.5
    st = np.array([2.0, 0.5, 3.0])
    p = cl.init_params(4, out_scale=1.0)
    y_std = co.forward(p.astype(np.float64), (x - mu) / sd)[-1] * st
    y_raw = co.forward(cl.fold_standardisation(p, mu, sd, st).astype(np.float64), x)[-1]
    np.testing.assert_allclose(y_raw, y_std, rtol=2e-5, atol=2e-5 * np.abs(y_std).max())


@pytest.mark.parametrize("dpf,ratio", [(0.04, 2), (0.02, 4)])
def test_fine_and_coarse_lattices_nest(dpf, ratio):
    pair = cl.Pair(0.25, dp_fine=dpf, tag="N", ratio=ratio)
    c = pair.coarse
    assert len(pair.coarse_row_fine_id) == c.np - c.npb
    f = pair.fine
    fp = f.pos[pair.coarse_row_fine_id]
    np.testing.assert_allclose(fp, c.pos[c.npb:], atol=1e-12)
    # every fine fluid particle in one block of at most ratio^3, whose corner it shares the cell of
    cnt = np.bincount(pair.fine_block, minlength=c.np - c.npb)
    assert cnt.sum() == f.np - f.npb and cnt.min() >= 1 and cnt.max() == ratio ** 3
    st = {"idp": f.idp, "pos": f.pos, "velrho": f.velrho}
    m, n = pair.block_mean(st, f.pos)
    assert np.array_equal(n, cnt)
    # the block mean lies within the block: at most (ratio - 1) / 2 fine spacings from the corner
    assert np.abs(m[:, :] - c.pos[c.npb:]).max() <= 0.5 * (ratio - 1) * dpf + 1e-12


def test_smoothed_targets_keep_constant_and_average_noise():
    """The kernel-weighted neighbourhood mean keeps a constant target field and
    shrinks particle-scale noise."""
    rng = np.random.default_rng(2)
    g = np.stack(np.meshgrid(*[np.arange(20) * 0.02] * 3, indexing="ij"), -1).reshape(-1, 3)
    c = np.full((len(g), 3), 1.5, np.float32)
    np.testing.assert_allclose(cl.smooth_targets(g, c, 0.026), c, rtol=1e-6)
    noise = rng.normal(0.0, 1.0, (len(g), 3)).astype(np.float32)
    sm = cl.smooth_targets(g, noise, 0.026)
    assert sm.std() < 0.5 * noise.std()
    # a field varying over many kernel lengths is kept, away from the edges
    lin = np.repeat(g[:, :1] * 10.0, 3, axis=1).astype(np.float32)
    inner = np.all((g > 0.06) & (g < 0.32), axis=1)
    np.testing.assert_allclose(cl.smooth_targets(g, lin, 0.026)[inner], lin[inner], atol=1e-5)


def test_judge_error_measures():
    """The judge's measures on synthetic probe series: a run equal to the
    reference has no error; a constant offset of the probes is the RMS of the
    offset in every pressure measure; a shifted front is the shift."""
    t = np.arange(1, 61) * 0.005
    p = np.stack([np.sin(40 * t + k) * 1000.0 for k in range(50)], axis=1)
    ref = {"t": t, "p": p, "front": 0.4 + 2.0 * t}
    same = cl.errors(ref, ref)
    assert all(v == 0.0 for v in same.values())
    off = {"t": t, "p": p + 30.0, "front": ref["front"] + 0.01}
    e = cl.errors(off, ref)
    assert abs(e["probe_rmse_pa"] - 30.0) < 1e-9
    assert abs(e["probe_rmse_pa_20ms_means"] - 30.0) < 1e-9
    assert abs(e["face_rmse_pa_20ms_means"] - 30.0) < 1e-9
    assert abs(e["front_rmse_m"] - 0.01) < 1e-12
    # window means remove what averages out within 20 ms
    fast = {"t": t, "p": p + 500.0 * np.where(np.arange(60) % 2 == 0, 1.0, -1.0)[:, None], "front": ref["front"]}
    assert cl.probe_error(fast, ref, 0.02) < 1e-9 < cl.probe_error(fast, ref)


# ---- GPU ------------------------------------------------------------------
@pytest.mark.gpu
def test_mlp_forward_and_gradient_match_oracle():
    x, t = _rand_data(3000, 4)
    p = cl.init_params(5, out_scale=1.0)
    tr = cl.Trainer(p)
    tr.set_data(x, t)
    pb = cl.from_bf16(cl.to_bf16(p)).astype(np.float64)      # the weights the kernels use
    master, w = tr.params()
    np.testing.assert_array_equal(master, p)
    np.testing.assert_array_equal(w, cl.to_bf16(p))
    y = tr.infer(x)
    yo = co.forward(pb, x)[-1]
    assert np.abs(y - yo).max() <= 2e-5 * max(1.0, np.abs(yo).max())
    g, loss = tr.grad()
    lo, go = co.loss_and_grad(pb, x, t)
    assert loss == pytest.approx(lo, rel=1e-5)
    assert np.abs(g - go).max() <= 1e-4 * np.abs(go).max()
    # a sub-range of the data
    g2, _ = tr.grad(100, 500)
    _, go2 = co.loss_and_grad(pb, x[100:600], t[100:600])
    assert np.abs(g2 - go2).max() <= 1e-4 * np.abs(go2).max()
    tr.close()


@pytest.mark.gpu
def test_adam_training_fits_a_smooth_target():
    x, t = _rand_data(20000, 6)
    tr = cl.Trainer(cl.init_params(7))
    tr.set_data(x, t)
    loss = tr.train(epochs=40, batch=512, lr=2e-3)
    assert np.isfinite(loss).all() and loss[-1] < 0.1 * loss[0]
    master, w = tr.params()
    np.testing.assert_array_equal(w, cl.to_bf16(master))       # the BF16 copy follows the master weights
    tr.close()


@pytest.mark.gpu
def test_features_match_oracle():
    from dualsphysics_gb300 import _lib
    from dualsphysics_gb300.sph import GbSphSingle
    cd = G.load_generated("mdbc_d04")
    s = GbSphSingle(0)
    s.setup(cd)
    s.MdbcBoundCorrection(_lib.INTERSTEP_SYMPREDICTOR)
    s.Interaction_Forces(_lib.INTERSTEP_SYMPREDICTOR)
    f = cl.features(s)
    st = s.download()
    ace, _ = s.forces()
    c = s.consts
    s.close()
    # the pressure every kernel uses: the Tait EOS in FP32 (rho/rho0 rounded to float)
    x = (st["velrho"][:, 3] / np.float32(c.rhopzero)).astype(np.float32)
    press = np.float32(c.cteb) * ((x.astype(np.float64) ** c.gamma).astype(np.float32) - np.float32(1.0))
    fo = co.features(st["pos"], st["velrho"], cd.npb, c, press)
    fo[:, 9:12] = ace[cd.npb:] / np.linalg.norm(np.asarray(c.gravity[:], np.float64))
    assert f.shape == fo.shape and np.isfinite(f).all()
    scale = np.maximum(np.abs(fo).max(axis=0), 1e-3)
    err = np.abs(f - fo).max(axis=0) / scale
    assert err.max() < 2e-4, err
    assert np.all(f[:, 13:] == 0)


def _run(cd, n, w=None, limit=0.2):
    from dualsphysics_gb300.sph import GbSphSingle
    s = GbSphSingle(0)
    s.setup(cd)
    if w is not None:
        cl.attach(s, w, limit)
    s.RunSteps(n, use_graph=True)
    st = s.download()
    nfb = cl.fallbacks(s) if w is not None else 0
    dt = s.step_dt()
    s.close()
    return st, nfb, dt


@pytest.mark.gpu
def test_zero_and_rejected_corrections_leave_the_run_unchanged():
    cd = G.load_generated("mdbc_d04")
    base, _, dt0 = _run(cd, 6)
    zero = cl.to_bf16(np.zeros(cl.NPARAMS, np.float32))
    st, nfb, dt = _run(cd, 6, zero)
    for k in ("idp", "pos", "velrho"):
        np.testing.assert_array_equal(st[k], base[k], err_msg=k)
    assert nfb == 0 and dt == dt0
    big = np.zeros(cl.NPARAMS, np.float32)
    big[-3:] = 1000.0                                          # output bias: 1000 g, always above 0.2 |ace|
    st, nfb, dt = _run(cd, 6, cl.to_bf16(big))
    for k in ("idp", "pos", "velrho"):
        np.testing.assert_array_equal(st[k], base[k], err_msg=k)
    assert nfb == 6 * 2 * (cd.np - cd.npb) and dt == dt0    # every fluid row, two passes per step


@pytest.mark.gpu
def test_trained_closure_lowers_the_held_out_acceleration_error():
    """Paired data of three column heights (fine dp 0.02, coarse 0.04);
    trained on them, the network lowers the coarse acceleration error of a
    fourth height against its fine run."""
    xs, ts, meta = cl.paired_samples([0.22, 0.28, 0.34], dp_fine=0.02, t_end=0.12, n_snap=4)
    xh, th, _ = cl.paired_samples([0.31], dp_fine=0.02, t_end=0.12, n_snap=4)
    assert meta["snapshots"] == 12 and len(xs) > 5000
    p, w, loss = cl.train_closure(xs, ts, epochs=60, seed=1)
    assert loss[-1] < loss[0]
    tr = cl.Trainer(cl.from_bf16(w))           # the folded BF16 weights the step would use
    yh = tr.infer(xh)
    plain = float(np.mean(th ** 2))                  # the coarse run's error with no correction
    learned = float(np.mean((th - yh) ** 2))
    assert learned < 0.8 * plain, (learned, plain)
    tr.close()
