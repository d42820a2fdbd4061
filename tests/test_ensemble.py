"""Batched ensembles and the autotuner (no reference counterpart: the
reference runs one case per process).

* CPU: the seeded draw of the cases (ranges, determinism), a sloshing case
  loads with its motion.
* GPU: one graph replay steps every case exactly as the case's own step does
  (bit-identical states against each case run alone, with and without the
  graph, moving cases included); the autotuner keeps the fastest candidate and
  the block size of the per-row kernel leaves results bit-identical.
"""
import numpy as np
import pytest

from dualsphysics_gb300.ensemble import ensemble_specs, load_ensemble_case

SMALL = dict(count_range=(3000, 12000))


def test_ensemble_draw_is_seeded_and_in_range():
    a, b = ensemble_specs(64, seed=5), ensemble_specs(64, seed=5)
    assert [x.spec for x in a] == [x.spec for x in b]
    assert ensemble_specs(8, seed=6)[0].spec != a[0].spec
    for ec in a:
        assert all(0.5 <= v <= 2.0 for v in ec.spec.tank)
        fill = np.prod(ec.spec.column) / np.prod(ec.spec.tank)
        assert 0.2 <= fill <= 0.6
        assert 20_000 <= ec.target <= 2_000_000
        if ec.sloshing:
            m = ec.spec.motion[0]
            assert m["type"] == "mvrectsinu" and 0 <= m["ampl"][0] <= 0.05 and 0.5 <= m["freq"][0] <= 2.0
    assert 0 < sum(ec.sloshing for ec in a) < 64


def test_sloshing_case_loads_with_its_motion(tmp_path):
    ec = next(e for e in ensemble_specs(16, seed=3, **SMALL) if e.sloshing)
    cd = load_ensemble_case(ec, str(tmp_path))
    assert cd.motion and cd.motion["movements"][0]["type"] == "mvrectsinu"
    assert cd.motion["objects"] == [(0, cd.npb)]


def _cases(n, seed):
    from dualsphysics_gb300.sph import GbSphSingle
    specs = ensemble_specs(n, seed=seed, **SMALL)
    cds = [load_ensemble_case(ec) for ec in specs]
    return specs, cds


def _sims(cds):
    from dualsphysics_gb300.sph import GbSphSingle
    out = []
    for cd in cds:
        s = GbSphSingle(0)
        s.setup(cd)
        out.append(s)
    return out


def _same(a, b, what):
    sa, sb = a.download(), b.download()
    for k in ("idp", "code", "dcell", "pos", "velrho"):
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=f"{what}: {k}")
    assert a.step_dt() == b.step_dt(), what


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [True, False])
def test_ensemble_steps_equal_each_case_alone(use_graph):
    from dualsphysics_gb300.ensemble import Ensemble
    specs, cds = _cases(6, seed=11)
    assert any(ec.sloshing for ec in specs) and not all(ec.sloshing for ec in specs)
    ens_sims, alone = _sims(cds), _sims(cds)
    e = Ensemble(ens_sims)
    e.run(3, use_graph=use_graph)
    e.run(4, use_graph=use_graph)   # a second call replays the same graph
    e.sync()
    if use_graph:
        assert e.launches_per_step() > 0
    for s in alone:
        s.RunSteps(7, use_graph=True)
    for k, (a, b) in enumerate(zip(ens_sims, alone)):
        _same(a, b, f"case {k}")
    # work issued on a case after the ensemble is ordered after it
    ens_sims[0].RunSteps(1, use_graph=False)
    alone[0].RunSteps(1, use_graph=False)
    _same(ens_sims[0], alone[0], "after the ensemble")
    e.close()
    for s in ens_sims + alone:
        s.close()


@pytest.mark.gpu
def test_autotuner_keeps_the_fastest_candidate():
    from dualsphysics_gb300.ensemble import tune
    _, cds = _cases(2, seed=12)
    (s,) = _sims(cds[:1])
    r = tune(s, reps=2)
    assert len(r["ms"]) == 8 and all(m > 0 for m in r["ms"])
    assert r["ms"][r["best"]] == min(r["ms"])
    assert list(zip(r["variant"], r["bsize"], r["split"])) == [(2, 128, 1), (2, 128, 2), (2, 128, 4), (3, 128, 1),
                                                                (0, 128, 1), (1, 64, 1), (1, 128, 1), (1, 256, 1)]
    assert s.get_option(4) == r["split"][r["best"]]
    assert r["bound_lanes"] == [1, 4, 32] and all(m > 0 for m in r["bound_ms"])
    assert r["bound_ms"][r["bound_best"]] == min(r["bound_ms"])
    assert s.get_option(6) == r["bound_lanes"][r["bound_best"]]
    if r["mdbc_best"] >= 0:
        assert r["mdbc_ms"][r["mdbc_best"]] == min(r["mdbc_ms"])
        assert s.get_option(8) == r["mdbc_split"][r["mdbc_best"]]
    # the tuned context steps as one set to the same configuration by hand
    (t,) = _sims(cds[:1])
    t.set_option(1, r["variant"][r["best"]])
    t.set_option(0, r["bsize"][r["best"]])
    t.set_option(4, r["split"][r["best"]])
    t.set_option(6, r["bound_lanes"][r["bound_best"]])
    if r["mdbc_best"] >= 0:
        t.set_option(8, r["mdbc_split"][r["mdbc_best"]])
    s.RunSteps(5, use_graph=True)
    t.RunSteps(5, use_graph=True)
    _same(s, t, "tuned vs set by hand")
    s.close()
    t.close()


@pytest.mark.gpu
def test_per_row_kernel_block_size_leaves_results_identical():
    _, cds = _cases(1, seed=13)
    sims = _sims(cds * 3)
    for s, bs in zip(sims, (64, 128, 256)):
        s.set_option(1, 1)
        s.set_option(0, bs)
        s.RunSteps(6, use_graph=True)
    _same(sims[0], sims[1], "64 vs 128")
    _same(sims[1], sims[2], "128 vs 256")
    for s in sims:
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["dbc_d04", "mdbc_d04", "peri_d04"])
def test_sort_digit_width_leaves_the_order_unchanged(name):
    """The divide's radix sort with 11-bit digits (fewer passes) gives the
    same stable order as with 8-bit digits: identical runs."""
    import goldens as G
    from dualsphysics_gb300.sph import GbSphSingle
    cd = G.load_generated(name)
    a, b = GbSphSingle(0), GbSphSingle(0)
    a.setup(cd)
    b.setup(cd)
    b.set_option(2, 11)
    b.RunCellDivide()                       # a divide of a divided state: the same order
    a.RunCellDivide()
    _same(a, b, "re-divided")
    a.RunSteps(6, use_graph=True)
    b.RunSteps(6, use_graph=True)
    _same(a, b, name)
    a.close()
    b.close()


@pytest.mark.gpu
def test_ensemble_level_tuner_keeps_the_fastest_policy():
    """tune_mix times whole ensemble replays under each policy and leaves
    every case at the kept policy applied to its own tuned options (the
    ensemble steps each case as the case alone with the same options:
    test_ensemble_steps_equal_each_case_alone)."""
    from dualsphysics_gb300.ensemble import MIX_POLICIES, Ensemble, case_options, tune, tune_mix
    _, cds = _cases(3, seed=5)
    sims = _sims(cds)
    for s in sims:
        tune(s, reps=1)
    ens = Ensemble(sims)
    r = tune_mix(ens, sims, reps=1)
    assert set(r["ms_per_replay"]) == set(MIX_POLICIES) and all(v > 0 for v in r["ms_per_replay"].values())
    assert r["ms_per_replay"][r["kept"]] == min(r["ms_per_replay"].values())
    for s, o in zip(sims, r["alone"]):
        assert case_options(s) == MIX_POLICIES[r["kept"]](o)
    ens.run(2, use_graph=True)
    ens.sync()
    ens.close()
    for s in sims:
        s.close()


@pytest.mark.gpu
def test_autotuner_tunes_the_mdbc_split_on_an_mdbc_case():
    """On an mDBC case the tuner also times the mDBC kernel at 1, 2 and 4 warps
    per row group and keeps the fastest; the tuned run equals the run with
    the same options set by hand."""
    import goldens as G
    from dualsphysics_gb300.ensemble import tune
    cd = G.load_generated("mdbc_d04")
    (s,) = _sims([cd])
    r = tune(s, reps=2)
    assert r["mdbc_split"] == [1, 2, 4] and 0 <= r["mdbc_best"] < 3 and all(m > 0 for m in r["mdbc_ms"])
    assert r["mdbc_ms"][r["mdbc_best"]] == min(r["mdbc_ms"])
    assert s.get_option(8) == s.get_option(9) == r["mdbc_split"][r["mdbc_best"]]
    (t,) = _sims([cd])
    for key, value in ((1, r["variant"][r["best"]]), (0, r["bsize"][r["best"]]), (4, r["split"][r["best"]]),
                       (6, r["bound_lanes"][r["bound_best"]]), (8, r["mdbc_split"][r["mdbc_best"]])):
        t.set_option(key, value)
    s.RunSteps(4, use_graph=True)
    t.RunSteps(4, use_graph=True)
    _same(s, t, "tuned vs set by hand (mDBC)")
    s.close()
    t.close()


@pytest.mark.gpu
def test_sort_tuner_keeps_a_valid_width_and_the_run():
    import ctypes as C
    import goldens as G
    from dualsphysics_gb300._lib import lib
    from dualsphysics_gb300.sph import GbSphSingle
    cd = G.load_generated("dbc_d04")
    a, b = GbSphSingle(0), GbSphSingle(0)
    a.setup(cd)
    b.setup(cd)
    bits = C.c_int()
    ms = np.zeros(2, np.float32)
    assert lib().gbsph_tune_sort(b.ctx, 3, C.byref(bits), ms.ctypes.data_as(C.c_void_p)) == 0
    assert bits.value in (8, 11) and (ms > 0).all() and ms[0 if bits.value == 8 else 1] == ms.min()
    assert lib().gbsph_set_option(b.ctx, 2, 9) != 0           # only 8 or 11
    a.RunSteps(5, use_graph=True)
    b.RunSteps(5, use_graph=True)
    _same(a, b, "tuned sort")
    a.close()
    b.close()
