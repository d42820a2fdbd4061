"""The oracle (CPU restatement) against golden fixtures produced by the
reference solver itself (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

import goldens as G
import pyoracle as po

CTE_KEYS = {"kernelh": "kernelh", "kernelsize": "kernelsize", "kernelsize2": "kernelsize2", "cs0": "cs0",
            "eta2": "eta2", "ddtkh": "ddtkh", "ddtgz": "ddtgz", "awen": "awen", "bwenh": "bwenh",
            "cteb": "cteb", "gamma": "gamma", "rhopzero": "rhopzero", "massfluid": "massfluid",
            "massbound": "massbound", "dtini": "dtini", "dtmin": "dtmin", "cflnumber": "cflnumber",
            "movlimit": "movlimit", "scell": "scell"}


def _sim(name):
    cd = G.load_generated(name)
    ct = po.config(po.params_from(cd.params))
    return cd, ct, po.Sim(ct, cd.pos, cd.velrho, cd.idp, cd.code, cd.npb, cd.boundnor)


@pytest.mark.parametrize("name", G.CASE_NAMES)
def test_constants_match_reference(name):
    g = G.golden(name)
    cd = G.load_generated(name)
    ct = po.config(po.params_from(cd.params))
    m = g["meta"]["s0"]
    for k, mk in CTE_KEYS.items():
        v = getattr(ct, k)
        ref = float(m[mk])
        if isinstance(v, float) and k not in ("cs0", "dtini", "dtmin", "cflnumber"):
            assert np.float32(v) == np.float32(ref), (k, v, ref)
        else:
            assert v == pytest.approx(ref, rel=1e-15, abs=0), (k, v, ref)
    assert ct.domcellcode == int(m["domcellcode"])
    assert list(ct.mapcells) == [int(x) for x in m["mapcells"].split(",")]
    assert list(ct.maprealposmin) == pytest.approx([float(x) for x in m["maprealposmin"].split(",")], rel=1e-15)


@pytest.mark.parametrize("name", G.CASE_NAMES)
def test_first_divide_bit_exact(name):
    g = G.golden(name)
    _, _, sim = _sim(name)
    st = sim.state()
    for k in ("idp", "code", "dcell", "pos", "velrho"):
        np.testing.assert_array_equal(st[k], g[f"s0_{k}"], err_msg=k)
    np.testing.assert_array_equal(sim.begincell(), g["s0_begincell"])
    m = g["meta"]["s0"]
    assert sim.np == int(m["np"]) and sim.npb == int(m["npb"]) and sim.npbok == int(m["npbok"])


@pytest.mark.parametrize("name", G.CASE_NAMES)
def test_forces_within_fp32_tolerance(name):
    """ace/ar of the oracle and of the reference, both against the FP64 oracle."""
    g = G.golden(name)
    _, _, sim = _sim(name)
    r64 = po.mdbc_f64(sim)
    sim.mdbc(False)
    rho_b = sim.state()["velrho"][:, 3]
    np.testing.assert_allclose(rho_b, g["s0mdbc_rho"], rtol=2e-6)
    # the reference's own mDBC densities meet the FP64 criterion of the GPU tests
    nb = sim.npbok
    G.assert_mdbc_parity(g["s0mdbc_rho"][:nb], rho_b[:nb], r64, "reference mDBC density")
    f64 = po.forces_f64(sim)
    sim.interaction()
    a32, r32 = sim.forces()
    npb = sim.npb
    for x32, ref, x64, s in ((a32[npb:], g["s0pred_ace"][npb:], f64["ace"][npb:], f64["absace"][npb:]),
                             (r32, g["s0pred_ar"], f64["ar"], f64["absar"])):
        # the oracle's FP32 evaluation and the reference's land at the same level
        G.assert_fp32_parity(x32, ref, x64, s, "oracle vs reference error level")
    if name in G.SHIFT_CASES:
        G.assert_shift_sums(sim.shiftpos()[npb:], g["s0pred_shiftpos"][npb:], f64["shiftpos"][npb:],
                            f64["absshift"][npb:], "oracle vs reference shifting")


@pytest.mark.parametrize("name", [n for n in G.CASE_NAMES if not G.is_verlet(n)])
def test_symplectic_step_bit_exact_given_reference_forces(name):
    """Integrator + divide: fed the reference's own ace/ar, the oracle reproduces
    the reference state bit for bit."""
    g = G.golden(name)
    _, _, sim = _sim(name)
    sim.mdbc(False)
    st = sim.state()
    vr = st["velrho"].copy()
    vr[:, 3] = g["s0mdbc_rho"]  # the reference's own mDBC densities
    sim.set_state(None, vr)
    sim.interaction()
    sim.set_forces(g["s0pred_ace"], g["s0pred_ar"])
    if "s0predsh_shiftpos" in g:  # the reference's shifting displacements
        sim.set_shiftpos(g["s0predsh_shiftpos"])
    dt = float(g["meta"]["s0pred"]["dt"])
    sim.symplectic_pre(dt)
    st = sim.state()
    nr = G.normal_rows(g["s0pre_code"])
    for k in ("idp", "code", "dcell", "pos", "velrho"):
        sel = nr if k in ("pos", "dcell") else slice(None)
        np.testing.assert_array_equal(st[k][sel], g[f"s0pre_{k}"][sel], err_msg=k)
    sim.divide()
    st = sim.state()
    for k in ("idp", "code", "dcell"):
        np.testing.assert_array_equal(st[k], g[f"s0div_{k}"], err_msg=k)
    np.testing.assert_array_equal(sim.begincell(), g["s0div_begincell"])
    sim.interaction()
    sim.set_forces(g["s0cor_ace"], g["s0cor_ar"])
    if "s0corsh_shiftpos" in g:
        sim.set_shiftpos(g["s0corsh_shiftpos"])
    sim.symplectic_cor(dt)
    st = sim.state()
    nr = G.normal_rows(g["s0corr_code"])
    for k in ("idp", "code", "dcell", "pos", "velrho"):
        sel = nr if k in ("pos", "dcell") else slice(None)
        np.testing.assert_array_equal(st[k][sel], g[f"s0corr_{k}"][sel], err_msg=k)


@pytest.mark.parametrize("name", [n for n in G.CASE_NAMES if G.is_verlet(n)])
def test_verlet_step_bit_exact_given_reference_forces(name):
    g = G.golden(name)
    _, _, sim = _sim(name)
    sim.interaction()
    sim.set_forces(g["s0pred_ace"], g["s0pred_ar"])
    if "s0predsh_shiftpos" in g:
        sim.set_shiftpos(g["s0predsh_shiftpos"])
    sim.verlet(float(g["meta"]["s0pred"]["dt"]))
    st = sim.state()
    nr = G.normal_rows(g["s0pre_code"])
    for k in ("idp", "code", "dcell", "pos", "velrho"):
        sel = nr if k in ("pos", "dcell") else slice(None)
        np.testing.assert_array_equal(st[k][sel], g[f"s0pre_{k}"][sel], err_msg=k)
    sim.divide()
    np.testing.assert_array_equal(sim.state()["idp"], g["s1_idp"])
    np.testing.assert_array_equal(sim.begincell(), g["s1_begincell"])


@pytest.mark.parametrize("name", G.SHIFT_CASES)
def test_run_shifting_bit_exact_given_reference_sums(name):
    """JSphShifting::RunCpu: fed the reference's shifting sums, the oracle's
    displacements equal the reference's bit for bit (double arithmetic)."""
    g = G.golden(name)
    _, _, sim = _sim(name)
    sim.interaction()
    dt = float(g["meta"]["s0pred"]["dt"])
    sim.set_shiftpos(g["s0pred_shiftpos"])
    sim.run_shifting(dt if G.is_verlet(name) else dt * 0.5)
    npb = sim.npb
    np.testing.assert_array_equal(sim.shiftpos()[npb:], g["s0predsh_shiftpos"][npb:])
    assert np.abs(g["s0predsh_shiftpos"][npb:, :3]).max() > 0   # some particles shift


@pytest.mark.parametrize("name", G.CASE_NAMES)
def test_dt_matches_reference(name):
    g = G.golden(name)
    _, _, sim = _sim(name)
    sim.mdbc(False)
    sim.interaction()
    dtp = sim.dtvariable()
    assert dtp == pytest.approx(float(g["meta"]["s0pred"]["dt_p"]), rel=1e-5)


@pytest.mark.parametrize("name", G.CASE_NAMES)
def test_multistep_run_against_reference(name):
    """Whole steps: per-step dt within 1e-5, particle count conserved (no
    exclusions), final state close to the reference's (trajectories diverge
    only through FP32 rounding over this short horizon)."""
    g = G.golden(name)
    _, _, sim = _sim(name)
    n = len(g["dtlist"])
    dts = [sim.step() for _ in range(n)]
    np.testing.assert_allclose(dts, g["dtlist"], rtol=1e-5)
    st = sim.state()
    assert sim.np == int(g["meta"]["end"]["np"])
    o1 = np.argsort(st["idp"])
    o2 = np.argsort(g["end_idp"])
    np.testing.assert_array_equal(st["idp"][o1], g["end_idp"][o2])
    np.testing.assert_allclose(st["pos"][o1], g["end_pos"][o2], atol=1e-6)
    np.testing.assert_allclose(st["velrho"][o1, :3], g["end_velrho"][o2, :3], atol=2e-3)
    np.testing.assert_allclose(st["velrho"][o1, 3], g["end_velrho"][o2, 3], rtol=1e-4)
