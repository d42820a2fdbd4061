"""Measurement gauges (velocity, SWL, max-z) of the reference's gauge system
(JDsGaugeItem.cpp:427-478, 614-641, 728-790, 1023-1087).

* CPU: the numpy restatement (oracle/gauges.py) reproduces the gauges the
  reference's own gauge classes computed on the final state of two golden
  runs (tests/golden/{dbc,mdbc}_d04.npz: gauge_kind, gauge_par, gauge_out);
  the Python gauge system's bookkeeping and CSV output.
* GPU: gbsph_gauge_* on the same final state, uploaded and divided on the
  device, against the reference's results and against the restatement at
  seeded random points.

Tolerances: the per-particle float arithmetic is the reference's, only the
order of the double sums differs, so velocities agree to 2 float ulps (rtol
3e-7); the max-z gauge involves no sum and is exact; an SWL surface point moves
by the step vector times the interpolation fraction, so it is compared with an
absolute 1e-6 m (1e-4 of the particle spacing of these cases).
"""
import numpy as np
import pytest

import goldens as G
import gauges as OG
from dualsphysics_gb300 import _lib
from dualsphysics_gb300.gauges import GaugeSystem

GAUGE_CASES = ["dbc_d04", "mdbc_d04"]
VEL_RTOL, VEL_ATOL = 3e-7, 1e-10
SWL_ATOL = 1e-6


def _state(name):
    g = G.golden(name)
    cd = G.load_generated(name)
    return g, cd, _lib.config(cd.params)


def _oracle_gauge(kind, p, g, cd, pc):
    pos, vr, code = g["end_pos"], g["end_velrho"], g["end_code"]
    mn, mx = cd.params.maprealposmin, cd.params.maprealposmax
    if kind == 0:
        return np.asarray(OG.gauge_velocity(p[:3], pos, vr, code, pc, mn, mx), np.float64)
    if kind == 1:
        return np.asarray(OG.gauge_swl(p[:3], p[3:6], p[6], p[7], pos, vr, code, pc), np.float64)
    return np.array([OG.gauge_maxz(p[:3], p[3], p[4], pos, code, mn[2]), 0.0, 0.0])


def _check(kind, got, ref, what):
    if kind == 0:
        np.testing.assert_allclose(got, ref, rtol=VEL_RTOL, atol=VEL_ATOL, err_msg=what)
    elif kind == 1:
        np.testing.assert_allclose(got, ref, rtol=0, atol=SWL_ATOL, err_msg=what)
    else:
        assert np.float32(got[0]) == np.float32(ref[0]), what


@pytest.mark.parametrize("name", GAUGE_CASES)
def test_oracle_gauges_match_reference(name):
    g, cd, pc = _state(name)
    assert len(g["gauge_kind"]) == 11 and set(g["gauge_kind"].tolist()) == {0, 1, 2}
    for i, (k, p, o) in enumerate(zip(g["gauge_kind"], g["gauge_par"], g["gauge_out"])):
        _check(int(k), _oracle_gauge(int(k), p, g, cd, pc), o, f"{name} gauge {i}")
    # the cases the fixtures hold: outside the map -> zero velocity; no fluid
    # along a SWL line -> point0; no fluid near a max-z line -> the map's lower z
    out = g["gauge_out"]
    assert not out[4].any() and not out[3].any()
    np.testing.assert_array_equal(out[7].astype(np.float32), g["gauge_par"][7][:3].astype(np.float32))
    assert np.float32(out[10][0]) == np.float32(cd.params.maprealposmin[2])


def test_oracle_swl_points_follow_setpoints():
    # PointNp = floor(dis/dp), +1 if the remainder is >= dp/10, at least 1
    n, d = OG.swl_points((0, 0, 0), (0, 0, 1.0), 0.33)   # remainder 0.01 < 0.033
    assert n == 3 and np.allclose(d, [0, 0, 1.0 / 3])
    n, d = OG.swl_points((0, 0, 0), (0, 0, 1.0), 0.3)    # remainder 0.1 >= 0.03
    assert n == 4 and np.allclose(d, [0, 0, 0.25])
    n, d = OG.swl_points((0, 0, 1.0), (0, 0, 0), 2.0)    # shorter than one step
    assert n == 1 and np.allclose(d, [0, 0, -1.0])
    n, d = OG.swl_points((0, 0, 0), (0, 0, 0), 0.1)
    assert n == 0 and not d.any()


class _FakeSph:
    ctx = None


def test_gauge_system_bookkeeping_and_csv(tmp_path):
    gs = GaugeSystem(_FakeSph())
    gs.AddGaugeVel("v1", (0.1, 0.2, 0.3))
    gs.AddGaugeSwl("s1", (0.1, 0.2, 0.0), (0.1, 0.2, 0.5), 0.01)
    gs.AddGaugeMaxZ("m1", (0.1, 0.2, 0.0), 0.5, 0.05)
    with pytest.raises(ValueError, match="already exists"):
        gs.AddGaugeVel("v1", (0, 0, 0))
    with pytest.raises(RuntimeError):
        gs.GetResult("s1")
    gs.GetGauge("v1").results.append((0.5, np.float32([1.5, 0, -2])))
    gs.GetGauge("s1").results.append((0.5, np.float32([0.1, 0.2, 0.25])))
    gs.GetGauge(2).results.append((0.5, np.float32(0.3)))
    assert gs.GetResult(2) == np.float32(0.3)
    files = gs.SaveResults(str(tmp_path))
    assert [f.split("/")[-1] for f in files] == ["GaugesVel_v1.csv", "GaugesSWL_s1.csv", "GaugesMaxZ_m1.csv"]
    lines = open(files[0]).read().splitlines()
    assert lines[0].startswith("time [s];velx [m/s]") and lines[1] == "0.5;1.5;0;-2;0.1;0.2;0.3"
    assert open(files[2]).read().splitlines()[1] == "0.5;0.3;0.1;0.2;0"


# ---- GPU ------------------------------------------------------------------
def _gpu_on_end_state(g, cd):
    from dualsphysics_gb300.sph import GbSphSingle
    from dataclasses import replace
    end = replace(cd, pos=np.ascontiguousarray(g["end_pos"]), velrho=np.ascontiguousarray(g["end_velrho"]),
                  idp=np.ascontiguousarray(g["end_idp"]), code=np.ascontiguousarray(g["end_code"]), boundnor=None)
    s = GbSphSingle(0)
    s.setup(end)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("name", GAUGE_CASES)
def test_gpu_gauges_match_reference(name):
    g, cd, pc = _state(name)
    s = _gpu_on_end_state(g, cd)
    gs = GaugeSystem(s)
    for i, (k, p) in enumerate(zip(g["gauge_kind"], g["gauge_par"])):
        if k == 0:
            gs.AddGaugeVel(f"g{i}", p[:3])
        elif k == 1:
            gs.AddGaugeSwl(f"g{i}", p[:3], p[3:6], p[6], p[7])
        else:
            gs.AddGaugeMaxZ(f"g{i}", p[:3], p[3], p[4])
    n0 = s.launch_count()
    gs.CalculeGpu(0.0)
    assert s.launch_count() - n0 == 3  # one launch per gauge type
    for i, (k, o) in enumerate(zip(g["gauge_kind"], g["gauge_out"])):
        r = np.atleast_1d(np.asarray(gs.GetResult(i), np.float64))
        _check(int(k), np.concatenate([r, np.zeros(3 - len(r))]), o, f"{name} gauge {i}")
    s.close()


@pytest.mark.gpu
def test_gpu_gauges_random_points_match_restatement():
    name = "dbc_d04"
    g, cd, pc = _state(name)
    s = _gpu_on_end_state(g, cd)
    rng = np.random.default_rng(7)
    lo = np.array(cd.params.maprealposmin)
    hi = np.array(cd.params.maprealposmax)
    # velocity: points inside, a few outside the map and on its faces
    pts = lo + (hi - lo) * rng.random((96, 3))
    pts[0] = lo
    pts[1] = hi
    pts[2] = lo - 0.01
    pts = np.ascontiguousarray(pts)
    vel = np.empty((len(pts), 3), np.float32)
    assert _lib.lib().gbsph_gauge_velocity(s.ctx, len(pts), _lib.ptr(pts), _lib.ptr(vel)) == 0
    for i, p in enumerate(pts):
        ref = _oracle_gauge(0, np.concatenate([p, np.zeros(5)]), g, cd, pc)
        _check(0, vel[i].astype(np.float64), ref, f"vel point {i}")
    assert not vel[1].any() and not vel[2].any()
    # SWL and max-z: vertical lines at random x, y (some downward, some tilted)
    m = 24
    xy = lo[:2] + (hi[:2] - lo[:2]) * rng.random((m, 2))
    p0p2 = np.zeros((m, 6))
    p0p2[:, :2] = xy
    p0p2[:, 2] = lo[2] + 0.02
    p0p2[:, 3:5] = xy
    p0p2[:, 5] = hi[2] - 0.02
    p0p2[::5, 3] += 0.05  # tilted
    p0p2 = np.ascontiguousarray(p0p2)
    pdp = np.full(m, cd.params.dp * 0.5)
    pdp[3] = 0.0  # no points: the result is point0
    ml = np.zeros(m, np.float32)
    ml[1] = pc.massfluid * 0.8
    surf = np.empty((m, 3), np.float32)
    assert _lib.lib().gbsph_gauge_swl(s.ctx, m, _lib.ptr(p0p2), _lib.ptr(pdp), _lib.ptr(ml), _lib.ptr(surf)) == 0
    for i in range(m):
        par = np.concatenate([p0p2[i], [pdp[i], ml[i]]])
        _check(1, surf[i].astype(np.float64), _oracle_gauge(1, par, g, cd, pc), f"swl line {i}")
    p0h = np.ascontiguousarray(np.column_stack([xy, np.full(m, lo[2]), np.full(m, hi[2] - lo[2])]))
    dl = np.full(m, 2.0 * pc.kernelh, np.float32)
    dl[0] = 0.5 * float(cd.params.dp)
    zmax = np.empty(m, np.float32)
    assert _lib.lib().gbsph_gauge_maxz(s.ctx, m, _lib.ptr(p0h), _lib.ptr(dl), _lib.ptr(zmax)) == 0
    for i in range(m):
        par = np.concatenate([p0h[i], [dl[i], 0, 0, 0]])
        _check(2, np.array([zmax[i], 0, 0], np.float64), _oracle_gauge(2, par, g, cd, pc), f"maxz line {i}")
    s.close()


@pytest.mark.gpu
def test_gpu_gauges_reject_bad_calls():
    g, cd, pc = _state("dbc_d04")
    s = _gpu_on_end_state(g, cd)
    L = _lib.lib()
    out = np.empty(3, np.float32)
    assert L.gbsph_gauge_velocity(s.ctx, 1, None, _lib.ptr(out)) == -1  # GBSPH_EINVAL
    assert L.gbsph_gauge_velocity(s.ctx, 0, None, None) == 0
    p = np.array([0.0, 0, 0, 0, 0, 1e9])
    dp = np.array([1e-9])
    ml = np.zeros(1, np.float32)
    assert L.gbsph_gauge_swl(s.ctx, 1, _lib.ptr(p), _lib.ptr(dp), _lib.ptr(ml), _lib.ptr(out)) == -1  # GBSPH_EINVAL
    assert b"too many points" in L.gbsph_last_error(s.ctx)
    s.close()
