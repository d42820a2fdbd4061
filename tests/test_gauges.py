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


MESH_RTOL = 2e-6    # of the conditioning scale (float sums; about 16 ulp)
ZSURF_ATOL = 1e-6


def _div(g, pc):
    m = g["meta"]["end"]
    return dict(ncx=m["ncx"], ncy=m["ncy"], ncz=m["ncz"], nsheet=m["nsheet"],
                cellmin=[int(x) for x in m["cellmin"].split(",")], cellfluid=m["cellfluid"],
                scelldiv=pc.cellmode_div, begincell=g["end_begincell"])


def _mesh_oracle(g, pc, k):
    mb = g["mesh_par"][k]
    return OG.gauge_mesh(mb[:21], mb[21], mb[22], mb[23], g["end_pos"], g["end_velrho"], g["end_code"],
                         _div(g, pc), pc)


def _mesh_ref(g, k):
    """The reference's mesh gauge k: (vel, veldir, rhop) per point, zsurf per column."""
    npt = g["mesh_npt"]
    o1 = int(sum(int(np.prod(n)) for n in npt[:k]))
    o2 = int(sum(int(n[0] * n[1]) for n in npt[:k]))
    n, n12 = int(np.prod(npt[k])), int(npt[k][0] * npt[k][1])
    pt = g["mesh_pt"][o1:o1 + n]
    return pt[:, :3], pt[:, 3], pt[:, 4], g["mesh_zs"][o2:o2 + n12]


def _check_mesh(got, ref, s_vel, s_rho, what):
    vel, vdir, rho, zs = got
    rvel, rvdir, rrho, rzs = ref
    assert (np.abs(np.asarray(vel, np.float64) - rvel) <= MESH_RTOL * s_vel + 1e-12).all(), what + " vel"
    assert (np.abs(np.asarray(vdir, np.float64) - rvdir) <= MESH_RTOL * s_vel.sum(axis=1) + 1e-12).all(), what + " vdir"
    assert (np.abs(np.asarray(rho, np.float64) - rrho) <= MESH_RTOL * s_rho + 1e-12).all(), what + " rhop"
    np.testing.assert_allclose(zs, rzs, rtol=0, atol=ZSURF_ATOL, err_msg=what + " zsurf")


@pytest.mark.parametrize("name", GAUGE_CASES)
def test_oracle_mesh_gauges_match_reference(name):
    g, cd, pc = _state(name)
    assert len(g["mesh_par"]) == 2
    for k in range(2):
        vel, vdir, rho, mass, zs, s_vel, s_rho = _mesh_oracle(g, pc, k)
        _check_mesh((vel, vdir, rho, zs), _mesh_ref(g, k), s_vel, s_rho, f"{name} mesh {k}")
    # the vertical grid crosses the free surface: columns inside the column of
    # water find it near its height, columns past the front stay at ptref.z
    zs = _mesh_ref(g, 0)[3]
    spec = G.case_spec(name)
    assert abs(zs[0] - spec.column[2]) < spec.dp and np.float32(zs[-1]) == np.float32(g["mesh_par"][0][2])


def test_mesh_points_host_entry_matches_reference_grid():
    from dualsphysics_gb300.gauges import GaugeSystem as GS
    g = G.golden("dbc_d04")
    gs = GS(_FakeSph())
    for k, mb in enumerate(g["mesh_par"]):
        gg = gs.AddGaugeMesh(f"m{k}", mb[0:3], mb[3:6], mb[6:9], mb[9:12], mb[12:15], mb[15:18], mb[18:21])
        assert GS.MeshPoints(gg) == tuple(int(x) for x in g["mesh_npt"][k])
        assert list(OG.mesh_points(mb)[2]) == list(g["mesh_npt"][k])
    # an axis with dis < dispt has one point; 2^26 points are the limit
    gg = gs.AddGaugeMesh("one", (0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0.005, 0.0, 1.0), (0.01, 0.01, 0.5))
    assert GS.MeshPoints(gg) == (1, 1, 3)
    gg = gs.AddGaugeMesh("big", (0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1.0, 1.0, 1.0), (1e-3, 1e-3, 1e-2))
    with pytest.raises(ValueError):
        GS.MeshPoints(gg)


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
@pytest.mark.parametrize("name", GAUGE_CASES)
def test_gpu_mesh_gauges_match_reference_and_restatement(name):
    g, cd, pc = _state(name)
    s = _gpu_on_end_state(g, cd)
    gs = GaugeSystem(s)
    for k, mb in enumerate(g["mesh_par"]):
        kcl = None if mb[21] == np.float32(np.finfo(np.float32).max) else mb[21]
        kcd = None if mb[22] == np.float32(np.finfo(np.float32).max) else mb[22]
        gs.AddGaugeMesh(f"m{k}", mb[0:3], mb[3:6], mb[6:9], mb[9:12], mb[12:15], mb[15:18], mb[18:21],
                        kclimit=kcl, kcdummy=kcd, masslimit=mb[23])
    gs.CalculeGpu(0.0)
    for k in range(2):
        r = gs.GetResult(k)
        vel, vdir, rho, mass, zs, s_vel, s_rho = _mesh_oracle(g, pc, k)
        got = (r["vel"], r["veldir"], r["rhop"], r["zsurf"])
        _check_mesh(got, _mesh_ref(g, k), s_vel, s_rho, f"{name} mesh {k} vs reference")
        _check_mesh(got, (vel, vdir, rho, zs), s_vel, s_rho, f"{name} mesh {k} vs restatement")
        np.testing.assert_allclose(r["mass"], mass, rtol=MESH_RTOL, atol=1e-12)
    p = gs.Pressure(gs.GetResult(0)["rhop"])
    assert np.isfinite(p).all() and p.max() > 0
    s.close()


@pytest.mark.gpu
def test_gpu_fluid_front_equals_numpy():
    g, cd, pc = _state("dbc_d04")
    s = _gpu_on_end_state(g, cd)
    pos, fl = g["end_pos"], (g["end_code"] & 0x1800) == 0x1800
    front, n = s.fluid_front()
    assert front == pos[fl, 0].max() and n == int(fl.sum())
    lo, hi = (0.0, 0.0, 0.0), (10.0, 10.0, 2 * cd.params.dp)
    inb = fl & (pos >= lo).all(axis=1) & (pos <= hi).all(axis=1)
    front, n = s.fluid_front((1.0, 0.0, 0.0), lo, hi)
    assert front == pos[inb, 0].max() and n == int(inb.sum())
    d = np.array([0.6, 0.0, -0.8])
    front, n = s.fluid_front(d)
    assert front == ((pos[fl, 0] * d[0] + pos[fl, 1] * d[1]) + pos[fl, 2] * d[2]).max()
    front, n = s.fluid_front((1.0, 0.0, 0.0), (5.0, 5.0, 5.0), (6.0, 6.0, 6.0))
    assert front == -np.inf and n == 0
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
