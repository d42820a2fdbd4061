"""Moving boundaries: the predefined motion (JDsMotion / JMotion) and its
application to the moving particles (RunMotion: MoveLinBound / MoveMatBound).

* CPU: the host motion (gbsph_motion_*, libgbsph.so, no device) fed the
  reference's own (time, dt) sequence gives the motion data the reference's
  JDsMotion gave in the same run (tests/golden/mov_d04.npz: motion): a chain of
  sinusoidal translation, sinusoidal pitch, uniform translation and uniform
  acceleration whose durations end inside steps.  The reference is compiled
  with -ffast-math, so its double arithmetic is not reproducible bit for bit:
  displacements and velocities agree to MOTION_RTOL of their size, matrices to
  MATRIX_ATOL (a few ulps).  Semantics of events, chaining and rotations on
  hand-made motions; the loader reads moving blocks and the motion XML.
* GPU: the sloshing-tank case stepped with its motion matches the
  reference's run, with Symplectic and with Verlet (tests/golden/movv_d04.npz):
  dt of every step, the moving particles' positions (the motion is
  independent of the flow, up to the dt it is given) and velocities, and the
  whole state within the multi-step tolerance.
"""
import ctypes as C

import numpy as np
import pytest

import goldens as G
from dualsphysics_gb300 import _lib
from dualsphysics_gb300.case import motion_structs

MOTION_RTOL = 1e-13
MATRIX_ATOL = 1e-15


def _motion(motion: dict, simulate2d: int = 0):
    objs, movs, nmov, evts, nevt = motion_structs(motion)
    m = C.c_void_p()
    rc = _lib.lib().gbsph_motion_create(len(motion["objects"]), objs, nmov, movs, nevt, evts, simulate2d,
                                        C.byref(m))
    assert rc == 0
    return m


def _process(m, nobj, t, dt):
    out = (_lib.MotionData * nobj)()
    rc = _lib.lib().gbsph_motion_process(m, t, dt, out)
    return rc, out


@pytest.mark.parametrize("name", ["mov_d04", "movv_d04"])
def test_host_motion_matches_reference_dump(name):
    cd = G.load_generated(name)
    g = G.golden(name)["motion"]
    assert len(g) == G.case_nsteps(name) + 1
    m = _motion(cd.motion)
    kinds = set()
    for r in g:
        rc, out = _process(m, 1, r[0], r[1])
        d = out[0]
        assert rc == 1 and d.type == int(r[3]), r[:4]
        kinds.add(d.type)
        if d.type == 1:
            mov, vel = np.array(d.linmov), np.array(d.linvel)
            np.testing.assert_allclose(mov, r[4:7], rtol=0, atol=MOTION_RTOL * np.abs(r[4:7]).max())
            np.testing.assert_allclose(vel, r[7:10], rtol=0, atol=MOTION_RTOL * np.abs(r[7:10]).max())
        else:
            np.testing.assert_allclose(np.array(d.mat), r[10:26], rtol=0, atol=MATRIX_ATOL)
    assert kinds == {1, 2}
    _lib.lib().gbsph_motion_destroy(m)


def _mv(**kw):
    base = {"obj": 0, "next": 0, "angdegrees": True}
    base.update(kw)
    return base


def test_host_motion_chaining_and_events():
    # wait 0.1 s, then 1 m/s along x for 0.2 s, then stop; the event starts at 0.05 s
    mot = {"objects": [(0, 10)],
           "movements": [_mv(type="wait", id=1, next=2, duration=0.1),
                         _mv(type="mvrect", id=2, duration=0.2, vel=(1.0, 0.0, 0.0))],
           "events": [(0, 1, 0.05, -1.0)]}
    m = _motion(mot)
    rc, out = _process(m, 1, 0.0, 0.04)          # before the event: nothing active
    assert rc == 0 and out[0].type == 0
    rc, out = _process(m, 1, 0.04, 0.1)          # waiting 0.05..0.15: active, not moving
    assert rc == 1 and out[0].type == 0
    rc, out = _process(m, 1, 0.14, 0.02)         # 0.01 s of the wait, then 0.01 s of motion
    assert out[0].type == 1 and abs(out[0].linmov[0] - 0.01) < 1e-15
    assert abs(out[0].linvel[0] - 0.01 / 0.02) < 1e-12
    rc, out = _process(m, 1, 0.16, 0.5)          # ends at 0.35: 0.19 s of motion left
    assert abs(out[0].linmov[0] - 0.19) < 1e-12
    rc, out = _process(m, 1, 0.66, 0.1)          # finished: stopped
    assert out[0].type == 0
    assert _lib.lib().gbsph_motion_process(m, 0.5, 0.1, out) < 0   # time may not go back
    _lib.lib().gbsph_motion_destroy(m)


def test_host_motion_rotation_and_2d():
    # a uniform rotation is a rigid motion about its axis; in 2-D the linear
    # y movement is dropped (JDsMotion::ProcesTime)
    mot = {"objects": [(0, 5), (5, 5)],
           "movements": [_mv(type="mvrot", id=1, duration=1.0, axisp1=(0.5, 0.0, 0.5), axisp2=(0.5, 1.0, 0.5),
                             vel=90.0),
                         _mv(obj=1, type="mvrect", id=1, duration=1.0, vel=(0.1, 0.2, 0.3))],
           "events": [(0, 1, 0.0, -1.0), (1, 1, 0.0, -1.0)]}
    m = _motion(mot, simulate2d=1)
    rc, out = _process(m, 2, 0.0, 0.5)
    assert out[0].type == 2 and out[1].type == 1
    a = np.array(out[0].mat).reshape(4, 4)
    p = np.array([1.5, 0.3, 0.5, 1.0])
    q = a @ p
    r45 = np.sqrt(0.5)  # 90 deg/s for 0.5 s: 45 degrees about the axis, radius 1 kept
    np.testing.assert_allclose(q[:3], [0.5 + r45, 0.3, 0.5 + r45 * np.sign(q[2] - 0.5)], atol=1e-12)
    np.testing.assert_allclose(a[:3, :3] @ a[:3, :3].T, np.eye(3), atol=1e-14)
    assert out[1].linmov[1] == 0 and out[1].linvel[1] == 0 and abs(out[1].linmov[0] - 0.05) < 1e-15
    _lib.lib().gbsph_motion_destroy(m)


def test_host_motion_rejects_invalid():
    bad = [{"objects": [(0, 5)], "movements": [_mv(type="mvrect", id=1, next=9, duration=1.0, vel=(1, 0, 0))],
            "events": []},
           {"objects": [(0, 5)], "movements": [_mv(type="mvrot", id=1, duration=1.0, axisp1=(0, 0, 0),
                                                    axisp2=(0, 0, 0), vel=1.0)], "events": []},
           {"objects": [(0, 5)], "movements": [_mv(type="mvrect", id=1, duration=1.0, vel=(1, 0, 0))],
            "events": [(0, 2, 0.0, -1.0)]}]
    for mot in bad:
        objs, movs, nmov, evts, nevt = motion_structs(mot)
        m = C.c_void_p()
        assert _lib.lib().gbsph_motion_create(1, objs, nmov, movs, nevt, evts, 0, C.byref(m)) == -1


def test_loader_reads_moving_blocks_and_motion():
    cd = G.load_generated("mov_d04")
    nb = cd.npb
    assert (cd.code[:nb] == 0x0800).all() and (cd.code[nb:] == 0x1800).all()
    assert cd.motion["objects"] == [(0, nb)]
    types = [m["type"] for m in cd.motion["movements"]]
    assert types == ["mvrectsinu", "mvrotsinu", "mvrect", "mvrectace"]
    assert cd.motion["movements"][0]["duration"] == float(np.float32(0.004))   # a float in the reference
    assert cd.motion["events"] == [(0, 1, 0.0, -1.0)]


# ---- GPU ------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mov_d04", "movv_d04"])
def test_moving_tank_matches_reference_run(name):
    """Symplectic (mov_d04) and Verlet (movv_d04, the motion advanced inside
    the step with the dt the step computes)."""
    from dualsphysics_gb300.sph import GbSphSingle
    g = G.golden(name)
    cd = G.load_generated(name)
    s = GbSphSingle(0)
    s.setup(cd)
    n = len(g["dtlist"])
    dts = []
    for _ in range(n):
        s.ComputeStep()
        dts.append(s.step_dt()[0])
    np.testing.assert_allclose(dts, g["dtlist"], rtol=1e-5)
    st = s.download()
    s.close()
    assert len(st["idp"]) == len(g["end_idp"])            # no particle left the domain
    o1, o2 = np.argsort(st["idp"]), np.argsort(g["end_idp"])
    pos, rpos = st["pos"][o1], g["end_pos"][o2]
    vr, rvr = st["velrho"][o1], g["end_velrho"][o2]
    nb = cd.npb
    # the moving walls: a rigid motion that depends on the flow only through dt
    disp = np.abs(rpos[:nb] - cd.pos[:nb]).max()
    assert disp > 1e-3                                    # the tank did move
    np.testing.assert_allclose(pos[:nb], rpos[:nb], rtol=0, atol=1e-5 * disp)
    np.testing.assert_allclose(vr[:nb, :3], rvr[:nb, :3], rtol=0, atol=1e-4 * np.abs(rvr[:nb, :3]).max())
    # the fluid, within the multi-step tolerance
    np.testing.assert_allclose(pos[nb:], rpos[nb:], atol=1e-6)
    np.testing.assert_allclose(vr[nb:, :3], rvr[nb:, :3], atol=2e-3)
    np.testing.assert_allclose(vr[:, 3], rvr[:, 3], rtol=1e-4)


@pytest.mark.gpu
def test_moving_tank_graph_replay_equals_eager():
    from dualsphysics_gb300.sph import GbSphSingle
    cd = G.load_generated("mov_d04")
    a, b = GbSphSingle(0), GbSphSingle(0)
    a.setup(cd)
    b.setup(cd)
    for _ in range(8):
        a.ComputeStep()
    b.RunSteps(8, use_graph=True)
    sa, sb = a.download(), b.download()
    for k in ("idp", "code", "dcell", "pos", "velrho"):
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    a.close()
    b.close()
