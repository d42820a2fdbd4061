"""Periodic conditions (JSphCpuSingle::RunPeriodic and the periodic UpdatePos).

The case is a channel periodic in x (tests/golden/peri_d04.npz, from the
reference solver): 40% of the particles lie within the kernel's reach of a
periodic face, so each divide appends 1,320 copies, and the fluid moves at
2 m/s, so columns leave the real domain through x = 0.78 and come back
through x = -0.02 within the 30 fixture steps.

* CPU: the configuration (map extended by the kernel size on the periodic
  axis, the axis increment), the default capacity, the normal-row filter.
* GPU: the first divide with its copies is bit-exact (the generic parity
  tests); here the 30-step run against the reference's end state with the
  wrap-around exercised, graph replay equal to eager stepping, a capacity too
  small for the copies reported as an error, and Part output without copies.
"""
import os

import numpy as np
import pytest

import goldens as G
from dualsphysics_gb300 import _lib, bi4
from dualsphysics_gb300.sph import default_capacity, normal_rows


def test_periodic_configuration_matches_reference():
    g = G.golden("peri_d04")
    cd = G.load_generated("peri_d04")
    assert list(cd.params.peri) == [1, 0, 0]
    c = _lib.config(cd.params)
    m = g["meta"]["s0"]
    size = c.maprealposmax[0] - c.maprealposmin[0]
    assert c.periinc[0] == -size and list(c.periinc)[1:] == [0.0] * 8
    assert c.mapposmin[0] == c.maprealposmin[0] - c.kernelsize
    assert c.mapposmax[0] == c.maprealposmax[0] + c.kernelsize
    assert list(c.domposmin) == [float(x) for x in m["domposmin"].split(",")]
    assert list(c.mapcells) == [int(x) for x in m["mapcells"].split(",")]


def test_default_capacity_and_normal_rows():
    cd = G.load_generated("peri_d04")
    assert default_capacity(cd) == 3 * cd.np
    assert default_capacity(G.load_generated("perixy_d04")) == 7 * G.load_generated("perixy_d04").np
    assert default_capacity(G.load_generated("dbc_d04")) == G.load_generated("dbc_d04").np
    code = np.array([0x1800, 0x3800, 0x0000, 0x2000, 0x5800], np.uint16)
    assert normal_rows(code).tolist() == [True, False, True, False, False]


def test_reference_run_wraps_particles():
    """The fixture run does carry fluid across the periodic face."""
    g = G.golden("peri_d04")
    cd = G.load_generated("peri_d04")
    keep = G.normal_rows(g["end_code"])
    idp, pos = g["end_idp"][keep], g["end_pos"][keep]
    x0 = cd.pos[idp, 0]   # case ids are the initial row indices
    assert (pos[:, 0] < x0 - 0.5).sum() > 0


# ---- GPU ------------------------------------------------------------------
def _wrapped(pos, pos0, size):
    """Particles that crossed a periodic face: moved by more than half a period."""
    d = np.abs(pos - pos0)
    return np.any(d[:, :2] > 0.5 * np.asarray(size[:2]), axis=1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["peri_d04", "perixy_d04"])
def test_periodic_channel_matches_reference_run(name):
    """x-periodic channel, and the xy-periodic box whose copies made for x
    are copied again for y."""
    from dualsphysics_gb300.sph import GbSphSingle
    g = G.golden(name)
    cd = G.load_generated(name)
    size = list(_lib.config(cd.params).maprealsize)
    s = GbSphSingle(0)
    s.setup(cd)
    dts = []
    for _ in range(len(g["dtlist"])):
        s.ComputeStep()
        dts.append(s.step_dt()[0])
    np.testing.assert_allclose(dts, g["dtlist"], rtol=1e-5)
    st = s.download()
    info = s.divinfo()
    s.close()
    # the same number of copies as the reference's last divide
    assert info["np"] == int(g["meta"]["end"]["np"]) and info["npb"] == int(g["meta"]["end"]["npb"])
    keep, rkeep = normal_rows(st["code"]), normal_rows(g["end_code"])
    assert keep.sum() == rkeep.sum() == cd.np
    o1 = np.argsort(st["idp"][keep])
    o2 = np.argsort(g["end_idp"][rkeep])
    np.testing.assert_array_equal(st["idp"][keep][o1], g["end_idp"][rkeep][o2])
    pos, rpos = st["pos"][keep][o1], g["end_pos"][rkeep][o2]
    vr, rvr = st["velrho"][keep][o1], g["end_velrho"][rkeep][o2]
    wrapped = _wrapped(pos, cd.pos, size)
    assert wrapped.sum() > 0 and (wrapped == _wrapped(rpos, cd.pos, size)).all()
    np.testing.assert_allclose(pos, rpos, atol=1e-6)
    np.testing.assert_allclose(vr[:, :3], rvr[:, :3], atol=2e-3)
    np.testing.assert_allclose(vr[:, 3], rvr[:, 3], rtol=1e-4)
    # each copy sits whole periods away from its source, along the periodic axes
    cp = ~keep
    src = {i: p for i, p in zip(st["idp"][keep], st["pos"][keep])}
    d = np.abs(np.array([st["pos"][k] - src[i] for k, i in zip(np.nonzero(cp)[0], st["idp"][cp])]))
    for k in range(2):
        on = cd.params.peri[k] != 0
        ok = (d[:, k] < 1e-12) | (on & (np.abs(d[:, k] - size[k]) < 1e-12))
        assert ok.all(), k
    assert (d[:, 2] < 1e-12).all() and (d[:, :2].max(axis=1) > 0).all()
    if name == "perixy_d04":   # copies of copies: one period along x and one along y
        assert ((np.abs(d[:, 0] - size[0]) < 1e-12) & (np.abs(d[:, 1] - size[1]) < 1e-12)).any()


@pytest.mark.gpu
def test_periodic_graph_replay_equals_eager():
    from dualsphysics_gb300.sph import GbSphSingle
    cd = G.load_generated("peri_d04")
    a, b = GbSphSingle(0), GbSphSingle(0)
    a.setup(cd)
    b.setup(cd)
    a.RunSteps(9, use_graph=False)
    b.RunSteps(9, use_graph=True)
    sa, sb = a.download(), b.download()
    for k in ("idp", "code", "dcell", "pos", "velrho"):
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    assert a.step_dt() == b.step_dt()
    a.close()
    b.close()


@pytest.mark.gpu
def test_periodic_copies_beyond_capacity_are_an_error():
    """The copies are counted on the device before any is written; when they
    do not fit, none is made and the host gets GBSPH_ECAPACITY."""
    from dualsphysics_gb300.sph import GbSphSingle
    cd = G.load_generated("peri_d04")
    ncopies = int(G.golden("peri_d04")["meta"]["s0"]["np"]) - cd.np
    assert ((cd.np + 255) & ~255) - cd.np < ncopies   # the rounded capacity cannot hold them
    s = GbSphSingle(0)
    with pytest.raises(_lib.GbsphError) as e:
        s.setup(cd, capacity=cd.np)
    assert e.value.code == -5 and "periodic" in str(e.value)   # GBSPH_ECAPACITY
    s.close()
    s = GbSphSingle(0)    # the device is still usable
    s.setup(cd)
    s.RunSteps(2, use_graph=False)
    s.close()


@pytest.mark.gpu
def test_periodic_part_output_holds_each_particle_once(tmp_path):
    from dualsphysics_gb300.sph import GbSphSingle
    cd = G.load_generated("peri_d04")
    s = GbSphSingle(0)
    s.setup(cd)
    s.dirout = str(tmp_path)
    s.part = 0
    s.RunSteps(5, use_graph=False)
    path = s.SaveData()
    st = s.download()
    s.close()
    assert (~normal_rows(st["code"])).sum() > 0           # the device state holds copies
    part = bi4.read(path, "JPartDataBi4")
    name = [it.name for it in part.items if it.name.startswith("PART_")][0]
    idp = part.item(name).array("Idp")
    assert np.array_equal(np.sort(idp), np.arange(cd.np))
    assert os.path.getsize(path) > 0
