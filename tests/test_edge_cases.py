"""Edge cases of the step on the device against the oracle: particles that
leave the domain or whose density leaves [RhopOutMin, RhopOutMax] (excluded
at the next divide, counted), a case with no fluid at all, and a case with a
single fluid particle."""
import copy

import numpy as np
import pytest

import goldens as G
import pyoracle as po

pytestmark = pytest.mark.gpu


def _sub(cd, rows):
    """The case restricted to `rows` (boundary rows first), ids renumbered."""
    c = copy.copy(cd)
    rows = np.asarray(rows)
    c.pos = np.ascontiguousarray(cd.pos[rows])
    c.velrho = np.ascontiguousarray(cd.velrho[rows])
    c.code = np.ascontiguousarray(cd.code[rows])
    c.idp = np.arange(len(rows), dtype=np.uint32)
    if cd.boundnor is not None:
        c.boundnor = np.ascontiguousarray(cd.boundnor[rows])
    c.npb = int(np.sum(rows < cd.npb))
    return c


def _run(cd, nsteps):
    from dualsphysics_gb300.sph import GbSphSingle
    s = GbSphSingle(0)
    s.setup(cd)
    o = po.Sim(po.config(po.params_from(cd.params)), cd.pos, cd.velrho, cd.idp, cd.code, cd.npb, cd.boundnor)
    dts = []
    for _ in range(nsteps):
        s.ComputeStep()
        dts.append((s.step_dt()[0], o.step()))
    st, info = s.download(), s.divinfo()
    s.close()
    return st, info, o, dts


def _compare(st, o):
    os_ = o.state()
    assert len(st["idp"]) == len(os_["idp"])
    o1, o2 = np.argsort(st["idp"]), np.argsort(os_["idp"])
    np.testing.assert_array_equal(st["idp"][o1], os_["idp"][o2])
    np.testing.assert_allclose(st["pos"][o1], os_["pos"][o2], atol=1e-6)
    np.testing.assert_allclose(st["velrho"][o1, 3], os_["velrho"][o2, 3], rtol=1e-4)


def test_particles_leaving_the_domain_and_the_density_range_are_excluded():
    cd = copy.copy(G.load_generated("dbc_d04"))
    cd.velrho = cd.velrho.copy()
    top = np.argsort(cd.pos[cd.npb:, 2])[-6:] + cd.npb      # the highest fluid particles ...
    cd.velrho[top, 2] = 60.0                                 # ... thrown up through the top of the map
    low = np.arange(cd.npb, cd.npb + 3)
    cd.velrho[low, 3] = 1400.0                               # above RhopOutMax = 1300
    st, info, o, dts = _run(cd, 12)
    assert info["nout_total"] == o.nout() == cd.np - len(st["idp"])
    assert info["nout_total"] >= 9
    gone = set(range(cd.np)) - set(int(i) for i in st["idp"])
    assert set(int(i) for i in cd.idp[low]) <= gone and set(int(i) for i in cd.idp[top]) <= gone
    np.testing.assert_allclose([a for a, _ in dts], [b for _, b in dts], rtol=1e-5)
    _compare(st, o)


def test_case_without_fluid():
    full = G.load_generated("dbc_d04")
    cd = _sub(full, np.arange(full.npb))
    st, info, o, dts = _run(cd, 4)
    assert info["np"] == info["npb"] == cd.npb
    np.testing.assert_allclose([a for a, _ in dts], [b for _, b in dts], rtol=1e-12)
    np.testing.assert_array_equal(np.sort(st["idp"]), np.arange(cd.npb))
    _compare(st, o)


def test_single_fluid_particle():
    full = G.load_generated("dbc_d04")
    k = full.npb + int(np.argmax(full.pos[full.npb:, 2]))    # the top fluid particle: free fall
    cd = _sub(full, np.r_[np.arange(full.npb), k])
    st, info, o, dts = _run(cd, 5)
    assert info["np"] - info["npb"] == 1
    np.testing.assert_allclose([a for a, _ in dts], [b for _, b in dts], rtol=1e-5)
    _compare(st, o)
    f = st["idp"] == cd.npb
    assert st["velrho"][f, 2][0] < 0                          # falling


# ---- failure detection (faults made on the host: no GPU fault is involved) ----
def test_nan_in_the_state_is_reported_as_nan_dt():
    """A NaN velocity uploaded in one fluid particle: its neighbours' density
    rates are NaN after the first interaction, the maximum behind dt keeps the
    NaN, and the step reports GBSPH_ENAN_DT (the reference's check of a NaN or
    infinite dt, JSphCpu.cpp:2053-2060, JSphGpu.cpp:1122-1131)."""
    from dualsphysics_gb300 import _lib
    from dualsphysics_gb300.sph import GbSphSingle
    cd = copy.copy(G.load_generated("dbc_d04"))
    cd.velrho = cd.velrho.copy()
    k = cd.npb + (cd.np - cd.npb) // 2                      # a fluid particle inside the column
    cd.velrho[k, 0] = np.nan
    s = GbSphSingle(0)
    s.setup(cd)
    with pytest.raises(_lib.GbsphError) as e:
        s.ComputeStep()
        s.step_dt()
    assert e.value.code == -3 and "NaN" in str(e.value)
    s.close()
    # the same state without the NaN steps normally
    cd.velrho[k, 0] = 0.0
    s = GbSphSingle(0)
    s.setup(cd)
    s.ComputeStep()
    assert np.isfinite(s.step_dt()[0])
    s.close()


def test_moving_boundary_driven_out_of_the_map_is_reported():
    """A moving tank driven upwards at 5 m/s by a uniform rectilinear motion
    (mvrect) leaves the map through its top: the divide after the step that
    moved boundary particles out reports GBSPH_EBOUND_OUT (the reference's
    "boundary particles out" exception, JSph.cpp:2837)."""
    from dualsphysics_gb300 import _lib
    from dualsphysics_gb300.sph import GbSphSingle
    cd = copy.copy(G.load_generated("mov_d04"))
    nb = cd.npb
    cd.motion = {"objects": [(0, nb)],
                 "movements": [{"obj": 0, "next": 0, "angdegrees": True, "type": "mvrect", "id": 1,
                                "duration": 100.0, "vel": (0.0, 0.0, 5.0)}],
                 "events": [(0, 1, 0.0, -1.0)]}
    s = GbSphSingle(0)
    s.setup(cd)
    steps = 0
    with pytest.raises(_lib.GbsphError) as e:
        for steps in range(1, 4001):
            s.ComputeStep()
            s.step_dt()
    assert e.value.code == -4 and "boundary" in str(e.value)
    assert steps > 1                                          # the tank first moved inside the map
    s.close()
