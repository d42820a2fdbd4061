"""The gbsph_run driver: the C++ host side above the C ABI (the Run loop of
JSphGpuSingle, JSphGpuSingle.cpp:950-1052, and the Part_%04u.bi4 writer of
JSph::SaveData, JSph.cpp:3062-3110).

* CPU: the driver's case loader (run XML + Case.bi4) reads the same case as the
  Python loader and derives the same constants (`-info`, no device touched);
  bad command lines and missing cases fail with the reference's exception line.
* GPU: the driver and the Python host loop (GbSphSingle.Run) write identical
  Part files for the same case and end time.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import goldens as G
from dualsphysics_gb300 import _lib, bi4
from dualsphysics_gb300 import casegen as cg
from dualsphysics_gb300.case import load_case
from dualsphysics_gb300.sph import GbSphSingle

DRIVER = os.path.join(G.ROOT, "dualsphysics_gb300", "gbsph_run")


def _driver():
    if not os.path.exists(DRIVER):
        pytest.fail("gbsph_run is not built (run __graft_entry__.build())")
    return DRIVER


def _write_case(tmp_path, name):
    spec = G.case_spec(name)
    cg.write_case(cg.make_dam_break(spec), str(tmp_path))
    return spec.name


@pytest.mark.parametrize("name", ["dbc_d04", "mdbc_d04", "sps_d04", "verlet_d04", "lam_d04", "half_d04", "mov_d04",
                                  "peri_d04"])
def test_driver_case_summary_matches_python_loader(tmp_path, name):
    import make_golden
    cn = _write_case(tmp_path, name)
    opts = make_golden.run_options(name)  # e.g. -cellmode:half, as the reference takes it
    out = subprocess.run([_driver(), str(tmp_path / cn), str(tmp_path / "out"), "-info"] + opts,
                         capture_output=True, text=True, check=True, timeout=120)
    info = json.loads(out.stdout)
    cd = load_case(str(tmp_path), cn, "half" if "-cellmode:half" in opts else "full")
    pc = _lib.config(cd.params)
    assert (info["np"], info["npb"]) == (len(cd.idp), cd.npb)
    assert (info["h"], info["b"], info["dp"]) == (cd.params.h, cd.params.b, cd.params.dp)
    assert info["maprealposmin"] == list(cd.params.maprealposmin)
    assert info["maprealposmax"] == list(cd.params.maprealposmax)
    assert np.float32(info["kernelsize2"]) == np.float32(pc.kernelsize2)
    assert info["cs0"] == pc.cs0
    assert info["domcellcode"] == pc.domcellcode
    assert info["mapcells"] == list(pc.mapcells)
    assert info["cellmode_div"] == cd.params.cellmode_div == pc.cellmode_div
    assert (info["tboundary"], info["tstep"], info["tdensity"], info["tvisco"]) == \
        (pc.tboundary, pc.tstep, pc.tdensity, pc.tvisco)
    # the particle arrays: exact integer sums, float sums to rounding of the order
    assert info["idsum"] == float(cd.idp.astype(np.float64).sum())
    assert info["codesum"] == float(cd.code.astype(np.float64).sum())
    assert info["possum"] == pytest.approx(float(cd.pos.sum()), rel=1e-12)
    assert info["rhosum"] == pytest.approx(float(cd.velrho[:, 3].astype(np.float64).sum()), rel=1e-12)
    nor = 0.0 if cd.boundnor is None else float(cd.boundnor.astype(np.float64).sum())
    assert info["norsum"] == pytest.approx(nor, rel=1e-9, abs=1e-9)
    mot = cd.motion or {"objects": [], "movements": [], "events": []}
    assert info["nmoving"] == sum(c for _, c in mot["objects"])
    assert (info["nmovements"], info["nevents"]) == (len(mot["movements"]), len(mot["events"]))


def test_driver_rejects_unknown_option_and_missing_case(tmp_path):
    cn = _write_case(tmp_path, "dbc_d04")
    r = subprocess.run([_driver(), str(tmp_path / cn), str(tmp_path / "out"), "-bogus"], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "*** Exception" in r.stderr and "-bogus" in r.stderr
    r = subprocess.run([_driver(), str(tmp_path / "NoSuchCase"), str(tmp_path / "out"), "-info"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "LoadCase" in r.stderr
    r = subprocess.run([_driver()], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "usage" in r.stderr


def _info(tmp_path, name, *opts):
    cn = _write_case(tmp_path, name)
    out = subprocess.run([_driver(), str(tmp_path / cn), str(tmp_path / "out"), "-info", *opts],
                         capture_output=True, text=True, timeout=120)
    return out


def test_driver_command_line_overrides_case_parameters(tmp_path):
    """The reference's run options override the XML parameters as
    JSph::LoadConfigCommands does (JSph.cpp:876-995); words are case-insensitive."""
    base = json.loads(_info(tmp_path, "mdbc_d04").stdout)
    assert (base["tstep"], base["tboundary"], base["tvisco"], base["tdensity"]) == (2, 2, 1, 2)
    r = _info(tmp_path, "mdbc_d04", "-gpu", "-Verlet:7", "-dbc", "-viscolamsps:1e-6", "-viscoboundfactor:0.5",
              "-ddt:1", "-cfl:0.1", "-rhopout:800:1200", "-stable", "-nortimes", "-svtimers:0", "-svpips:1:50")
    assert r.returncode == 0, r.stderr
    i = json.loads(r.stdout)
    assert (i["tstep"], i["verletsteps"], i["tboundary"], i["tvisco"], i["tdensity"]) == (1, 7, 1, 2, 1)
    assert np.float32(i["visco"]) == np.float32(1e-6) and i["viscoboundfactor"] == 0.5
    assert i["ddtvalue"] == base["ddtvalue"] and i["cflnumber"] == 0.1
    assert (i["rhopoutmin"], i["rhopoutmax"]) == (800.0, 1200.0)
    # -ddt:0 drops the diffusion value; -ddtvalue sets it; -ddt on a case without one takes 0.1
    i = json.loads(_info(tmp_path, "mdbc_d04", "-ddt:0").stdout)
    assert (i["tdensity"], i["ddtvalue"]) == (0, 0.0)
    i = json.loads(_info(tmp_path, "mdbc_d04", "-ddt:3", "-ddtvalue:0.2").stdout)
    assert (i["tdensity"], np.float32(i["ddtvalue"])) == (3, np.float32(0.2))
    i = json.loads(_info(tmp_path, "dbc_d04", "-CELLMODE:H", "-symplectic", "-wendland").stdout)
    assert i["cellmode_div"] == 2 and i["tstep"] == 2


@pytest.mark.parametrize("opt", ["-viscoart:11", "-ddt:4", "-ddtvalue:2", "-cfl:0", "-svpips:3", "-cubic", "-cpu",
                                 "-mdbc_noslip", "-sv:vtk", "-cellmode:x"])
def test_driver_rejects_invalid_options(tmp_path, opt):
    r = _info(tmp_path, "dbc_d04", opt)
    assert r.returncode == 1 and "*** Exception: options" in r.stderr


def test_driver_mdbc_needs_normals(tmp_path):
    r = _info(tmp_path, "dbc_d04", "-mdbc")
    assert r.returncode == 1 and "normals" in r.stderr


def _parts(dirout):
    d = os.path.join(dirout, "data")
    return sorted(f for f in os.listdir(d) if f.startswith("Part_") and f.endswith(".bi4"))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["dbc_d04", "mdbc_d04", "mov_d04", "peri_d04"])
def test_driver_parts_equal_python_run(tmp_path, name):
    """gbsph_run and GbSphSingle.Run step the same case to the same end time
    and write bit-identical particle data in every Part file."""
    cn = _write_case(tmp_path, name)
    tmax = 0.012
    d_out, p_out = str(tmp_path / "drv"), str(tmp_path / "py")
    r = subprocess.run([_driver(), str(tmp_path / cn), d_out, f"-tmax:{tmax}", "-sv:bi4"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "Steps per second" in r.stdout
    s = GbSphSingle(0)
    res = s.Run(str(tmp_path), cn, p_out, time_max=tmax)
    s.close()
    ncase = load_case(str(tmp_path), cn).np
    dp, pp = _parts(d_out), _parts(p_out)
    assert dp == pp and len(dp) >= 2, (dp, pp)
    for f in dp:
        a = bi4.read(os.path.join(d_out, "data", f), "JPartDataBi4")
        b = bi4.read(os.path.join(p_out, "data", f), "JPartDataBi4")
        ka = [it.name for it in a.items if it.name.startswith("PART_")]
        assert ka == [it.name for it in b.items if it.name.startswith("PART_")] and len(ka) == 1
        pa, pb = a.item(ka[0]), b.item(ka[0])
        assert pa.get("Step") == pb.get("Step") and pa.get("TimeStep") == pb.get("TimeStep")
        for arr in ("Idp", "Vel", "Rhop"):
            np.testing.assert_array_equal(pa.array(arr), pb.array(arr), err_msg=f"{f}: {arr}")
        # each particle of the case at most once: periodic copies are not saved
        idp = pa.array("Idp")
        assert len(np.unique(idp)) == len(idp) <= ncase
        posname = "Posd" if "Posd" in pa.arrays else "Pos"
        np.testing.assert_array_equal(pa.array(posname), pb.array(posname), err_msg=f"{f}: {posname}")
    assert res["steps"] > 0


@pytest.mark.gpu
def test_driver_pips_summary_and_csv(tmp_path):
    """-svpips:2:<n> samples the interaction count every n steps and at the
    last, prints the reference's summary lines and writes PIPS.csv."""
    cn = _write_case(tmp_path, "dbc_d04")
    out = str(tmp_path / "out")
    r = subprocess.run([_driver(), str(tmp_path / cn), out, "-nsteps:12", "-sv:none", "-svpips:2:5"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "GPIPS" in r.stdout and "Total particle interactions (f+b)" in r.stdout
    rows = open(os.path.join(out, "PIPS.csv")).read().strip().split("\n")
    assert rows[0].startswith("Time [s];RunTime [s];Nstep;RealFluid")
    steps = [int(x.split(";")[2]) for x in rows[1:]]
    assert steps == [0, 5, 10, 12]
    # the count of a sample equals a direct count of the same state at step 0
    s = GbSphSingle(0)
    s.setup(load_case(str(tmp_path), cn))
    p = s.pips()
    s.close()
    first = rows[1].split(";")
    assert (int(first[3]), int(first[4]), int(first[5]), int(first[6])) == \
        (p["real_fluid"], p["real_bound"], p["checked_fluid"], p["checked_bound"])


# ---- restart from a Part file (-partbegin) --------------------------------------
def _restart_fixture(tmp_path):
    """The restart fixture (make_golden.py restart): the reference's state after
    n1 steps written by this library's Part writer, and what the reference did
    with it.  Returns (fixture, case name, directory holding Part_0001.bi4)."""
    z = np.load(os.path.join(G.GOLDEN, "restart_dbc_d04.npz"))
    cn = _write_case(tmp_path, "dbc_d04")
    d = tmp_path / "part" / "data"
    d.mkdir(parents=True)
    (d / "Part_0001.bi4").write_bytes(z["part_bytes"].tobytes())
    return z, cn, str(d)


def _meta(z, key):
    return json.loads(bytes(z[key]).decode())


def test_reference_reads_our_part_file_losslessly():
    """The reference restarted (-partbegin:1:1, its own JPartsLoad4 reader) from
    a Part_0001.bi4 and Part_Head.ibi4 written by this library's writers: the
    state it loaded is the one written, bit for bit, with the Part's time and
    SymplecticDtPre; its restarted run then ran as its continuous run did."""
    z = np.load(os.path.join(G.GOLDEN, "restart_dbc_d04.npz"))
    a, b = np.argsort(z["first_idp"]), np.argsort(z["restart_s0_idp"])
    np.testing.assert_array_equal(z["first_idp"][a], z["restart_s0_idp"][b])
    np.testing.assert_array_equal(z["first_pos"][a], z["restart_s0_pos"][b])
    np.testing.assert_array_equal(z["first_velrho"][a], z["restart_s0_velrho"][b])
    m1, m0 = _meta(z, "first_meta_json"), _meta(z, "restart_s0_meta_json")
    assert m0["timestep"] == m1["timestep"] and m0["symplecticdtpre"] == m1["symplecticdtpre"]
    n2 = int(z["n2"])
    np.testing.assert_array_equal(z["restart_dtlist"], z["cont_dtlist"][-n2:])


def test_driver_reads_the_restart_part(tmp_path):
    """gbsph_run -partbegin:1:1 <dir> loads the same state from the same file
    (host only: -info touches no device)."""
    z, cn, d = _restart_fixture(tmp_path)
    r = subprocess.run([_driver(), str(tmp_path / cn), str(tmp_path / "out"), "-partbegin:1:1", d, "-info"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    i = json.loads(r.stdout)
    m1 = _meta(z, "first_meta_json")
    assert i["np"] == len(z["restart_s0_idp"]) and i["npb"] == int(m1["npb"])
    assert i["idsum"] == float(z["restart_s0_idp"].astype(np.float64).sum())
    assert i["possum"] == pytest.approx(float(z["restart_s0_pos"].sum()), rel=1e-12)
    assert i["rhosum"] == pytest.approx(float(z["restart_s0_velrho"][:, 3].astype(np.float64).sum()), rel=1e-12)
    assert i["parttime"] == float(m1["timestep"]) == i["timeini"]
    assert i["dtpre"] == float(m1["symplecticdtpre"])
    # with first = 0 the run's clock starts at 0 (JSph.cpp:2224-2225)
    i0 = json.loads(subprocess.run([_driver(), str(tmp_path / cn), str(tmp_path / "out"), "-partbegin:1", d, "-info"],
                                   capture_output=True, text=True, timeout=120, check=True).stdout)
    assert i0["timeini"] == 0.0 and i0["parttime"] == i["parttime"]
    r = subprocess.run([_driver(), str(tmp_path / cn), str(tmp_path / "out"), "-partbegin:2:1", d, "-info"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "LoadPart" in r.stderr            # no Part_0002 there
    r = subprocess.run([_driver(), str(tmp_path / cn), str(tmp_path / "out"), "-partbegin:1"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "directory" in r.stderr


@pytest.mark.gpu
def test_driver_restart_matches_reference_restart(tmp_path):
    """gbsph_run restarted from the same Part file steps as the reference's
    restarted run: every dt within 1e-5 and the final state within the
    multi-step tolerance; its first Part is the restart state itself."""
    z, cn, d = _restart_fixture(tmp_path)
    n2 = int(z["n2"])
    out = str(tmp_path / "out")
    r = subprocess.run([_driver(), str(tmp_path / cn), out, "-partbegin:1:1", d, f"-nsteps:{n2}", "-tout:1e-12",
                        "-sv:bi4"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    parts = _parts(out)
    assert parts == ["Part_%04u.bi4" % k for k in range(1, n2 + 2)], parts
    assert os.path.exists(os.path.join(out, "data", "Part_Head.ibi4"))
    pts = []
    for f in parts:
        root = bi4.read(os.path.join(out, "data", f), "JPartDataBi4")
        pts.append(root.item([it.name for it in root.items if it.name.startswith("PART_")][0]))
    m1, mr = _meta(z, "first_meta_json"), _meta(z, "restart_meta_json")
    times = np.array([p.get("TimeStep") for p in pts])
    assert times[0] == float(m1["timestep"])
    np.testing.assert_allclose(np.diff(times), z["restart_dtlist"], rtol=1e-5)
    assert times[-1] == pytest.approx(float(mr["timestep"]), rel=1e-6)
    last = pts[-1]
    idp = last.array("Idp")
    o1, o2 = np.argsort(idp), np.argsort(z["restart_idp"])
    np.testing.assert_array_equal(idp[o1], z["restart_idp"][o2])
    np.testing.assert_allclose(last.array("Posd")[o1], z["restart_pos"][o2], atol=1e-6)
    np.testing.assert_allclose(last.array("Vel")[o1], z["restart_velrho"][o2, :3], atol=2e-3)
    np.testing.assert_allclose(last.array("Rhop")[o1], z["restart_velrho"][o2, 3], rtol=1e-4)
