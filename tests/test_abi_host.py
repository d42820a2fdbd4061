"""Host-side checks that need no GPU: the C ABI library loads and exports every
entry point of include/gbsph.h; the product's constant derivation equals the
oracle's and the reference's; the bi4 and case-XML readers/writers."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import goldens as G
import pyoracle as po
from dualsphysics_gb300 import _lib, bi4
from dualsphysics_gb300 import casegen as cg
from dualsphysics_gb300.case import load_case

HEADER = os.path.join(G.ROOT, "include", "gbsph.h")


def header_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gbsph_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    L = _lib.lib()
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_lib.SIGNATURES), "ctypes signatures out of sync with the header"


@pytest.mark.parametrize("name", G.CASE_NAMES)
def test_product_config_equals_oracle_and_reference(name):
    cd = G.load_generated(name)
    pc = _lib.config(cd.params)
    oc = po.config(po.params_from(cd.params))
    assert C.sizeof(pc) == C.sizeof(oc)
    assert bytes(pc) == bytes(oc), "product and oracle constants differ"
    m = G.golden(name)["meta"]["s0"]
    assert pc.domcellcode == int(m["domcellcode"])
    assert np.float32(pc.kernelsize2) == np.float32(float(m["kernelsize2"]))
    assert pc.cs0 == pytest.approx(float(m["cs0"]), rel=1e-15)


def test_config_rejects_invalid():
    p = _lib.Params()
    with pytest.raises(_lib.GbsphError):
        _lib.config(p)


def test_bi4_roundtrip(tmp_path):
    root = bi4.make_partdata_root(casename="t", appname="a", data2d=False, casenp=3, casenfixed=1, casenmoving=0,
                                  casenfloat=0, casenfluid=2, caseposmin=(0, 0, 0), caseposmax=(1, 1, 1), dp=0.1,
                                  h=0.2, b=1e5, rhop0=1000, gamma=7, massbound=1, massfluid=1)
    pos = np.array([[0, 0, 0], [0.5, 0.25, 0.125], [1, 1, 1]], np.float64)
    vel = np.arange(9, dtype=np.float32).reshape(3, 3)
    root.items.append(bi4.make_part(0, 0.5, 3, 0, 7, (0, 0, 0), (1, 1, 1), np.arange(3, dtype=np.uint32), pos, vel,
                                    np.array([1000, 1001, 1002], np.float32), posdouble=True))
    path = str(tmp_path / "x.bi4")
    bi4.write(path, root)
    with open(path, "rb") as f:
        head = f.read(64)
    assert head.startswith(b"#FileJBD JPartDataBi4") and head[58:60] == b"\n\x00" and head[60] == 0
    r = bi4.read(path, "JPartDataBi4")
    assert r.get("CaseNp") == 3 and r.get("Gamma") == 7.0 and r.get("Data2d") is False
    p = r.item("PART_0000")
    assert p.get("Step") == 7 and p.get("TimeStep") == 0.5
    np.testing.assert_array_equal(p.array("Posd"), pos)
    np.testing.assert_array_equal(p.array("Vel"), vel)
    with pytest.raises(bi4.Bi4Error):
        bi4.read(path, "SomethingElse")


def test_bi4_rejects_corrupt(tmp_path):
    path = str(tmp_path / "bad.bi4")
    with open(path, "wb") as f:
        f.write(b"#FileJBD JPartDataBi4" + b" " * 37 + b"\n\x00" + bytes([0, 0, 0, 0]) + b"\x05\x00\x00\x00junk")
    with pytest.raises(bi4.Bi4Error):
        bi4.read(path)


def test_case_generator_counts():
    c1 = cg.make_dam_break(cg.spec_c1(dp=0.01))
    assert (c1.np - c1.npb, c1.npb) == (86428, 94884)
    c5 = cg.make_dam_break(cg.spec_c5())
    assert c5.np - c5.npb == 11424


def test_case_loader_reads_generated_files(tmp_path):
    case = cg.make_dam_break(cg.spec_c2(dp=0.04, name="ld"))
    cg.write_case(case, str(tmp_path))
    cd = load_case(str(tmp_path), "ld")
    assert cd.np == case.np and cd.npb == case.npb
    np.testing.assert_array_equal(cd.pos, case.pos)
    assert cd.boundnor is not None and np.any(cd.boundnor[: cd.npb] != 0)
    assert cd.params.tboundary == _lib.BC_MDBC and cd.params.tstep == _lib.STEP_SYMPLECTIC
    assert np.all(cd.code[cd.npb:] == 0x1800)


def test_case_loader_rejects_unsupported(tmp_path):
    spec = cg.spec_c1(dp=0.05, name="ux", extra_params={"Kernel": 1})
    cg.write_case(cg.make_dam_break(spec), str(tmp_path))
    from dualsphysics_gb300.case import CaseError
    with pytest.raises(CaseError):
        load_case(str(tmp_path), "ux")
