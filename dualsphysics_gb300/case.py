"""Loading of a run case: the run XML and the initial particle file.

Host-side mirror of what JSph::LoadCaseConfig (JSph.cpp:1003-1100),
JSph::LoadCaseParticles (JSph.cpp:2151-2200), JPartsLoad4::LoadParticles
(JPartsLoad4.cpp:164-290) and JSph::ResizeMapLimits (JSph.cpp:1445-1476) read
and compute for the hot path: constants, execution parameters, particle
blocks (codes), positions/velocity/density/normals and the real map limits.
"""
from __future__ import annotations

import math
import os
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import bi4
from ._lib import Params

CODE_TYPE_FIXED, CODE_TYPE_MOVING, CODE_TYPE_FLOATING, CODE_TYPE_FLUID = 0x0, 0x800, 0x1000, 0x1800
BORDER_MAP = 0.05  # DualSphDef.h:112


class CaseError(ValueError):
    pass


@dataclass
class CaseData:
    name: str
    params: Params
    pos: np.ndarray      # (n,3) float64, ordered as in the file (boundary first)
    velrho: np.ndarray   # (n,4) float32
    idp: np.ndarray      # (n,) uint32
    code: np.ndarray     # (n,) uint16
    boundnor: np.ndarray | None  # (n,3) float32 or None
    npb: int
    nfluid: int
    time_max: float
    time_out: float
    savepos_double: bool
    raw: dict = field(default_factory=dict)

    @property
    def np(self) -> int:
        return int(self.pos.shape[0])


def _f(el, attr="value", default=None):
    if el is None:
        if default is None:
            raise CaseError("missing XML element")
        return default
    v = el.get(attr)
    if v is None:
        if default is None:
            raise CaseError(f"missing attribute '{attr}' in <{el.tag}>")
        return default
    return float(v)


def _pos_value(text: str, isposmin: bool):
    """JCaseEParms::CheckPosValue (JCaseEParms.cpp:374-414): returns (mode, value)
    with mode 'default', 'fixed', 'defvalue' or 'defprc'."""
    v = text.replace(" ", "").replace("\t", "").lower()
    if v == "default":
        return "default", 0.0
    if v.startswith("default+") or v.startswith("default-"):
        sign = v[7]
        if (isposmin and sign == "+") or (not isposmin and sign == "-"):
            raise CaseError(f"invalid simulationdomain value '{text}'")
        if v.endswith("%"):
            return "defprc", float(v[8:-1]) / 100.0
        return "defvalue", float(v[8:])
    return "fixed", float(v)


def load_case(casedir: str, casename: str, cellmode: str = "full") -> CaseData:
    """Reads <casename>.xml and <casename>.bi4.  `cellmode` is the reference's
    -cellmode run option: "full" (cells of 2h) or "half" (cells of h)."""
    if cellmode not in ("full", "half"):
        raise CaseError(f"unknown cell mode {cellmode!r} (full or half)")
    xml_path = os.path.join(casedir, casename + ".xml")
    bi4_path = os.path.join(casedir, casename + ".bi4")
    if not os.path.exists(xml_path):
        raise CaseError(f"case configuration was not found: {xml_path}")
    root = ET.parse(xml_path).getroot()
    ex = root.find("execution")
    if ex is None:
        raise CaseError("missing <execution> in the case XML")
    cte = ex.find("constants")
    par = ex.find("parameters")
    parts = ex.find("particles")
    if cte is None or par is None or parts is None:
        raise CaseError("missing constants/parameters/particles in the case XML")
    # --- parameters (JSph.cpp:663-857)
    kv = {}
    for p in par.findall("parameter"):
        kv[p.get("key")] = p.get("value")

    def gi(k, d):
        return int(float(kv[k])) if k in kv else d

    def gf(k, d):
        return float(kv[k]) if k in kv else d

    if gi("Kernel", 2) != 2:
        raise CaseError("only the Wendland kernel (Kernel=2) is implemented")
    if gi("Shifting", 0) != 0:
        raise CaseError("shifting is outside the implemented hot path")
    prm = Params()
    prm.tstep = gi("StepAlgorithm", 1)
    prm.verletsteps = gi("VerletSteps", 40)
    prm.tvisco = gi("ViscoTreatment", 1)
    prm.visco = gf("Visco", 0.0)
    prm.viscoboundfactor = gf("ViscoBoundFactor", 1.0)
    prm.tboundary = gi("Boundary", 1)
    if prm.tboundary == 2 and gi("SlipMode", 1) != 1:
        raise CaseError("only mDBC SlipMode=1 (vel=0) is implemented")
    prm.tdensity = gi("DensityDT", 0)
    prm.ddtvalue = gf("DensityDTvalue", 0.1)
    prm.coefdtmin = gf("CoefDtMin", 0.05)
    prm.dtini = max(0.0, gf("DtIni", 0.0))
    prm.dtmin = max(0.0, gf("DtMin", 0.0))
    prm.dtallparticles = 1 if gi("DtAllParticles", 0) == 1 else 0
    prm.rhopoutmin = gf("RhopOutMin", 700.0)
    prm.rhopoutmax = gf("RhopOutMax", 1300.0)
    prm.cellmode_div = 2 if cellmode == "half" else 1  # JSph.cpp:1880 (ScellDiv)
    # --- constants (JCaseCtes.cpp:208-222)
    prm.simulate2d = 1 if (cte.find("data2d") is not None and cte.find("data2d").get("value", "false").lower()
                           in ("1", "true")) else 0
    g = cte.find("gravity")
    prm.gravity[0], prm.gravity[1], prm.gravity[2] = (_f(g, "x"), _f(g, "y"), _f(g, "z"))
    prm.cflnumber = _f(cte.find("cflnumber"))
    prm.gamma = _f(cte.find("gamma"))
    prm.rhop0 = _f(cte.find("rhop0"))
    prm.dp = _f(cte.find("dp"))
    prm.h = _f(cte.find("h"))
    prm.b = _f(cte.find("b"))
    prm.massbound = _f(cte.find("massbound"))
    prm.massfluid = _f(cte.find("massfluid"))
    # --- particle blocks (JCaseParts.cpp:540-577) and codes (JSphMk.cpp:86-123)
    np_tot = int(parts.get("np"))
    nb = int(parts.get("nb"))
    blocks = []
    counters = {"fixed": 0, "moving": 0, "floating": 0, "fluid": 0}
    for el in parts:
        if el.tag.startswith("_") or el.tag == "properties":
            continue
        if el.tag not in counters:
            raise CaseError(f"unknown particle block <{el.tag}>")
        if el.tag in ("moving", "floating"):
            raise CaseError(f"<{el.tag}> particle blocks are outside the implemented hot path")
        blocks.append((el.tag, int(el.get("begin")), int(el.get("count"))))
    code_of = []
    nfixed = sum(1 for b in blocks if b[0] == "fixed")
    ifix = ifl = 0
    for kind, begin, count in blocks:
        if kind == "fixed":
            code_of.append((begin, count, CODE_TYPE_FIXED | ifix)); ifix += 1
        else:
            code_of.append((begin, count, CODE_TYPE_FLUID | ifl)); ifl += 1
    _ = nfixed
    # --- particles (JPartsLoad4.cpp:164-290)
    root_b = bi4.read(bi4_path, "JPartDataBi4")
    part = root_b.item("PART_0000")
    if part is None:
        raise CaseError("PART data is invalid")
    npok = int(part.get("Npok"))
    if npok != np_tot:
        raise CaseError("particle number does not match the configuration of the case")
    if "Idp" not in part.arrays:
        raise CaseError("only Idp (32 bits) is valid")
    idp = part.array("Idp").astype(np.uint32)
    pos = part.array("Posd").astype(np.float64) if "Posd" in part.arrays else part.array("Pos").astype(np.float64)
    vel = part.array("Vel").astype(np.float32)
    rhop = part.array("Rhop").astype(np.float32)
    velrho = np.concatenate([vel, rhop[:, None]], axis=1).astype(np.float32)
    boundnor = None
    if "BoundNor" in part.arrays:
        bn = part.array("BoundNor").astype(np.float32)
        boundnor = np.zeros((npok, 3), np.float32)
        boundnor[idp < nb] = bn[idp[idp < nb]]
    code = np.zeros(npok, np.uint16)
    for begin, count, cd in code_of:
        sel = (idp >= begin) & (idp < begin + count)
        code[sel] = cd
    # JSph::CheckRhoLimits (JSph.cpp:2140-2149)
    fl = idp >= nb
    if np.any((rhop[fl] < prm.rhopoutmin) | (rhop[fl] > prm.rhopoutmax)):
        raise CaseError("initial fluid density is out of limits")
    # --- map limits (JSph.cpp:2169-2178 + ResizeMapLimits 1445-1476)
    mpmin = np.array(root_b.get("MapPosMin", (0.0, 0.0, 0.0)), dtype=np.float64)
    mpmax = np.array(root_b.get("MapPosMax", (0.0, 0.0, 0.0)), dtype=np.float64)
    if np.any(mpmin != mpmax):
        mapmin, mapmax = mpmin, mpmax
    else:
        cmin = np.array(root_b.get("CasePosMin"), dtype=np.float64)
        cmax = np.array(root_b.get("CasePosMax"), dtype=np.float64)
        if np.all(cmin == cmax):
            cmin, cmax = pos.min(axis=0), pos.max(axis=0)
        border = float(np.float32(prm.h)) * BORDER_MAP
        mapmin, mapmax = cmin - border, cmax + border
        # simulationdomain
        sd = par.find("simulationdomain")
        dmin, dmax = mapmin.copy(), mapmax.copy()
        if sd is not None:
            dif = mapmax - mapmin
            pmin, pmax = sd.find("posmin"), sd.find("posmax")
            for k, ax in enumerate("xyz"):
                if pmin is not None and pmin.get(ax) is not None:
                    mode, v = _pos_value(pmin.get(ax), True)
                    if mode == "defprc":
                        dmin[k] = dmin[k] - dif[k] * v
                    elif mode == "defvalue":
                        dmin[k] = dmin[k] - v
                    elif mode == "fixed":
                        dmin[k] = v
                if pmax is not None and pmax.get(ax) is not None:
                    mode, v = _pos_value(pmax.get(ax), False)
                    if mode == "defprc":
                        dmax[k] = dmax[k] + dif[k] * v
                    elif mode == "defvalue":
                        dmax[k] = dmax[k] + v
                    elif mode == "fixed":
                        dmax[k] = v
            if np.any(dmin > mapmin) or np.any(dmax < mapmax):
                raise CaseError("domain limits are not valid")
        mapmin, mapmax = dmin, dmax
    for k in range(3):
        prm.maprealposmin[k] = float(mapmin[k])
        prm.maprealposmax[k] = float(mapmax[k])
    # order by id as the reference expects (boundary first)
    order = np.argsort(idp, kind="stable")
    return CaseData(name=casename, params=prm, pos=np.ascontiguousarray(pos[order]),
                    velrho=np.ascontiguousarray(velrho[order]), idp=np.ascontiguousarray(idp[order]),
                    code=np.ascontiguousarray(code[order]),
                    boundnor=None if boundnor is None else np.ascontiguousarray(boundnor[order]),
                    npb=nb, nfluid=npok - nb, time_max=gf("TimeMax", 0.0), time_out=gf("TimeOut", 0.0),
                    savepos_double=bool(gi("SavePosDouble", 0)), raw={"params": kv})


def params_to_dict(p: Params) -> dict:
    out = {}
    for name, _t in p._fields_:
        v = getattr(p, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def consts_to_dict(c) -> dict:
    out = {}
    for name, _t in c._fields_:
        v = getattr(c, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def math_isclose(a, b, rel=1e-12):
    return math.isclose(a, b, rel_tol=rel, abs_tol=0.0)
