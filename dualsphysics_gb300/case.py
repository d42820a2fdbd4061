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
    # moving boundaries: {"objects": [(idbegin, count)], "movements": [dict],
    # "events": [(obj, mov, start, finish)]} or None (read_motion)
    motion: dict | None = None

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
    # standard shifting (JSph.cpp:744-759); advanced shifting (4) is not built
    tshift = gi("Shifting", 0)
    if tshift not in (0, 1, 2, 3):
        raise CaseError(f"Shifting mode {tshift} is not supported (0-3)")
    prm = Params()
    # periodic conditions (JSph.cpp:815-826): Xperiodic with increments in y/z, ...
    for key, ax, comp in (("XPeriodicIncY", 0, 1), ("XPeriodicIncZ", 0, 2), ("YPeriodicIncX", 1, 0),
                          ("YPeriodicIncZ", 1, 2), ("ZPeriodicIncX", 2, 0), ("ZPeriodicIncY", 2, 1)):
        if key in kv:
            prm.peri[ax] = 1
            prm.periinc[3 * ax + comp] = float(kv[key])
    for key, axes in (("XYPeriodic", (0, 1)), ("XZPeriodic", (0, 2)), ("YZPeriodic", (1, 2))):
        if key in kv:
            for k in range(3):
                prm.peri[k] = int(k in axes)
            for k in range(9):
                prm.periinc[k] = 0.0
    prm.tshift = tshift
    if tshift:
        prm.shiftcoef = gf("ShiftCoef", -2.0)
        prm.shifttfs = gf("ShiftTFS", 0.0)
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
        if el.tag == "floating":
            raise CaseError(f"<{el.tag}> particle blocks are outside the implemented hot path")
        blocks.append((el.tag, int(el.get("begin")), int(el.get("count"))))
    order_kinds = [{"fixed": 0, "moving": 1, "fluid": 3}[b[0]] for b in blocks]
    if order_kinds != sorted(order_kinds):
        raise CaseError("particle blocks must come as fixed, moving, fluid")
    code_of = []
    ifix = imov = ifl = 0
    for kind, begin, count in blocks:
        if kind == "fixed":
            code_of.append((begin, count, CODE_TYPE_FIXED | ifix)); ifix += 1
        elif kind == "moving":
            code_of.append((begin, count, CODE_TYPE_MOVING | imov)); imov += 1
        else:
            code_of.append((begin, count, CODE_TYPE_FLUID | ifl)); ifl += 1
    motion = None
    if imov:
        motion = read_motion(ex.find("motion"), [(b, c) for k, b, c in blocks if k == "moving"])
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
        # JPartsLoad4::CalculeLimitsPos: dp/2 on periodic axes (JPartsLoad4.cpp:389-399)
        border = np.array([prm.dp / 2.0 if prm.peri[k] else float(np.float32(prm.h)) * BORDER_MAP
                           for k in range(3)])
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
        # ResizeMapLimits applies the domain to non-periodic axes only (JSph.cpp:1473-1475)
        for k in range(3):
            if not prm.peri[k]:
                mapmin[k], mapmax[k] = dmin[k], dmax[k]
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
                    savepos_double=bool(gi("SavePosDouble", 0)), raw={"params": kv}, motion=motion)


_VEC3 = ("vel", "ace", "velini", "freq", "ampl", "phase", "axisp1", "axisp2")


def _f32(v) -> float:
    """A value the reference reads with GetAttributeFloat (float, then double)."""
    return float(np.float32(float(v)))


def read_motion(node, objects: list) -> dict:
    """``case.execution.motion`` as JMotion::ReadXml reads it (JMotion.cpp:692-905):
    one ``<objreal ref>`` per moving block (ref k = the k-th moving block,
    JDsMotion::ConfigObjects), its movements and its ``<begin>`` events.
    Durations and event times are floats in the reference's reader."""
    if node is None:
        raise CaseError("moving particles without <motion> in the case XML")
    movs, evts = [], []
    seen = set()
    for obj in node:
        if obj.tag.startswith("_"):
            continue
        if obj.tag != "objreal":
            raise CaseError(f"<{obj.tag}> in <motion> is not supported (only <objreal> without children)")
        ref = int(obj.get("ref"))
        if ref < 0 or ref >= len(objects) or ref in seen:
            raise CaseError(f"motion reference {ref} does not match the moving blocks")
        seen.add(ref)
        for el in obj:
            if el.tag.startswith("_"):
                continue
            if el.tag == "begin":
                evts.append((ref, int(el.get("mov")), _f32(el.get("start")),
                             _f32(el.get("finish")) if el.get("finish") is not None else -1.0))
                continue
            if el.tag in ("obj", "objreal"):
                raise CaseError("nested motion objects are not supported")
            if el.tag not in ("wait", "mvrect", "mvrectace", "mvrot", "mvrotace", "mvrectsinu", "mvrotsinu",
                              "mvnull"):
                raise CaseError(f"movement <{el.tag}> is not supported")
            m = {"type": el.tag, "obj": ref, "id": int(el.get("id")), "next": int(el.get("next", 0)),
                 "duration": _f32(el.get("duration")) if el.tag != "mvnull" else 0.0,
                 "angdegrees": el.get("anglesunits", "degrees") == "degrees"}
            if el.get("anglesunits", "degrees") not in ("degrees", "radians"):
                raise CaseError("anglesunits must be degrees or radians")
            for ch in el:
                if ch.tag in ("axisp1", "axisp2") or (ch.tag in _VEC3 and el.tag in ("mvrect", "mvrectace",
                                                                                      "mvrectsinu")):
                    m[ch.tag] = (float(ch.get("x")), float(ch.get("y")), float(ch.get("z")))
                elif ch.tag in ("vel", "ace", "velini"):
                    m[ch.tag] = float(ch.get("ang"))
                elif ch.tag in ("freq", "ampl", "phase"):
                    m[ch.tag] = float(ch.get("v"))
            movs.append(m)
    if len(seen) != len(objects):
        raise CaseError("the number of moving objects does not match the predefined motions")
    return {"objects": list(objects), "movements": movs, "events": evts}


def motion_structs(motion: dict):
    """The gbsph_motion_create arguments of a read_motion() result."""
    from . import _lib
    objs = (_lib.MotionObject * len(motion["objects"]))(*[_lib.MotionObject(b, c) for b, c in motion["objects"]])
    movs = (_lib.Movement * max(1, len(motion["movements"])))()
    for i, m in enumerate(motion["movements"]):
        d = movs[i]
        d.type = _lib.MOV_TYPES[m["type"]]
        d.obj, d.id, d.nextid, d.duration = m["obj"], m["id"], m["next"], m["duration"]
        d.angdegrees = int(m["angdegrees"])
        t = m["type"]
        if t == "mvrect":
            d.v[:] = m["vel"]
        elif t == "mvrectace":
            d.a[:] = m["ace"]
            d.prev = int("velini" not in m)
            if "velini" in m:
                d.v[:] = m["velini"]
        elif t == "mvrectsinu":
            d.v[:], d.a[:] = m["freq"], m["ampl"]
            d.prev = int("phase" not in m)
            if "phase" in m:
                d.p[:] = m["phase"]
        elif t in ("mvrot", "mvrotace", "mvrotsinu"):
            d.axisp1[:], d.axisp2[:] = m["axisp1"], m["axisp2"]
            if t == "mvrot":
                d.s[0] = m["vel"]
            elif t == "mvrotace":
                d.s[1] = m["ace"]
                d.prev = int("velini" not in m)
                d.s[0] = m.get("velini", 0.0)
            else:
                d.s[0], d.s[1] = m["freq"], m["ampl"]
                d.prev = int("phase" not in m)
                d.s[2] = m.get("phase", 0.0)
    evts = (_lib.MotionEvent * max(1, len(motion["events"])))(
        *[_lib.MotionEvent(o, mv, st, fi) for o, mv, st, fi in motion["events"]])
    return objs, movs, len(motion["movements"]), evts, len(motion["events"])


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
