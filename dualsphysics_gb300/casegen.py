"""Synthetic case generator for the 3-D dam-break workloads.

The reference's pre-processor (GenCase) is not part of the reference source
tree, so cases are generated here and written in the reference's own run
formats: the run XML read by JSph::LoadCaseConfig (JSph.cpp:1003-1100;
``case.execution.{constants,parameters,particles}``, JCaseCtes.cpp:208-222,
JCaseParts.cpp:540-577, JCaseEParms.cpp:444-478) and the particle file read by
JPartsLoad4::LoadParticles (JPartsLoad4.cpp:164-290).

Geometry (all sizes in metres):

* tank interior ``[0,Lx]x[0,Ly]x[0,Lz]``, fluid column against the x=0 wall on
  the lattice ``(i,j,k)*dp``;
* 3-layer DBC walls and floor outside the interior, open top, up to z=Lz;
* optional box obstacle (solid lattice block) standing on the floor;
* hydrostatic initial density of the fluid, rho = rho0*(1+rho0*g*(H-z)/B)^(1/gamma)
  with H the top of the fluid column (the "water column" density gradient);
  boundary particles start at rho0;
* mDBC normals (``BoundNor``): vector from each boundary particle to the
  nearest point of the boundary surface, which lies dp/2 outside the outer
  particle layer of each solid; the solver doubles it to reach the ghost node
  (JSph.cpp:1411-1418);
* optional tank motion (sloshing): the walls become one moving block with a
  chain of predefined movements in the run XML's ``case.execution.motion``
  (the schema JMotion::ReadXml reads, JMotion.cpp:692-905), starting at t=0.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import bi4

CODE_TYPE_FLUID = 0x1800
CODE_TYPE_MOVING = 0x0800


@dataclass
class CaseSpec:
    name: str = "Dam"
    tank: tuple = (1.6, 0.67, 0.4)
    column: tuple = (0.4, 0.67, 0.3)
    dp: float = 0.01
    obstacle: tuple | None = None           # (x0, y0, sx, sy, sz)
    boundary: str = "dbc"                   # dbc | mdbc
    jitter: float = 0.0                     # fraction of dp, uniform in [-j,j]^3
    init_vel: float = 0.0                   # seeded uniform fluid velocity in [-v,v]^3 (m/s)
    seed: int = 0
    coefh: float = 1.2
    coefsound: float = 20.0
    hswl: float | None = None               # defaults to the column height
    rhop0: float = 1000.0
    gamma: float = 7.0
    gravity: tuple = (0.0, 0.0, -9.81)
    cflnumber: float = 0.2
    visco_treatment: int = 1                # 1 artificial, 2 laminar+sps, 3 laminar
    visco: float = 0.01
    viscoboundfactor: float = 1.0
    density_dt: int = 2
    density_dt_value: float = 0.1
    step_algorithm: int = 2                 # 1 verlet, 2 symplectic
    verlet_steps: int = 40
    time_max: float = 0.5
    time_out: float = 0.01
    posmax_z: str = "default + 50%"
    posmin_x: str = "default"               # a moving tank needs room beyond its walls
    posmax_x: str = "default"
    extra_params: dict = field(default_factory=dict)
    # movements of the tank walls (JMotion XML), each a dict with type
    # (mvrect, mvrectace, mvrot, mvrotace, mvrectsinu, mvrotsinu, wait), id,
    # duration, optional next and anglesunits, and its elements (vector
    # values as (x, y, z), rotation scalars as numbers); the first one starts
    # at t=0.  None: fixed walls.
    motion: list | None = None
    # periodic in x (a channel): walls only on the floor and the y sides, the
    # fluid fills the whole period [0, Lx) with spacing dp, and the run XML
    # declares XPeriodicIncY=0; init_vel_x gives the fluid a uniform x velocity
    periodic_x: bool = False
    init_vel_x: float = 0.0
    # periodic in y as well (or alone): no walls on the y sides, the fluid fills
    # the period [0, Ly), YPeriodicIncX=0; init_vel_y a uniform y velocity
    periodic_y: bool = False
    init_vel_y: float = 0.0
    # periodic in z: no floor, the fluid fills the period [0, Lz) and falls
    # through the bottom face back in at the top (ZPeriodicIncX=0)
    periodic_z: bool = False
    init_vel_z: float = 0.0
    # cross increment of the x periodicity: a particle leaving through x = Lx
    # comes back at x = 0 shifted by this much in y (XPeriodicIncY)
    peri_inc_y: float = 0.0


@dataclass
class Case:
    spec: CaseSpec
    pos: np.ndarray        # (n,3) f64
    vel: np.ndarray        # (n,3) f32
    rhop: np.ndarray       # (n,) f32
    idp: np.ndarray        # (n,) u32
    code: np.ndarray       # (n,) u16
    boundnor: np.ndarray   # (nbound,3) f32
    blocks: list           # [(kind, mkbound/mkfluid, begin, count)]
    npb: int
    h: float
    b: float
    mass: float

    @property
    def np(self) -> int:
        return int(self.pos.shape[0])


def _lattice(n0, n1, n2):
    i, j, k = np.meshgrid(np.arange(n0[0], n0[1] + 1), np.arange(n1[0], n1[1] + 1),
                          np.arange(n2[0], n2[1] + 1), indexing="ij")
    # z slowest, then y, then x (x fastest) for memory order close to cells
    return np.stack([i.transpose(2, 1, 0).ravel(), j.transpose(2, 1, 0).ravel(),
                     k.transpose(2, 1, 0).ravel()], axis=1)


def _nsteps(length: float, dp: float) -> int:
    return int(math.floor(length / dp + 1e-6))


def make_dam_break(spec: CaseSpec) -> Case:
    dp = spec.dp
    nx, ny, nz = (_nsteps(v, dp) for v in spec.tank)
    # --- walls: lattice i in [-3,nx+3], j in [-3,ny+3], k in [-3,nz] minus interior
    # one period [0, n*dp) of the walls along each periodic axis
    wx = (0, nx - 1) if spec.periodic_x else (-3, nx + 3)
    wy = (0, ny - 1) if spec.periodic_y else (-3, ny + 3)
    wl = _lattice(wx, wy, (0, nz - 1) if spec.periodic_z else (-3, nz))
    inside = ((wl[:, 0] >= 0) & (wl[:, 0] <= nx) & (wl[:, 1] >= 0) & (wl[:, 1] <= ny) & (wl[:, 2] >= 0))
    wall = wl[~inside].astype(np.float64) * dp
    # --- obstacle: solid lattice block on the floor
    obst = np.zeros((0, 3))
    if spec.obstacle is not None:
        x0, y0, sx, sy, sz = spec.obstacle
        i0, j0 = int(round(x0 / dp)), int(round(y0 / dp))
        ob = _lattice((i0, i0 + _nsteps(sx, dp)), (j0, j0 + _nsteps(sy, dp)), (0, _nsteps(sz, dp)))
        obst = ob.astype(np.float64) * dp
    # --- fluid column
    fx, fy, fz = (_nsteps(v, dp) for v in spec.column)
    if spec.periodic_x:
        fx = nx - 1
    if spec.periodic_y:
        fy = ny - 1
    if spec.periodic_z:
        fz = nz - 1
    fl = _lattice((0, fx), (0, fy), (0, fz)).astype(np.float64) * dp
    if spec.obstacle is not None and len(obst):
        lo, hi = obst.min(axis=0) - 0.5 * dp, obst.max(axis=0) + 0.5 * dp
        keep = ~np.all((fl > lo) & (fl < hi), axis=1)
        fl = fl[keep]
    if spec.jitter:
        rng = np.random.default_rng(spec.seed)
        fl = fl + rng.uniform(-spec.jitter * dp, spec.jitter * dp, size=fl.shape)
    nbw, nbo, nf = len(wall), len(obst), len(fl)
    npb = nbw + nbo
    pos = np.concatenate([wall, obst, fl], axis=0)
    n = len(pos)
    # --- constants (GenCase conventions, CaseDambreak_Def.xml constantsdef)
    g = abs(spec.gravity[2])
    hswl = spec.hswl if spec.hswl is not None else spec.column[2]
    cs0 = spec.coefsound * math.sqrt(g * hswl)
    b = cs0 * cs0 * spec.rhop0 / spec.gamma
    h = spec.coefh * math.sqrt(3.0 * dp * dp)
    mass = spec.rhop0 * dp ** 3
    # --- density: hydrostatic fluid, rho0 boundary
    rhop = np.full(n, spec.rhop0, dtype=np.float64)
    if nf:
        htop = fl[:, 2].max()
        depth = np.maximum(htop - fl[:, 2], 0.0)
        rhop[npb:] = spec.rhop0 * (1.0 + spec.rhop0 * g * depth / b) ** (1.0 / spec.gamma)
    # --- codes: fixed blocks 0 (tank), 1 (obstacle); fluid block 0 -- or,
    # with a tank motion, the walls as moving block 0 (JSphMk.cpp:86-123)
    code = np.zeros(n, dtype=np.uint16)
    code[nbw:npb] = 1
    code[npb:] = CODE_TYPE_FLUID
    if spec.motion:
        if nbo:
            raise ValueError("a moving tank with an obstacle is not generated (fixed blocks must come first)")
        code[:nbw] = CODE_TYPE_MOVING
        blocks = [("moving", 0, 0, nbw)]
    else:
        blocks = [("fixed", 0, 0, nbw)]
    if nbo:
        blocks.append(("fixed", 1, nbw, nbo))
    blocks.append(("fluid", 0, npb, nf))
    # --- mDBC normals
    boundnor = np.zeros((npb, 3), dtype=np.float32)
    if spec.boundary == "mdbc":
        half = 0.5 * dp
        lo = np.array([-half, -half, -half])
        hi = np.array([nx * dp + half, ny * dp + half, np.inf])
        q = np.clip(wall, lo, hi)
        boundnor[:nbw] = (q - wall).astype(np.float32)
        if nbo:
            olo, ohi = obst.min(axis=0) - half, obst.max(axis=0) + half
            ohi[2] = ohi[2]  # top face is a boundary too
            d = np.stack([obst[:, 0] - olo[0], ohi[0] - obst[:, 0], obst[:, 1] - olo[1],
                          ohi[1] - obst[:, 1], np.full(nbo, np.inf), ohi[2] - obst[:, 2]], axis=1)
            face = np.argmin(d, axis=1)
            dist = d[np.arange(nbo), face]
            nvec = np.zeros((nbo, 3))
            sign = np.array([-1, 1, -1, 1, -1, 1], dtype=np.float64)
            axis = face // 2
            nvec[np.arange(nbo), axis] = sign[face] * dist
            boundnor[nbw:npb] = nvec.astype(np.float32)
    vel = np.zeros((n, 3), np.float32)
    if spec.init_vel and nf:
        rng = np.random.default_rng(spec.seed + 1)
        vel[npb:] = rng.uniform(-spec.init_vel, spec.init_vel, size=(nf, 3)).astype(np.float32)
    if spec.init_vel_x and nf:
        vel[npb:, 0] += np.float32(spec.init_vel_x)
    if spec.init_vel_y and nf:
        vel[npb:, 1] += np.float32(spec.init_vel_y)
    if spec.init_vel_z and nf:
        vel[npb:, 2] += np.float32(spec.init_vel_z)
    return Case(spec=spec, pos=pos, vel=vel, rhop=rhop.astype(np.float32),
                idp=np.arange(n, dtype=np.uint32), code=code, boundnor=boundnor, blocks=blocks,
                npb=npb, h=h, b=b, mass=mass)


def _fmt(v: float) -> str:
    return repr(float(v))


_ROT_SCALAR = {"vel": "ang", "ace": "ang", "velini": "ang", "freq": "v", "ampl": "v", "phase": "v"}


def _motion_xml(movements: list) -> list:
    """``case.execution.motion`` for moving object 0 (the tank walls)."""
    lines = ['    <motion>', '      <objreal ref="0">',
             f'        <begin mov="{int(movements[0]["id"])}" start="0" />']
    for m in movements:
        attrs = f'id="{int(m["id"])}"'
        if m["type"] != "mvnull":
            attrs += f' duration="{_fmt(m["duration"])}"'
            if m.get("next"):
                attrs += f' next="{int(m["next"])}"'
            if m.get("anglesunits"):
                attrs += f' anglesunits="{m["anglesunits"]}"'
        lines.append(f'        <{m["type"]} {attrs}>')
        for k, v in m.items():
            if k in ("type", "id", "duration", "next", "anglesunits"):
                continue
            if isinstance(v, (tuple, list)):
                lines.append(f'          <{k} x="{_fmt(v[0])}" y="{_fmt(v[1])}" z="{_fmt(v[2])}" />')
            else:
                lines.append(f'          <{k} {_ROT_SCALAR[k]}="{_fmt(v)}" />')
        lines.append(f'        </{m["type"]}>')
    lines += ['      </objreal>', '    </motion>']
    return lines


def write_case(case: Case, dirpath: str) -> tuple[str, str]:
    """Writes ``<name>.xml`` and ``<name>.bi4`` into ``dirpath``; returns their paths."""
    s = case.spec
    os.makedirs(dirpath, exist_ok=True)
    nf = case.np - case.npb
    nmoving = sum(c for k, _, _, c in case.blocks if k == "moving")
    params = {
        "SavePosDouble": 1, "StepAlgorithm": s.step_algorithm, "VerletSteps": s.verlet_steps,
        "Kernel": 2, "ViscoTreatment": s.visco_treatment, "Visco": s.visco,
        "ViscoBoundFactor": s.viscoboundfactor, "Boundary": 2 if s.boundary == "mdbc" else 1,
        "SlipMode": 1, "DensityDT": s.density_dt, "DensityDTvalue": s.density_dt_value,
        "Shifting": 0, "RigidAlgorithm": 1, "CoefDtMin": 0.05, "DtIni": 0, "DtMin": 0,
        "TimeMax": s.time_max, "TimeOut": s.time_out, "RhopOutMin": 700, "RhopOutMax": 1300,
    }
    if s.boundary != "mdbc":
        params.pop("SlipMode")
    if s.periodic_x:
        params["XPeriodicIncY"] = s.peri_inc_y
    if s.periodic_y:
        params["YPeriodicIncX"] = 0
    if s.periodic_z:
        params["ZPeriodicIncX"] = 0
    params.update(s.extra_params)
    lines = ['<?xml version="1.0" encoding="UTF-8" ?>',
             '<case app="dualsphysics_gb300.casegen">',
             '  <execution>',
             '    <parameters>']
    for k, v in params.items():
        lines.append(f'      <parameter key="{k}" value="{v}" />')
    lines += ['      <simulationdomain>',
              f'        <posmin x="{s.posmin_x}" y="default" z="default" />',
              f'        <posmax x="{s.posmax_x}" y="default" z="{s.posmax_z}" />',
              '      </simulationdomain>',
              '    </parameters>',
              '    <constants>',
              '      <data2d value="false" />',
              f'      <gravity x="{_fmt(s.gravity[0])}" y="{_fmt(s.gravity[1])}" z="{_fmt(s.gravity[2])}" />',
              f'      <cflnumber value="{_fmt(s.cflnumber)}" />',
              f'      <gamma value="{_fmt(s.gamma)}" />',
              f'      <rhop0 value="{_fmt(s.rhop0)}" />',
              f'      <dp value="{_fmt(s.dp)}" />',
              f'      <h value="{_fmt(case.h)}" />',
              f'      <b value="{_fmt(case.b)}" />',
              f'      <massbound value="{_fmt(case.mass)}" />',
              f'      <massfluid value="{_fmt(case.mass)}" />',
              '    </constants>',
              f'    <particles np="{case.np}" nb="{case.npb}" nbf="{case.npb - nmoving}" mkboundfirst="11" '
              'mkfluidfirst="1">']
    for kind, mk, begin, count in case.blocks:
        if kind == "fixed":
            lines.append(f'      <fixed mkbound="{mk}" mk="{11 + mk}" begin="{begin}" count="{count}" />')
        elif kind == "moving":
            lines.append(f'      <moving mkbound="{mk}" mk="{11 + mk}" begin="{begin}" count="{count}" '
                         'refmotion="0" />')
        else:
            lines.append(f'      <fluid mkfluid="{mk}" mk="{1 + mk}" begin="{begin}" count="{count}" />')
    lines += ['    </particles>']
    if s.motion:
        lines += _motion_xml(s.motion)
    lines += ['  </execution>', '</case>', '']
    xml_path = os.path.join(dirpath, s.name + ".xml")
    with open(xml_path, "w") as f:
        f.write("\n".join(lines))
    root = bi4.make_partdata_root(
        casename=s.name, appname="dualsphysics_gb300.casegen", data2d=False, casenp=case.np,
        casenfixed=case.npb - nmoving, casenmoving=nmoving, casenfloat=0, casenfluid=nf,
        caseposmin=case.pos.min(axis=0), caseposmax=case.pos.max(axis=0), dp=s.dp, h=case.h, b=case.b,
        rhop0=s.rhop0, gamma=s.gamma, massbound=case.mass, massfluid=case.mass)
    part = bi4.make_part(0, 0.0, case.np, 0, 0, case.pos.min(axis=0), case.pos.max(axis=0), case.idp, case.pos,
                         case.vel, case.rhop, posdouble=True,
                         boundnor=case.boundnor if s.boundary == "mdbc" else None)
    root.items.append(part)
    bi4_path = os.path.join(dirpath, s.name + ".bi4")
    bi4.write(bi4_path, root)
    return xml_path, bi4_path


# ---------------------------------------------------------------------------
# The dam-break workloads (the particle counts of the generated geometry are
# those the generator produces, counted after generation).
# ---------------------------------------------------------------------------
OBSTACLE_C2 = (0.9, 0.24, 0.12, 0.12, 0.45)


def spec_c1(dp: float = 0.01, **kw) -> CaseSpec:
    """3-D dam break, plain WCSPH with DBC walls (tank 1.6x0.67x0.4, column 0.4x0.67x0.3)."""
    return CaseSpec(name=kw.pop("name", "DamC1"), dp=dp, time_max=0.5, **kw)


def spec_c2(dp: float = 0.0025, **kw) -> CaseSpec:
    """Same dam break with mDBC boundaries and the 0.12x0.12x0.45 box obstacle at x=0.9 m."""
    return CaseSpec(name=kw.pop("name", "DamC2"), dp=dp, obstacle=OBSTACLE_C2, boundary="mdbc", time_max=1.0, **kw)


def spec_c3(dp: float = 0.004, column_height: float = 0.6, **kw) -> CaseSpec:
    """Dam-break geometry scaled x4 (tank 6.4x2.68x1.6) with a 1.6x2.68xH column."""
    return CaseSpec(name=kw.pop("name", "DamC3"), tank=(6.4, 2.68, 1.6), column=(1.6, 2.68, column_height),
                    dp=dp, hswl=0.3, **kw)


def spec_c5(dp: float = 0.02, **kw) -> CaseSpec:
    """C2 geometry at coarse resolution (the learned-closure workload)."""
    return spec_c2(dp=dp, name=kw.pop("name", "DamC5"), **kw)
