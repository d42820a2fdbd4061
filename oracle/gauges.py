"""Oracle (test infrastructure only): numpy restatement of the reference's
measurement gauges -- JGaugeVelocity, JGaugeSwl, JGaugeMaxZ
(JDsGaugeItem.cpp:427-478, 614-641, 728-790, 1045-1087) -- on a particle
state.  Used only by tests/, as the checker of the GPU gauges; pinned against
the gauges the reference itself computes (tests/golden/*.npz, gauge_*).

Neighbours are found by brute force over all particles instead of the cell
search: the fluid particles within 2h of a point are exactly those the
reference reaches through the 27 cells around it, so only the order of the
double sums differs (last bits before the final rounding to float).
"""
from __future__ import annotations

import numpy as np

F = np.float32


def _wendland_wab(rr2: np.ndarray, awen: float, h: float) -> np.ndarray:
    """GetKernelWendland_Wab (FunSphKernel.h:213-220), in float."""
    rad = np.sqrt(rr2.astype(F))
    qq = (rad / F(h)).astype(F)
    wqq = (qq + qq + F(1)).astype(F)
    wqq1 = (F(1) - F(0.5) * qq).astype(F)
    wqq2 = (wqq1 * wqq1).astype(F)
    return (F(awen) * wqq * wqq2 * wqq2).astype(F)


def _rr2(point, pos: np.ndarray) -> np.ndarray:
    """nsearch::Distance2 (JCellSearch_inline.h:99-104): float of the double differences."""
    d = (np.asarray(point, np.float64)[None, :] - pos).astype(F)
    return (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]).astype(F)


def _fluid(code: np.ndarray) -> np.ndarray:
    return (code.astype(np.uint32) & 0x1800) == 0x1800


def _point_out(p, mapmin, mapmax) -> bool:
    """JGaugeItem::PointIsOut (JDsGaugeItem.h:223-227) with the map limits."""
    return any(v != v for v in p) or any(p[k] < mapmin[k] or p[k] >= mapmax[k] for k in range(3))


def gauge_velocity(point, pos, velrho, code, ctes, mapmin, mapmax) -> np.ndarray:
    """JGaugeVelocity::CalculeCpuT: sum of W*m/rho*v (no normalisation)."""
    if _point_out(point, mapmin, mapmax):
        return np.zeros(3, F)
    rr2 = _rr2(point, pos)
    sel = (rr2 <= F(ctes.kernelsize2)) & (rr2 >= F(1e-18)) & _fluid(code)
    wab = _wendland_wab(rr2[sel], ctes.awen, ctes.kernelh)
    wab = (wab * (F(ctes.massfluid) / velrho[sel, 3].astype(F)).astype(F)).astype(F)
    v = (wab[:, None] * velrho[sel, :3].astype(F)).astype(F).astype(np.float64)
    return v.sum(axis=0).astype(F)


def _mass(point, pos, velrho, code, ctes) -> np.float32:
    """JGaugeSwl::CalculeMassCpu: sum of W*m/rho*m (no normalisation)."""
    rr2 = _rr2(point, pos)
    sel = (rr2 <= F(ctes.kernelsize2)) & (rr2 >= F(1e-18)) & _fluid(code)
    wab = _wendland_wab(rr2[sel], ctes.awen, ctes.kernelh)
    wab = (wab * (F(ctes.massfluid) / velrho[sel, 3].astype(F)).astype(F)).astype(F)
    return F((wab * F(ctes.massfluid)).astype(F).astype(np.float64).sum())


def swl_points(p0, p2, pointdp):
    """JGaugeSwl::SetPoints (JDsGaugeItem.cpp:614-641): number of steps and step vector."""
    p0 = np.asarray(p0, np.float64)
    p2 = np.asarray(p2, np.float64)
    v = p0 - p2
    dis = float(np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]))
    if dis > 0 and pointdp > 0:
        n = int(dis / pointdp)
        if dis - (pointdp * n) >= pointdp * 0.1:
            n += 1
        if n < 1:
            n += 1
        dp = dis / n
        u = p2 - p0
        m = float(np.sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]))
        d = (np.array([u[0] / m, u[1] / m, u[2] / m]) if m else u) * dp
        return n, d
    return 0, np.zeros(3)


def gauge_swl(p0, p2, pointdp, masslimit, pos, velrho, code, ctes) -> np.ndarray:
    """JGaugeSwl::CalculeCpuT: first crossing of the mass limit going from p0 to p2
    (default limit: JGaugeSystem::AddGaugeSwl, JDsGaugeSystem.cpp:408)."""
    ml = F(masslimit) if masslimit > 0 else F(F(ctes.massfluid) * F(0.4 if ctes.simulate2d else 0.5))
    n, d = swl_points(p0, p2, pointdp)
    p0 = np.asarray(p0, np.float64)
    ptsurf = None
    mpre = F(0)
    pt = p0.copy()
    for _ in range(n + 1):
        mass = _mass(pt, pos, velrho, code, ctes)
        if mass > ml:
            mpre = mass
        if mass < ml and mpre:
            fxm1 = F(F(F(ml - mpre) / F(mass - mpre)) - F(1))
            ptsurf = pt + d * float(fxm1)
            break
        pt = pt + d
    if ptsurf is None:
        ptsurf = p0 + d * float(n if mpre else 0)
    return ptsurf.astype(F)


def gauge_maxz(p0, height, distlimit, pos, code, mapmin_z) -> np.float32:
    """JGaugeMaxZ::CalculeCpu: highest fluid particle within distlimit of the
    vertical line through p0 (the column of cells from p0.z to p0.z+height,
    widened by the search radius, holds every candidate here)."""
    d = (np.asarray(p0, np.float64)[None, :2] - pos[:, :2]).astype(F)
    rr2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(F)
    sel = (rr2 <= F(F(distlimit) * F(distlimit))) & _fluid(code)
    zmax = F(pos[sel, 2].max()) if sel.any() else F(-np.finfo(np.float32).max)
    return max(zmax, F(mapmin_z))


# ---- mesh gauge ---------------------------------------------------------------
def _vec_unitary(v):
    """fgeo::VecUnitary for tdouble3 (FunGeo3d.h:293-296)."""
    v = np.asarray(v, np.float64)
    m = float(np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]))
    return np.array([v[0] / m, v[1] / m, v[2] / m]) if m else v


def _vec_unitary_f(v):
    """fgeo::VecUnitary for tfloat3 (FunGeo3d.h:302-305), in float."""
    v = np.asarray(v, np.float32)
    m = F(np.sqrt(F(F(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])))
    return np.array([v[0] / m, v[1] / m, v[2] / m], np.float32) if m else v


def mesh_points(mb):
    """JMeshData::MakeMeshPt (JMeshData.cpp:474-503).  mb: 24 parameters
    (ptref, vec1, vec2, vec3, dis1..3, dispt1..3, dirdat, ...).  Returns
    (ptref, [vdp1, vdp2, vdp3], [npt1, npt2, npt3], dirdat)."""
    mb = [float(x) for x in mb]
    vdp, npt = [], []
    for a in range(3):
        vec = np.array(mb[3 + 3 * a:6 + 3 * a])
        dis, dispt = mb[12 + a], mb[15 + a]
        if vec.any() and dispt > 0 and dis >= dispt:
            vdp.append(_vec_unitary(vec) * dispt)
            npt.append(int((dis + dispt * 0.01) / dispt) + 1)
        else:
            vdp.append(np.zeros(3))
            npt.append(1)
    return np.array(mb[0:3]), vdp, npt, _vec_unitary_f(_vec_unitary_f(mb[18:21]))


def _ordered_candidates(pt, div, c) -> np.ndarray:
    """Particle indices nsearch::Init(pos)/ParticleRange visit for a point, in
    their order: z, then y, then the x run of cells (JCellSearch_inline.h:43-68)."""
    sd = int(div["scelldiv"])
    nc = (int(div["ncx"]), int(div["ncy"]), int(div["ncz"]))
    cel = []
    for k in range(3):
        q = (float(pt[k]) - float(c.domposmin[k])) / float(np.float32(c.scell))
        cel.append(int(q) - int(div["cellmin"][k]))
    lo, hi = [], []
    for k in range(3):
        ck = cel[k]
        lo.append(ck - (ck if ck < sd else sd))
        hi.append(ck + ((nc[k] - ck - 1) if nc[k] - ck - 1 < sd else sd) + 1)
    if not (lo[0] < hi[0]):
        return np.zeros(0, np.int64)
    bc = div["begincell"]
    idx = []
    for z in range(lo[2], hi[2]):
        for y in range(lo[1], hi[1]):
            v = int(div["nsheet"]) * z + nc[0] * y + int(div["cellfluid"])
            a, b = int(bc[v + lo[0]]), int(bc[v + hi[0]])
            if b > a:
                idx.append(np.arange(a, b))
    return np.concatenate(idx) if idx else np.zeros(0, np.int64)


def _serial_sum(x: np.ndarray) -> np.float32:
    """Sum in float32 one term after another from 0 (the reference's loop)."""
    return np.add.accumulate(x.astype(F), dtype=F)[-1] if len(x) else F(0)


def gauge_mesh(mb, kclimit, kcdummy, masslimit, pos, velrho, code, div, c):
    """JGaugeMesh::CalculeCpuT (JDsGaugeItem.cpp:1484-1596) on a divided state
    (pos/velrho/code in cell order, div: ncx, ncy, ncz, nsheet, cellmin,
    cellfluid, scelldiv, begincell).  Float sums one term after another in the
    reference's cell order; the reference itself is compiled with -ffast-math,
    which lets the compiler reassociate them, so the two agree to a few float
    ulps of the sums' scale (also returned: S_vel = sum |w*v| per component,
    S_rho = sum w*rho, each divided by sum w where the kernel correction
    applies).  Returns vel (npt,3), veldir, rhop, mass (npt), zsurf
    (npt1*npt2), S_vel (npt,3), S_rho (npt)."""
    ptref, vdp, npt, vdir = mesh_points(mb)
    n1, n2, n3 = npt
    n12, n = n1 * n2, n1 * n2 * n3
    ml = F(masslimit) if masslimit > 0 else F(F(c.massfluid) * F(0.4 if c.simulate2d else 0.5))
    fmax = F(np.finfo(np.float32).max)
    kcl, kcd = F(kclimit), F(kcdummy)
    massf = F(c.massfluid)
    vel = np.zeros((n, 3), F)
    vdd = np.zeros(n, F)
    rho = np.zeros(n, F)
    mass = np.zeros(n, F)
    s_vel = np.zeros((n, 3))
    s_rho = np.zeros(n)
    fl = _fluid(code)
    for cp in range(n):
        cp3, r = divmod(cp, n12)
        cp2, cp1 = divmod(r, n1)
        pt = ((ptref + vdp[0] * float(cp1)) + vdp[1] * float(cp2)) + vdp[2] * float(cp3)
        cand = _ordered_candidates(pt, div, c)
        rr2 = _rr2(pt, pos[cand]) if len(cand) else np.zeros(0, F)
        sel = cand[(rr2 <= F(c.kernelsize2)) & fl[cand]]
        rr2 = rr2[(rr2 <= F(c.kernelsize2)) & fl[cand]]
        w = _wendland_wab(rr2, c.awen, c.kernelh)
        vr = velrho[sel].astype(F)
        w = (w * (massf / vr[:, 3]).astype(F)).astype(F)
        swab = _serial_sum(w)
        smass = _serial_sum((w * massf).astype(F))
        srho = _serial_sum((w * vr[:, 3]).astype(F))
        sv = np.array([_serial_sum((w * vr[:, k]).astype(F)) for k in range(3)], F)
        s_vel[cp] = [float(np.abs(w.astype(np.float64) * vr[:, k]).sum()) for k in range(3)]
        s_rho[cp] = float((w.astype(np.float64) * vr[:, 3]).sum())
        if kcl != fmax:
            if swab >= kcl:
                sv = (sv / swab).astype(F)
                srho = F(srho / swab)
                s_vel[cp] /= float(swab)
                s_rho[cp] /= float(swab)
            elif kcd != fmax:
                sv = np.array([kcd, kcd, kcd], F)
                srho = kcd
                s_vel[cp] = 0.0
                s_rho[cp] = 0.0
        vel[cp] = sv
        vdd[cp] = F(F(F(sv[0] * vdir[0]) + F(sv[1] * vdir[1])) + F(sv[2] * vdir[2]))
        rho[cp] = srho
        mass[cp] = smass
    zs = np.zeros(n12, F)
    for cp2 in range(n2):
        for cp1 in range(n1):
            masspre, cpsurf, fsurf = F(0), 0, F(0)
            cp = cp1 + cp2 * n1
            for cp3 in range(n3):
                if cpsurf:
                    break
                m = mass[cp]
                if m > ml:
                    masspre = m
                if m < ml and masspre:
                    fsurf = F(F(ml - masspre) / F(m - masspre))
                    cpsurf = cp3
                cp += n12
            z = F(ptref[2] + vdp[0][2] * cp1 + vdp[1][2] * cp2)
            if cpsurf == 0 and masspre:
                z = F(z + F(vdp[2][2] * (n3 - 1)))
            if cpsurf:
                z = F(z + F(vdp[2][2] * (cpsurf - 1) + vdp[2][2] * float(fsurf)))
            zs[cp1 + cp2 * n1] = z
    return vel, vdd, rho, mass, zs, s_vel, s_rho
