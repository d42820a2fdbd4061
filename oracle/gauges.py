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
