"""Oracle of the learned closure (test infrastructure only: tests/ import it
as the checker; the product never does).

FP64 NumPy restatement of what gbsph_closure.cu computes:
* the MLP 16-64-64-64-3 (tanh hidden layers, linear output) on the flat
  parameter vector W0[64][16] b0 W1[64][64] b1 W2[64][64] b2 W3[3][64] b3,
  its loss mean((y - t)^2) and the gradient of that loss by backpropagation;
* the closure features of the fluid rows by a brute-force pair loop (the
  same definitions: Wendland C2 W and grad W of the case, V_j = m_j/rho_j,
  pressure from the Tait equation of state).
The gradient restatement is itself pinned by central finite differences.
"""
from __future__ import annotations

import numpy as np

NF, NH, NO = 16, 64, 3


def unpack(p: np.ndarray):
    p = np.asarray(p, np.float64)
    o, out = 0, []
    for nin, nout in ((NF, NH), (NH, NH), (NH, NH), (NH, NO)):
        w = p[o:o + nin * nout].reshape(nout, nin)
        o += nin * nout
        b = p[o:o + nout]
        o += nout
        out.append((w, b))
    assert o == p.size
    return out


def forward(p, x):
    layers = unpack(p)
    hs = [np.asarray(x, np.float64)]
    for k, (w, b) in enumerate(layers):
        a = hs[-1] @ w.T + b
        hs.append(np.tanh(a) if k < 3 else a)
    return hs


def loss_and_grad(p, x, t):
    layers = unpack(p)
    hs = forward(p, x)
    y = hs[-1]
    n = x.shape[0]
    e = y - np.asarray(t, np.float64)
    loss = float(np.mean(e * e))
    d = 2.0 * e / (NO * n)
    grads = []
    for k in range(3, -1, -1):
        w, _ = layers[k]
        grads.append((d.T @ hs[k], d.sum(axis=0)))
        if k > 0:
            d = (d @ w) * (1.0 - hs[k] ** 2)
    g = []
    for gw, gb in reversed(grads):
        g.append(gw.ravel())
        g.append(gb)
    return loss, np.concatenate(g)


def features(pos, velrho, npb, ctes, press):
    """Closure features of rows npb.. by brute force (FP64).  pos (n,3),
    velrho (n,4), press (n,) pressure of every particle, ctes with kernelh,
    kernelsize2, awen, bwenh, massfluid, massbound, rhopzero, cs0, gravity."""
    pos = np.asarray(pos, np.float64)
    vr = np.asarray(velrho, np.float64)
    h = float(ctes.kernelh)
    ks2 = float(ctes.kernelsize2)
    g = float(np.linalg.norm(np.asarray(ctes.gravity[:], np.float64)))
    mass = np.where(np.arange(len(pos)) < npb, float(ctes.massbound), float(ctes.massfluid))
    out = np.zeros((len(pos) - npb, NF))
    for r, i in enumerate(range(npb, len(pos))):
        dr = pos[i] - pos
        rr2 = np.einsum("ij,ij->i", dr, dr)
        nb = (rr2 <= ks2) & (rr2 >= 1e-18)
        q = np.sqrt(rr2[nb]) / h
        w1 = 1.0 - 0.5 * q
        w = float(ctes.awen) * (2.0 * q + 1.0) * w1 ** 4
        fac = float(ctes.bwenh) * w1 ** 3
        vj = mass[nb] / vr[nb, 3]
        vw = vj * w
        shep = float(ctes.massfluid) / vr[i, 3] * float(ctes.awen) + vw.sum()
        sb = vw[np.nonzero(nb)[0] < npb].sum()
        dv = (vw[:, None] * (vr[nb, :3] - vr[i, :3])).sum(axis=0)
        gp = ((vj * (press[nb] - press[i]) * fac)[:, None] * dr[nb]).sum(axis=0)
        divr = -(vj * fac * rr2[nb]).sum()
        f = out[r]
        f[0] = (vr[i, 3] / float(ctes.rhopzero) - 1.0) * 50.0
        f[1:4] = dv / shep / (0.1 * float(ctes.cs0))
        f[4:7] = gp / (g * float(ctes.rhopzero))
        f[7] = shep - 1.0
        f[8] = divr - 3.0
        f[12] = sb
    return out
