"""Independent FP64 adjoint of the reference algorithm, in numpy.

TEST INFRASTRUCTURE ONLY: the checker for the library's hand-written adjoint
kernels (imported by tests/ only).

The forward is the oracle (the C restatement of kernels.cl, push form): its
states R_0 .. R_T (what iterations 1 .. T+1 read) are stored, and the adjoint
of R_{k+1} = S C(R_k) is applied backwards, vectorised over the lattice:
    b_i(s) = a_{k+1}(s + e_i, i)            (0 when s + e_i is a wall)
    a_k(s) = J_C(R_k(s))^T b(s)            per site kind:
      FLUID   BGK:  a_j = (1-w) b_j + w sum_i b_i dfeq_i/dg_j,  dJ/dw += sum b (feq - g)
      MOVING  (kernels.cl:343-349, 393-398): out = feq(rho', lid), rho' over g with
              the five -z slots replaced by their opposites
      bounce-back (kernels.cl:400-408): a_j = b_opp(j);  CORNER: a = b;  WALL: 0
The loss is J = mean over the FLUID sites of plane y of (u_x(R_T) - target)^2.
"""
from __future__ import annotations

import numpy as np

from . import pyoracle as po

W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
E = np.stack([po.EX, po.EY, po.EZ], axis=1).astype(np.float64)  # [19, 3]


def _moments(g):
    rho = g.sum(0)
    j = np.einsum("ia,i...->a...", E, g)
    with np.errstate(invalid="ignore", divide="ignore"):  # walls hold zeros
        return rho, j / rho


def _feq(rho, u, lid_x=None):
    """w_i rho (1 + 3 e.u + 4.5 (e.u)^2 - 1.5 u^2) for fields u [3, ...]."""
    eu = np.einsum("ia,a...->i...", E, u)
    u2 = (u * u).sum(0)
    return W.reshape((19,) + (1,) * rho.ndim) * rho * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * u2)


def run(dim, viscosity, lid, tau, iterations, plane_y, target, f0=None, noise=0.0, seed=0):
    """Forward (oracle, FP64) + reference adjoint.  lid: dim*dim [x + y*dim];
    target: dim*dim [x + z*dim].  Returns (J, dJ/dtau, dJ/dlid [y, x], dJ/dR_0 [19, z, y, x])."""
    n = dim ** 3
    lid = np.asarray(lid, np.float64).reshape(-1)
    # the oracle takes the viscosity; tau = 3 nu + 0.5
    L = po.OracleLattice(dim, (tau - 0.5) / 3.0, 0.0, "f64", stride=8, lid=lid, seed=seed, noise_sigma=noise)
    if f0 is not None:
        raise NotImplementedError("explicit initial populations: use the init state")
    omega = 1.0 / (3.0 * ((tau - 0.5) / 3.0) + 0.5)
    states = [L.f_soa().copy()]
    for _ in range(iterations):
        L.step(1, every=0)
        states.append(L.f_soa().copy())
    ct = L.map.reshape(dim, dim, dim)
    wall = ct == po.WALL
    fluid = ct == po.FLUID
    moving = (ct & po.MOVING) != 0
    corner = ct == po.CORNER
    bounce = ~wall & ~fluid & ~moving & ~corner

    # loss and seed a_T
    RT = np.nan_to_num(states[-1])
    rhoT, uT = _moments(RT)
    tgt = np.asarray(target, np.float64).reshape(dim, dim)  # [z, x]
    onp = np.zeros((dim, dim, dim), bool)
    onp[:, plane_y, :] = True
    onp &= fluid
    M = onp.sum()
    diff = np.where(onp, uT[0] - tgt[:, None, :], 0.0)
    J = float((diff ** 2).sum() / M)
    a = np.zeros((19, dim, dim, dim))
    with np.errstate(invalid="ignore", divide="ignore"):
        for i in range(19):
            a[i] = np.where(onp, (2.0 / M) * diff * (E[i, 0] - uT[0]) / rhoT, 0.0)

    lidf = lid.reshape(dim, dim)  # [y, x]
    dw = 0.0
    glid = np.zeros((dim, dim))
    for k in range(iterations - 1, -1, -1):
        g = states[k].copy()
        # wall-sourced slots keep the reference's constants: replace NaN-free
        g = np.nan_to_num(g)
        # reverse streaming b_i(s) = a(s + e_i, i), zero outside / at walls
        b = np.zeros_like(a)
        for i in range(19):
            ex, ey, ez = int(po.EX[i]), int(po.EY[i]), int(po.EZ[i])
            src = a[i]
            sh = np.zeros_like(src)
            zs = slice(max(0, -ez), dim - max(0, ez))
            ys = slice(max(0, -ey), dim - max(0, ey))
            xs = slice(max(0, -ex), dim - max(0, ex))
            zd = slice(max(0, ez), dim - max(0, -ez))
            yd = slice(max(0, ey), dim - max(0, -ey))
            xd = slice(max(0, ex), dim - max(0, -ex))
            sh[zs, ys, xs] = src[zd, yd, xd]
            b[i] = sh
        out = np.zeros_like(b)
        # FLUID
        rho, u = _moments(g)
        feq = _feq(rho, u)
        eu = np.einsum("ia,a...->i...", E, u)
        B0 = (b * W.reshape(19, 1, 1, 1) * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * (u * u).sum(0))).sum(0)
        SB = (b * W.reshape(19, 1, 1, 1)).sum(0)
        G = np.einsum("i...,ia->a...", b * W.reshape(19, 1, 1, 1) * (3 + 9 * eu), E) - 3 * u * SB
        c = B0 - (G * u).sum(0)
        flu = (1 - omega) * b + omega * (c + np.einsum("a...,ia->i...", G, E))
        out = np.where(fluid, flu, out)
        dw += float(np.where(fluid, (b * (feq - g)).sum(0), 0.0).sum())
        # MOVING
        gp = g.copy()
        for i, j in ((5, 6), (11, 17), (12, 18), (13, 15), (14, 16)):
            gp[i] = g[j]
        rhop = gp.sum(0)
        lx = np.broadcast_to(lidf[None, :, :], (dim, dim, dim))
        ul = np.stack([lx, np.zeros_like(lx), np.zeros_like(lx)])
        eul = np.einsum("ia,a...->i...", E, ul)
        pl = 1 + 3 * eul + 4.5 * eul * eul - 1.5 * lx * lx
        s_ = (b * W.reshape(19, 1, 1, 1) * pl).sum(0)
        mult = np.ones(19)
        mult[[5, 11, 12, 13, 14]] = 0
        mult[[6, 15, 16, 17, 18]] = 2
        mov = mult.reshape(19, 1, 1, 1) * s_
        out = np.where(moving, mov, out)
        dl = (b * W.reshape(19, 1, 1, 1) * rhop * (3 * E[:, 0].reshape(19, 1, 1, 1)
                                                   + (9 * E[:, 0].reshape(19, 1, 1, 1) ** 2 - 3) * lx)).sum(0)
        glid += np.where(moving, dl, 0.0).sum(0)  # moving sites: one per (y, x) column
        # bounce-back and corners
        out = np.where(bounce, b[po.OPP], out)
        out = np.where(corner, b, out)
        a = out
    # the init state's lid dependence (FRONT sites start at the lid equilibrium)
    front = (ct & po.FRONT) != 0
    ex0 = E[:, 0].reshape(19, 1, 1, 1)
    lx = np.broadcast_to(lidf[None, :, :], (dim, dim, dim))
    dR0 = W.reshape(19, 1, 1, 1) * (3 * ex0 + (9 * ex0 ** 2 - 3) * lx)
    glid += np.where(front, (a * dR0).sum(0), 0.0).sum(0)
    return J, -omega * omega * dw, glid, a
