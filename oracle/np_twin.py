"""NumPy FP64 twin of the C oracle, written independently for cross-checking.

TEST INFRASTRUCTURE ONLY.  Vectorised restatement of src/mol.ml:796-903
(inter and intra sums), src/rot.ml:52-66 and 121-146, src/mol.ml:610-631 and
src/optim.ml:64-80 (UnixJunkie/MMO).
"""
from __future__ import annotations

import numpy as np

ELEC = 332.0637 / 4.0
UFF = {0: (0.0, 0.0), 1: (2.886, 0.044), 6: (3.851, 0.105), 7: (3.660, 0.069),
       8: (3.500, 0.060), 9: (3.364, 0.050), 12: (3.021, 0.111), 15: (4.147, 0.305),
       16: (4.035, 0.274), 17: (3.947, 0.227), 35: (4.189, 0.251), 53: (4.500, 0.339)}


def params(anum):
    xi = np.array([UFF[int(a)][0] for a in anum])
    di = np.array([UFF[int(a)][1] for a in anum])
    return xi, di


def pair_energy(r, qq, xij, dij, w, dielectric=0):
    p6 = (xij / r) ** 6
    el = qq / r if dielectric == 0 else qq / (r * r)
    return w * ELEC * el + w * dij * (p6 * p6 - 2.0 * p6)


def ene_inter(pxyz, pq, panum, lxyz, lq, lanum, shifted=True, mixing=0, dielectric=0,
              absolute=False):
    """Sum of pair energies, or of the absolute values of their parts
    (absolute=True: w (|elec| + D (x/r)^12 + 2 D (x/r)^6), the conditioning
    scale used by the parity tests)."""
    xp, dp = params(panum)
    xl, dl = params(lanum)
    d = np.linalg.norm(pxyz[:, None, :] - lxyz[None, :, :], axis=2)
    r = np.maximum(d, 0.01)
    xij = np.sqrt(xp[:, None] * xl[None, :]) if mixing == 0 else 0.5 * (xp[:, None] + xl[None, :])
    dij = np.sqrt(dp[:, None] * dl[None, :])
    if shifted:
        w = np.where(d * d < 144.0, (1.0 - (r / 12.0) ** 2) ** 2, 0.0)
    else:
        w = np.ones_like(r)
    e = pair_energy(r, pq[:, None] * lq[None, :], xij, dij, w, dielectric)
    if absolute:
        e = np.abs(w * ELEC * (pq[:, None] * lq[None, :]) / (r if dielectric == 0 else r * r)) + \
            np.abs(w * dij) * ((xij / r) ** 12 + 2.0 * (xij / r) ** 6)
    return float(e.sum())


def ene_intra(lxyz, lq, lanum, interacting, dielectric=0, absolute=False):
    xl, dl = params(lanum)
    n = lxyz.shape[0]
    iu = np.triu_indices(n, 1)
    mask = interacting[iu].astype(bool)
    i, j = iu[0][mask], iu[1][mask]
    r = np.maximum(np.linalg.norm(lxyz[i] - lxyz[j], axis=1), 0.01)
    xij, dij, qq = np.sqrt(xl[i] * xl[j]), np.sqrt(dl[i] * dl[j]), lq[i] * lq[j]
    if absolute:
        p6 = (xij / r) ** 6
        return float((np.abs(ELEC * qq / (r if dielectric == 0 else r * r)) +
                      np.abs(dij) * (p6 * p6 + 2.0 * p6)).sum())
    return float(pair_energy(r, qq, xij, dij, np.ones_like(r), dielectric).sum())


def rot_xyz(a, b, g):
    ca, sa, cb, sb, cg, sg = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(g), np.sin(g)
    Rx = np.array([[1, 0, 0], [0, ca, -sa], [0, sa, ca]])
    Ry = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
    Rz = np.array([[cg, -sg, 0], [sg, cg, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def axis_angle(u, th):
    K = np.array([[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]])
    return np.eye(3) * np.cos(th) + np.sin(th) * K + (1 - np.cos(th)) * np.outer(u, u)


def apply_config(xyz0, rbonds, rgroups, conf, recenter=False):
    xyz = np.array(xyz0, dtype=np.float64)
    for t, (left, right) in enumerate(rbonds):
        c = xyz[right].copy()
        a = c - xyz[left]
        R = axis_angle(a / np.linalg.norm(a), conf[6 + t])
        g = np.asarray(rgroups[t], int)
        xyz[g] = (xyz[g] - c) @ R.T + c
    if recenter:
        xyz = xyz - xyz.mean(axis=0)
    return xyz @ rot_xyz(conf[3], conf[4], conf[5]).T + np.asarray(conf[:3])
