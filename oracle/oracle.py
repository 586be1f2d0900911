"""ctypes front end of the FP64 C oracle (uff_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg, never by the mmo_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

F_INTER, F_INTRA, F_RECENTER = 1, 2, 8
S_TOO_LONG, S_NONFINITE = 1, 2


class Physics(C.Structure):
    _fields_ = [("dielectric", C.c_int), ("mixing", C.c_int), ("inter_form", C.c_int),
                ("intra_form", C.c_int)]


class CMol(C.Structure):
    _fields_ = [("n", C.c_int), ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("z", C.POINTER(C.c_double)), ("q", C.POINTER(C.c_double)),
                ("anum", C.POINTER(C.c_int))]


class Lattice(C.Structure):
    _fields_ = [("step", C.c_double), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("o", C.c_double * 3)]


def lattice(step, dims, origin) -> Lattice:
    g = Lattice()
    g.step = float(step)
    g.nx, g.ny, g.nz = (int(v) for v in dims)
    g.o[:] = [float(v) for v in origin]
    return g


class MCParams(C.Structure):
    _fields_ = [("kT", C.c_double), ("rot", C.c_double), ("trans", C.c_double),
                ("tors", C.c_double), ("law", C.c_int), ("adapt", C.c_int),
                ("flip_every", C.c_int), ("seed", C.c_uint64), ("roi_c", C.c_double * 3),
                ("roi_r", C.c_double), ("reset_zero", C.c_int), ("too_long_ends", C.c_int)]


class MCStats(C.Structure):
    _fields_ = [("proposals", C.c_long), ("proposal_mismatch", C.c_long),
                ("decisions", C.c_long), ("decision_mismatch", C.c_long),
                ("ambiguous", C.c_long), ("resets", C.c_long), ("adapt_events", C.c_long),
                ("max_rel_err_E", C.c_double)]


class CLigand(C.Structure):
    _fields_ = [("m", CMol), ("interacting", C.POINTER(C.c_uint8)), ("nrb", C.c_int),
                ("bond_lr", C.POINTER(C.c_int)), ("grp_off", C.POINTER(C.c_int)),
                ("grp_atoms", C.POINTER(C.c_int))]


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(
                os.path.join(HERE, "uff_oracle.c")):
            build()
        L = C.CDLL(LIB)
        P = C.POINTER
        d, i, v = C.c_double, C.c_int, None
        sig = {
            "orc_elec_weight": (d, []),
            "orc_uff_params": (i, [i, P(d), P(d)]),
            "orc_pair_params": (v, [P(Physics), i, i, P(d), P(d)]),
            "orc_shift_12A": (d, [d]),
            "orc_non_zero_dist": (d, [d]),
            "orc_dihedral": (d, [P(d), P(d), P(d), P(d)]),
            "orc_rot_xyz": (v, [d, d, d, P(d)]),
            "orc_rot_axis_angle": (v, [P(d), d, P(d)]),
            "orc_rotate_bond": (v, [i, P(d), P(d), P(d), i, i, P(i), i, d]),
            "orc_ene_inter": (d, [P(Physics), P(CMol), P(CMol)]),
            "orc_ene_inter_parts": (v, [P(Physics), P(CMol), P(CMol), P(d)]),
            "orc_ene_intra": (d, [P(Physics), P(CMol), P(C.c_uint8)]),
            "orc_cells_build": (C.c_void_p, [P(CMol)]),
            "orc_cells_free": (v, [C.c_void_p]),
            "orc_ene_inter_cells": (d, [P(Physics), C.c_void_p, P(CMol)]),
            "orc_apply_config": (i, [P(CLigand), P(d), i, P(d), P(d), P(d)]),
            "orc_score_conf": (d, [P(Physics), P(CMol), C.c_void_p, P(CLigand), P(d), i, P(i)]),
            "orc_grad_fd": (v, [P(Physics), P(CMol), C.c_void_p, P(CLigand), P(d), i, P(d),
                                P(d)]),
            "orc_grad_analytic": (d, [P(Physics), P(CMol), P(CLigand), P(d), i, P(d), P(d),
                                      P(i)]),
            "orc_grad_scale": (d, [P(Physics), P(CMol), P(CLigand), P(d), i, P(d)]),
            "orc_mc_replay": (v, [P(Physics), P(CMol), P(CLigand), P(MCParams), i,
                                  P(C.c_float), i, P(C.c_float), P(d), P(C.c_int), d, i,
                                  P(MCStats)]),
            "orc_mc_run": (v, [P(Physics), P(CMol), P(CLigand), P(MCParams), i, P(C.c_float),
                               i, P(C.c_float), P(d), P(C.c_int), i, P(MCStats)]),
            "orc_score_batch": (v, [P(Physics), P(CMol), P(CLigand), i, P(C.c_float), i, i,
                                    P(d), i, i, P(d), P(d), P(i)]),
            "orc_grid_point": (v, [P(Physics), P(CMol), P(d), i, P(i), P(d), d, P(d)]),
            "orc_grid_points": (v, [P(Physics), P(CMol), i, P(d), i, P(i), P(d), d, i, P(d),
                                    P(d)]),
            "orc_trilin": (d, [d, i, i, i, P(C.c_float), P(d), P(i)]),
            "orc_vdw_radius": (d, [i]),
            "orc_clash2": (d, [i, i]),
            "orc_masks": (v, [P(Lattice), i, P(d), P(d), P(d), P(d), d, P(C.c_uint8),
                              P(C.c_uint8)]),
            "orc_clash_or": (i, [P(Lattice), P(C.c_uint8), P(d)]),
            "orc_clash_and": (i, [P(Lattice), P(C.c_uint8), P(d)]),
            "orc_protein_ligand_clash": (i, [P(Lattice), P(C.c_uint8), i, P(d), P(d), P(d)]),
            "orc_center_occupied": (i, [i, P(d), P(d), P(d), P(d)]),
            "orc_heavy_atom_clash": (i, [P(CMol), i, P(d), P(d), P(d), P(i)]),
            "orc_intra_clash": (i, [i, P(d), P(d), P(d), P(i), P(C.c_uint8)]),
            "orc_so3_rotation": (v, [i, i, P(d)]),
            "orc_dock_scores": (v, [P(Lattice), P(C.c_float), P(C.c_uint8), P(CMol), P(i), P(d),
                                    P(d), d, d, i, P(d), d, P(i), P(d)]),
            "orc_desolv_constant": (d, []),
            "orc_protein_desolv": (v, [P(Lattice), P(CMol), P(C.c_uint8), P(d), d, P(d)]),
            "orc_desolvation_penalty": (v, [P(Lattice), P(d), P(C.c_uint8), i, P(d), P(d), P(d),
                                            P(d), P(d), d, P(d)]),
            "orc_ene_inter_interp": (d, [d, i, i, i, P(C.c_float), i, P(d), P(d), P(d), P(i),
                                         P(i)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def physics(dielectric=0, mixing=0, inter_form=0, intra_form=0) -> Physics:
    return Physics(dielectric, mixing, inter_form, intra_form)


REF = physics()


class OMol:
    """Keeps the numpy buffers of a CMol alive."""

    def __init__(self, x, y, z, q, anum):
        self.arrs = [np.ascontiguousarray(a, np.float64) for a in (x, y, z, q)]
        self.anum = np.ascontiguousarray(anum, np.int32)
        self.c = CMol(len(self.anum), *(_dp(a) for a in self.arrs), _ip(self.anum))

    @classmethod
    def of(cls, m, xyz=None):
        if xyz is None:
            return cls(m.x, m.y, m.z, m.q, m.anum)
        xyz = np.asarray(xyz, np.float64)
        return cls(xyz[:, 0], xyz[:, 1], xyz[:, 2], m.q, m.anum)


class OLigand:
    def __init__(self, m):
        self.mol = OMol.of(m)
        self.inter = np.ascontiguousarray(m.interacting, np.uint8)
        self.bonds = np.ascontiguousarray(m.rbonds.reshape(-1), np.int32)
        off, atoms = m.group_arrays()
        self.off = np.ascontiguousarray(off, np.int32)
        self.atoms = np.ascontiguousarray(atoms if atoms.size else np.zeros(1, np.int32), np.int32)
        self.nrb = m.nrb
        self.c = CLigand(self.mol.c, self.inter.ctypes.data_as(C.POINTER(C.c_uint8)), m.nrb,
                         _ip(self.bonds if self.bonds.size else np.zeros(1, np.int32)),
                         _ip(self.off), _ip(self.atoms))
        self._keep = [self.bonds]


def elec_weight() -> float:
    return lib().orc_elec_weight()


def pair_params(a1, a2, ph=REF):
    xo, do = C.c_double(), C.c_double()
    lib().orc_pair_params(C.byref(ph), a1, a2, C.byref(xo), C.byref(do))
    return xo.value, do.value


def shift_12A(d):
    return lib().orc_shift_12A(d)


def non_zero_dist(d):
    return lib().orc_non_zero_dist(d)


def dihedral(i, j, k, l):
    arrs = [np.ascontiguousarray(v, np.float64) for v in (i, j, k, l)]
    return lib().orc_dihedral(*(_dp(a) for a in arrs))


def rot_xyz(a, b, g):
    R = np.zeros(9)
    lib().orc_rot_xyz(a, b, g, _dp(R))
    return R.reshape(3, 3)


def rotate_bond(xyz, left, right, group, alpha):
    xyz = np.asarray(xyz, np.float64)
    x, y, z = (np.ascontiguousarray(xyz[:, d]) for d in range(3))
    g = np.ascontiguousarray(group, np.int32)
    lib().orc_rotate_bond(len(x), _dp(x), _dp(y), _dp(z), left, right,
                          _ip(g if g.size else np.zeros(1, np.int32)), len(g), alpha)
    return np.stack([x, y, z], axis=1)


def ene_inter(prot, lig, xyz=None, ph=REF):
    p, l = OMol.of(prot), OMol.of(lig, xyz)
    return lib().orc_ene_inter(C.byref(ph), C.byref(p.c), C.byref(l.c))


def ene_inter_parts(prot, lig, xyz=None, ph=REF):
    p, l = OMol.of(prot), OMol.of(lig, xyz)
    out = np.zeros(2)
    lib().orc_ene_inter_parts(C.byref(ph), C.byref(p.c), C.byref(l.c), _dp(out))
    return out


def ene_inter_cells(prot, lig, xyz=None, ph=REF):
    p, l = OMol.of(prot), OMol.of(lig, xyz)
    cells = lib().orc_cells_build(C.byref(p.c))
    try:
        return lib().orc_ene_inter_cells(C.byref(ph), cells, C.byref(l.c))
    finally:
        lib().orc_cells_free(cells)


def ene_intra(lig, xyz=None, ph=REF):
    l = OMol.of(lig, xyz)
    inter = np.ascontiguousarray(lig.interacting, np.uint8)
    return lib().orc_ene_intra(C.byref(ph), C.byref(l.c),
                               inter.ctypes.data_as(C.POINTER(C.c_uint8)))


def apply_config(lig, conf, flags=0):
    L = OLigand(lig)
    conf = np.ascontiguousarray(conf, np.float64)
    x, y, z = np.zeros(lig.n), np.zeros(lig.n), np.zeros(lig.n)
    st = lib().orc_apply_config(C.byref(L.c), _dp(conf), flags, _dp(x), _dp(y), _dp(z))
    return np.stack([x, y, z], axis=1), st


def score_conf(prot, lig, conf, flags=F_INTER | F_INTRA, ph=REF):
    p, L = OMol.of(prot), OLigand(lig)
    conf = np.ascontiguousarray(conf, np.float64)
    st = C.c_int()
    e = lib().orc_score_conf(C.byref(ph), C.byref(p.c), None, C.byref(L.c), _dp(conf), flags,
                             C.byref(st))
    return e, st.value


def grad_fd(prot, lig, conf, eps, flags=F_INTER | F_INTRA, ph=REF):
    p, L = OMol.of(prot), OLigand(lig)
    conf = np.ascontiguousarray(conf, np.float64)
    eps = np.ascontiguousarray(np.broadcast_to(eps, conf.shape), np.float64)
    g = np.zeros_like(conf)
    lib().orc_grad_fd(C.byref(ph), C.byref(p.c), None, C.byref(L.c), _dp(conf), flags, _dp(eps),
                      _dp(g))
    return g


def grad_analytic(prot, lig, conf, flags=F_INTER | F_INTRA, ph=REF, want_xyz=False):
    p, L = OMol.of(prot), OLigand(lig)
    conf = np.ascontiguousarray(conf, np.float64)
    g = np.zeros_like(conf)
    gx = np.zeros(3 * lig.n)
    st = C.c_int()
    e = lib().orc_grad_analytic(C.byref(ph), C.byref(p.c), C.byref(L.c), _dp(conf), flags,
                                _dp(g), _dp(gx), C.byref(st))
    if want_xyz:
        return e, g, gx.reshape(-1, 3), st.value
    return e, g, st.value


def _mc_params(params: dict) -> MCParams:
    mp = MCParams()
    for k, v in params.items():
        if k == "roi_c":
            mp.roi_c[:] = [float(x) for x in v]
        else:
            setattr(mp, k, v)
    return mp


def mc_run(prot, lig, params: dict, start, steps, nthreads=16, ph=REF):
    """The oracle's own run of the chains (orc_mc_run): (trial [steps, B, nd],
    E [steps, B], event [steps, B], stats)."""
    p, L = OMol.of(prot), OLigand(lig)
    start = np.ascontiguousarray(start, np.float32)
    B, nd = start.shape
    trial = np.zeros((steps, B, nd), np.float32)
    E = np.zeros((steps, B))
    event = np.zeros((steps, B), np.int32)
    st = MCStats()
    f = C.POINTER(C.c_float)
    lib().orc_mc_run(C.byref(ph), C.byref(p.c), C.byref(L.c), C.byref(_mc_params(params)), B,
                     start.ctypes.data_as(f), steps, trial.ctypes.data_as(f), _dp(E),
                     event.ctypes.data_as(C.POINTER(C.c_int)), nthreads, C.byref(st))
    return trial, E, event, {k: getattr(st, k) for k, _ in MCStats._fields_}


def mc_replay(prot, lig, params: dict, start, trial, E, event, e_tol=1e-5, nthreads=16,
              ph=REF) -> dict:
    """Replay of a GPU Monte Carlo trace (orc_mc_replay): start [B, nd] float32,
    trial [steps, B, nd] float32, E [steps, B], event [steps, B]."""
    p, L = OMol.of(prot), OLigand(lig)
    start = np.ascontiguousarray(start, np.float32)
    trial = np.ascontiguousarray(trial, np.float32)
    E = np.ascontiguousarray(E, np.float64)
    event = np.ascontiguousarray(event, np.int32)
    steps, B = E.shape
    mp = _mc_params(params)
    st = MCStats()
    f = C.POINTER(C.c_float)
    lib().orc_mc_replay(C.byref(ph), C.byref(p.c), C.byref(L.c), C.byref(mp), B,
                        start.ctypes.data_as(f), steps, trial.ctypes.data_as(f), _dp(E),
                        event.ctypes.data_as(C.POINTER(C.c_int)), e_tol, nthreads,
                        C.byref(st))
    return {k: getattr(st, k) for k, _ in MCStats._fields_}


def grad_scale(prot, lig, conf, flags=F_INTER | F_INTRA, ph=REF):
    """(S, grad_abs): the condition scales of the energy and of each analytic
    gradient component of one configuration (orc_grad_scale)."""
    p, L = OMol.of(prot), OLigand(lig)
    conf = np.ascontiguousarray(conf, np.float64)
    g = np.zeros_like(conf)
    S = lib().orc_grad_scale(C.byref(ph), C.byref(p.c), C.byref(L.c), _dp(conf), flags, _dp(g))
    return S, g


def score_batch(prot, lig, dofs, flags=F_INTER | F_INTRA, mode=0, eps=None, use_cells=False,
                nthreads=1, ph=REF):
    """mode 0: energy; 1: + analytic gradient; 2: + central differences;
    3: condition scales (E = sum of |pair energies|, G = per-component sums of
    |terms| of the analytic gradient)."""
    p, L = OMol.of(prot), OLigand(lig)
    dofs = np.ascontiguousarray(dofs, np.float32)
    B, nd = dofs.shape
    E = np.zeros(B)
    G = np.zeros((B, nd)) if mode else None
    st = np.zeros(B, np.int32)
    eps_a = np.ascontiguousarray(np.broadcast_to(eps if eps is not None else 1e-4, (nd,)),
                                 np.float64)
    lib().orc_score_batch(C.byref(ph), C.byref(p.c), C.byref(L.c), B,
                          dofs.ctypes.data_as(C.POINTER(C.c_float)), flags, mode, _dp(eps_a),
                          int(use_cells), nthreads, _dp(E), _dp(G) if G is not None else None,
                          _ip(st))
    return E, G, st


def grid_point(prot, p, type_anum, type_q, max_E=100000.0, ph=REF):
    """Grid values of Lds.pre_calculate_FF_components_grid at point p (one per type)."""
    P = OMol.of(prot)
    ta = np.ascontiguousarray(type_anum, np.int32)
    tq = np.ascontiguousarray(type_q, np.float64)
    out = np.zeros(len(ta))
    pp = np.ascontiguousarray(p, np.float64)
    lib().orc_grid_point(C.byref(ph), C.byref(P.c), _dp(pp), len(ta), _ip(ta), _dp(tq),
                         C.c_double(max_E), _dp(out))
    return out


def grid_points(prot, pts, type_anum, type_q, max_E=100000.0, nthreads=1, ph=REF,
                with_scale=False):
    """grid_point at many points (cell list, threads): float64 [n, ntypes]
    (and the sum of |pair terms| of each value with with_scale)."""
    P = OMol.of(prot)
    ta = np.ascontiguousarray(type_anum, np.int32)
    tq = np.ascontiguousarray(type_q, np.float64)
    pp = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
    out = np.zeros((len(pp), len(ta)))
    sc = np.zeros_like(out) if with_scale else None
    lib().orc_grid_points(C.byref(ph), C.byref(P.c), len(pp), _dp(pp), len(ta), _ip(ta),
                          _dp(tq), C.c_double(max_E), int(nthreads), _dp(out),
                          _dp(sc) if sc is not None else None)
    return (out, sc) if with_scale else out


def trilin(step, dims, values, p):
    """G3D.trilin on float32 values [nz][ny][nx] (x fastest); (value, off-lattice)."""
    v = np.ascontiguousarray(values, np.float32)
    pp = np.ascontiguousarray(p, np.float64)
    off = C.c_int(0)
    f = lib().orc_trilin
    e = f(C.c_double(step), dims[0], dims[1], dims[2], v.ctypes.data_as(C.POINTER(C.c_float)),
          _dp(pp), C.byref(off))
    return e, bool(off.value)


def ene_inter_interp(step, dims, grids, xyz, types):
    """Mol.ene_inter_UFF_interp: grids float32 [ntypes][nz][ny][nx], xyz in the
    lattice frame; (energy, off-lattice)."""
    g = np.ascontiguousarray(grids, np.float32)
    xyz = np.asarray(xyz, np.float64)
    x, y, z = (np.ascontiguousarray(xyz[:, k]) for k in range(3))
    t = np.ascontiguousarray(types, np.int32)
    off = C.c_int(0)
    f = lib().orc_ene_inter_interp
    e = f(C.c_double(step), dims[0], dims[1], dims[2], g.ctypes.data_as(C.POINTER(C.c_float)),
          len(t), _dp(x), _dp(y), _dp(z), _ip(t), C.byref(off))
    return e, bool(off.value)


def _u8(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def _xyz(xyz):
    xyz = np.asarray(xyz, np.float64).reshape(-1, 3)
    return [np.ascontiguousarray(xyz[:, k]) for k in range(3)]


def vdw_radius(anum) -> float:
    return lib().orc_vdw_radius(int(anum))


def clash2(a1, a2) -> float:
    return lib().orc_clash2(int(a1), int(a2))


def masks(g: Lattice, xyz, radius, r_w=1.4):
    """(vdW volume, solvent shell) uint8 [nz, ny, nx] of Lds.vdW_volume /
    Lds.first_solvent_shell."""
    x, y, z = _xyz(xyz)
    r = np.ascontiguousarray(radius, np.float64)
    v = np.zeros((g.nz, g.ny, g.nx), np.uint8)
    sh = np.zeros_like(v)
    lib().orc_masks(C.byref(g), len(r), _dp(x), _dp(y), _dp(z), _dp(r), C.c_double(r_w), _u8(v),
                    _u8(sh))
    return v, sh


def protein_ligand_clash(g: Lattice, vdw, xyz) -> bool:
    x, y, z = _xyz(xyz)
    v = np.ascontiguousarray(vdw, np.uint8)
    return bool(lib().orc_protein_ligand_clash(C.byref(g), _u8(v), len(x), _dp(x), _dp(y), _dp(z)))


def clash_and(g: Lattice, vdw, p) -> bool:
    v = np.ascontiguousarray(vdw, np.uint8)
    pp = np.ascontiguousarray(p, np.float64)
    return bool(lib().orc_clash_and(C.byref(g), _u8(v), _dp(pp)))


def center_occupied(xyz, radius) -> bool:
    x, y, z = _xyz(xyz)
    r = np.ascontiguousarray(radius, np.float64)
    return bool(lib().orc_center_occupied(len(r), _dp(x), _dp(y), _dp(z), _dp(r)))


def heavy_atom_clash(prot, xyz, anum) -> bool:
    P = OMol.of(prot)
    x, y, z = _xyz(xyz)
    a = np.ascontiguousarray(anum, np.int32)
    return bool(lib().orc_heavy_atom_clash(C.byref(P.c), len(a), _dp(x), _dp(y), _dp(z), _ip(a)))


def intra_clash(xyz, anum, interacting) -> bool:
    x, y, z = _xyz(xyz)
    a = np.ascontiguousarray(anum, np.int32)
    it = np.ascontiguousarray(interacting, np.uint8)
    return bool(lib().orc_intra_clash(len(a), _dp(x), _dp(y), _dp(z), _ip(a), _u8(it)))


def so3_rotation(n, i):
    R = np.zeros(9)
    lib().orc_so3_rotation(int(n), int(i), _dp(R))
    return R.reshape(3, 3)


def dock_scores(g: Lattice, grids, vdw, lig_mol, lig_type, lig_radius, center, radius, step,
                rotations, const_intra=0.0):
    """Every exhaustive-docking score (+inf where skipped), in frame order."""
    L = OMol.of(lig_mol)
    gr = np.ascontiguousarray(grids, np.float32)
    v = np.ascontiguousarray(vdw, np.uint8)
    lt = np.ascontiguousarray(lig_type, np.int32)
    lr = np.ascontiguousarray(lig_radius, np.float64)
    c = np.ascontiguousarray(center, np.float64)
    R = np.ascontiguousarray(rotations, np.float64).reshape(-1, 9)
    dim = int(np.ceil(2.0 * radius / step)) + 1
    out = np.zeros(dim ** 3 * len(R))
    dims = np.zeros(3, np.int32)
    lib().orc_dock_scores(C.byref(g), gr.ctypes.data_as(C.POINTER(C.c_float)), _u8(v),
                          C.byref(L.c), _ip(lt), _dp(lr), _dp(c), C.c_double(radius),
                          C.c_double(step), len(R), _dp(R), C.c_double(const_intra), _ip(dims),
                          _dp(out))
    return out, tuple(int(d) for d in dims)


def protein_desolv(g: Lattice, prot, shell, center, radius):
    P = OMol.of(prot)
    sh = np.ascontiguousarray(shell, np.uint8)
    c = np.ascontiguousarray(center, np.float64)
    out = np.zeros((g.nz, g.ny, g.nx))
    lib().orc_protein_desolv(C.byref(g), C.byref(P.c), _u8(sh), _dp(c), C.c_double(radius),
                             _dp(out))
    return out


def desolvation_penalty(g: Lattice, contrib, shell, xyz, q, radius, r_w=1.4):
    x, y, z = _xyz(xyz)
    pc = np.ascontiguousarray(contrib, np.float64)
    sh = np.ascontiguousarray(shell, np.uint8)
    qq = np.ascontiguousarray(q, np.float64)
    r = np.ascontiguousarray(radius, np.float64)
    out = np.zeros(2)
    lib().orc_desolvation_penalty(C.byref(g), _dp(pc), _u8(sh), len(qq), _dp(x), _dp(y), _dp(z),
                                  _dp(qq), _dp(r), C.c_double(r_w), _dp(out))
    return float(out[0]), float(out[1])
