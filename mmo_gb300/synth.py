"""Seeded synthetic ligands, pockets and poses for the scoring workloads.

The reference publishes no benchmark inputs, so every workload is synthetic and
seeded (numpy PCG64):

* ligand: a random tree grown by attaching each new atom 1.5 A from a random
  atom with fewer than 4 neighbours, at 109.5 degrees from that atom's first
  bond, rejecting positions within 1.2 A of an existing atom; rotatable bonds
  are drawn among internal bonds (both ends of degree > 1) and each rotation
  group is the smaller side (src/mol_graph.ml:155-192); UFF types drawn
  uniformly from {C_3, C_R, N_3, N_R, O_3, O_2, S_3, H_}; charges N(0, 0.3)
  shifted to a net charge of 0; the conformer is centred (src/mol.ml:699-702);
* pocket: atoms uniform in a sphere with a 1.2 A minimum separation, same
  types, charges N(0, 0.4);
* poses: the optimiser layout [x, y, z, a, b, g, tau...] of src/optim.ml:19-22,
  rotations uniform on SO(3) (Shoemake quaternions) written as the Euler
  angles of Rot.decompose (src/rot.ml:71-75), translations uniform in a cube,
  torsions uniform in [-pi, pi).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .topology import Mol, axis_and_group, dist_matrix, rot_group

# UFF type labels and the element each maps to (the reference keys UFF
# parameters by element only, src/UFF.ml:10-22, src/mol.ml:810-812)
TYPE_LABELS = ("C_3", "C_R", "N_3", "N_R", "O_3", "O_2", "S_3", "H_")
TYPE_ANUM = np.array([6, 6, 7, 7, 8, 8, 16, 1], np.int32)

BOND = 1.5
ANGLE = math.radians(109.5)
MIN_SEP = 1.2


def _unit(v):
    return v / np.linalg.norm(v)


def _perp(u, rng):
    a = rng.normal(size=3)
    a -= a.dot(u) * u
    return _unit(a)


def random_ligand(rng: np.random.Generator, n_atoms: int, n_rot: int, name="lig",
                  charge_sigma=0.3) -> Mol:
    """Random tree ligand; ``n_rot`` is capped by the number of internal bonds."""
    xyz = [np.zeros(3)]
    nbr: list[list[int]] = [[]]
    bonds: list[tuple[int, int]] = []
    tries = 0
    while len(xyz) < n_atoms:
        tries += 1
        if tries > 200000:
            raise RuntimeError("ligand growth stalled")
        cand = [i for i in range(len(xyz)) if len(nbr[i]) < 4]
        p = int(cand[rng.integers(len(cand))])
        if nbr[p]:
            b = _unit(xyz[nbr[p][0]] - xyz[p])
            w = _perp(b, rng)
            d = math.cos(ANGLE) * b + math.sin(ANGLE) * w
        else:
            d = _unit(rng.normal(size=3))
        pos = xyz[p] + BOND * d
        arr = np.asarray(xyz)
        if np.min(np.linalg.norm(arr - pos, axis=1)) < MIN_SEP:
            continue
        k = len(xyz)
        xyz.append(pos)
        nbr.append([p])
        nbr[p].append(k)
        bonds.append((p, k))
    n = n_atoms
    deg = [len(a) for a in nbr]
    internal = [b for b in bonds if deg[b[0]] > 1 and deg[b[1]] > 1]
    n_rot = min(n_rot, len(internal))
    pick = sorted(rng.choice(len(internal), size=n_rot, replace=False).tolist()) if n_rot else []
    rb = [internal[i] for i in pick]
    types = rng.integers(0, len(TYPE_LABELS), size=n)
    anum = TYPE_ANUM[types]
    q = rng.normal(0.0, charge_sigma, size=n)
    q -= q.mean()
    xyz = np.asarray(xyz)
    xyz -= xyz.mean(axis=0)
    axes, groups = [], []
    for bnd in rb:
        ax, g = axis_and_group(bnd, rot_group(n, bonds, bnd))
        axes.append(ax)
        groups.append(np.asarray(g, np.int32))
    m = Mol(name, xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy(), q, anum.astype(np.int32),
            None, dist_matrix(n, bonds), np.asarray(axes, np.int32).reshape(-1, 2), groups)
    m.bonds = bonds  # kept for the mol2/pqrs writers
    m.type_labels = [TYPE_LABELS[t] for t in types]
    return m


def sphere_points(rng: np.random.Generator, n: int, radius: float, min_sep=MIN_SEP,
                  batch=None) -> np.ndarray:
    """``n`` points uniform in a ball with pairwise distance >= min_sep.

    Dart throwing in batches: a candidate is kept when it is farther than
    min_sep from every kept point and from every earlier candidate of its
    batch that survived the first test."""
    from scipy.spatial import cKDTree

    pts = np.zeros((0, 3))
    batch = batch or max(256, n // 4)
    rounds = 0
    while pts.shape[0] < n:
        rounds += 1
        if rounds > 10000:
            raise RuntimeError("sphere packing stalled: density too high")
        c = rng.uniform(-radius, radius, size=(batch * 2, 3))
        c = c[np.einsum("ij,ij->i", c, c) <= radius * radius][:batch]
        if pts.shape[0]:
            d, _ = cKDTree(pts).query(c, k=1, distance_upper_bound=min_sep)
            c = c[~(d < min_sep)]
        if c.shape[0] == 0:
            continue
        pairs = cKDTree(c).query_pairs(min_sep, output_type="ndarray")
        keep = np.ones(c.shape[0], bool)
        if pairs.size:
            # drop the later candidate of every close pair, in candidate order
            for i, j in pairs[np.argsort(pairs[:, 1], kind="stable")]:
                if keep[i] and keep[j]:
                    keep[j] = False
        pts = np.concatenate([pts, c[keep]])
    return pts[:n]


def random_pocket(rng: np.random.Generator, n_atoms: int, radius: float, name="pocket",
                  charge_sigma=0.4) -> Mol:
    xyz = sphere_points(rng, n_atoms, radius)
    types = rng.integers(0, len(TYPE_LABELS), size=n_atoms)
    q = rng.normal(0.0, charge_sigma, size=n_atoms)
    m = Mol(name, xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy(), q,
            TYPE_ANUM[types].astype(np.int32), np.zeros(n_atoms))
    m.type_labels = [TYPE_LABELS[t] for t in types]
    return m


def decompose(R: np.ndarray):
    """Rot.decompose (src/rot.ml:71-75) for row-major R = Rz Ry Rx."""
    a, d, g, h, i = R[..., 0, 0], R[..., 1, 0], R[..., 2, 0], R[..., 2, 1], R[..., 2, 2]
    beta = np.arctan2(-g, np.sqrt(a * a + d * d))
    cb = np.cos(beta)
    return np.arctan2(h / cb, i / cb), beta, np.arctan2(d / cb, a / cb)


def quat_to_matrix(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    R = np.empty(q.shape[:-1] + (3, 3))
    R[..., 0, 0] = 1 - 2 * (y * y + z * z)
    R[..., 0, 1] = 2 * (x * y - z * w)
    R[..., 0, 2] = 2 * (x * z + y * w)
    R[..., 1, 0] = 2 * (x * y + z * w)
    R[..., 1, 1] = 1 - 2 * (x * x + z * z)
    R[..., 1, 2] = 2 * (y * z - x * w)
    R[..., 2, 0] = 2 * (x * z - y * w)
    R[..., 2, 1] = 2 * (y * z + x * w)
    R[..., 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def shoemake_quats(rng: np.random.Generator, n: int) -> np.ndarray:
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    return np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                     b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)


def random_poses(rng: np.random.Generator, n_poses: int, n_rot: int, half_box: float,
                 center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """float32 [n_poses, 6 + n_rot] in the optimiser layout."""
    q = shoemake_quats(rng, n_poses)
    al, be, ga = decompose(quat_to_matrix(q))
    t = rng.uniform(-half_box, half_box, size=(n_poses, 3)) + np.asarray(center)
    tau = rng.uniform(-np.pi, np.pi, size=(n_poses, n_rot))
    return np.concatenate([t, np.stack([al, be, ga], axis=1), tau], axis=1).astype(np.float32)


@dataclass
class System:
    """One pocket, one ligand and a batch of poses."""

    name: str
    pocket: Mol
    ligand: Mol
    poses: np.ndarray  # float32 [B, 6 + nrb]


# Ptable.vdW_radii (src/ptable.ml:41-53) of the synthetic elements
VDW_RADIUS = {1: 1.2, 6: 1.7, 7: 1.6, 8: 1.55, 16: 1.8}


def radii(mol: Mol) -> np.ndarray:
    """Ptable.vdW_radii of each atom (the .pqrs radius column of real inputs)."""
    return np.array([VDW_RADIUS[int(a)] for a in mol.anum], np.float64)


def docking_site(seed=0, n_pocket=3000, r_in=7.5, r_out=16.0, n_atoms=16, n_rot=3) -> System:
    """A cavity for docking: pocket atoms between r_in and r_out about the
    origin, and a small ligand that fits in the empty core; no poses."""
    rng = np.random.default_rng(seed)
    pts = sphere_points(rng, int(n_pocket * 1.7), r_out)
    pts = pts[np.einsum("ij,ij->i", pts, pts) >= r_in * r_in][:n_pocket]
    types = rng.integers(0, len(TYPE_LABELS), size=len(pts))
    q = rng.normal(0.0, 0.4, size=len(pts))
    pocket = Mol("cavity%d" % len(pts), pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), q,
                 TYPE_ANUM[types].astype(np.int32), np.zeros(len(pts)))
    pocket.type_labels = [TYPE_LABELS[t] for t in types]
    pocket.radius = radii(pocket)
    lig = random_ligand(rng, n_atoms, n_rot, "lig%d" % n_atoms)
    lig.radius = radii(lig)
    return System("dock_site_P%d_L%d" % (len(pts), n_atoms), pocket, lig,
                  np.zeros((0, 6 + lig.nrb), np.float32))


def single_pose(seed=0) -> System:
    """Plain single-pose score: 32-atom ligand with 5 rotatable bonds at the
    centre of a 1,500-atom pocket in a 14 A sphere, random torsions."""
    rng = np.random.default_rng(seed)
    lig = random_ligand(rng, 32, 5, "lig32")
    pocket = random_pocket(rng, 1500, 14.0, "pocket1500")
    tau = rng.uniform(-np.pi, np.pi, size=lig.nrb)
    poses = np.concatenate([np.zeros(6), tau])[None, :].astype(np.float32)
    return System("single_pose_L32_P1500", pocket, lig, poses)


def pose_batch(n_poses=65536, seed=1, n_atoms=48, n_rot=8, n_pocket=6000, radius=18.0,
               half_box=4.0) -> System:
    """Plain-vs-batched pose scoring: 48-atom ligand, 8 rotatable bonds, 6,000
    pocket atoms in an 18 A sphere, translations in an 8 A cube about the
    centre.  The energy+gradient workload is the same system with 4,096 poses."""
    rng = np.random.default_rng(seed)
    lig = random_ligand(rng, n_atoms, n_rot, "lig%d" % n_atoms)
    pocket = random_pocket(rng, n_pocket, radius, "pocket%d" % n_pocket)
    poses = random_poses(np.random.default_rng(seed + 1000), n_poses, lig.nrb, half_box)
    return System("poses%d_L%d_P%d" % (n_poses, n_atoms, n_pocket), pocket, lig, poses)


def ragged_system(index: int, seed=3, poses_per=64, density=None) -> System:
    """System ``index`` of the uneven batch: ligand size log-uniform in 12-80
    atoms, 0-15 rotatable bonds, pocket size uniform in 2,000-8,000 atoms at the
    density of the 6,000-atom 18 A pocket, ``poses_per`` random poses.  Each
    system has its own generator (seeded by (seed, index)), so a batch can be
    made in any order or in parallel."""
    rng = np.random.default_rng([seed, index])
    density = density or 6000.0 / (4.0 / 3.0 * math.pi * 18.0 ** 3)
    n_l = int(round(math.exp(rng.uniform(math.log(12), math.log(80)))))
    n_r = int(rng.integers(0, 16))
    n_p = int(rng.integers(2000, 8001))
    radius = (3.0 * n_p / (4.0 * math.pi * density)) ** (1.0 / 3.0)
    lig = random_ligand(rng, n_l, n_r, "lig%d" % index)
    pocket = random_pocket(rng, n_p, radius, "pocket%d" % index)
    poses = random_poses(rng, poses_per, lig.nrb, 4.0)
    return System("sys%d" % index, pocket, lig, poses)


def _ragged_one(a):
    return ragged_system(*a)


def ragged_systems(n_systems=1024, poses_per=64, seed=3, density=None, workers=0) -> list[System]:
    """The uneven batch of ragged_system 0 .. n_systems - 1; workers > 1 makes
    them in that many spawned processes (start them before CUDA is used)."""
    args = [(s, seed, poses_per, density) for s in range(n_systems)]
    if workers and workers > 1 and n_systems > 1:
        import concurrent.futures as cf
        import multiprocessing as mp

        with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            return list(ex.map(_ragged_one, args, chunksize=max(1, n_systems // (4 * workers))))
    return [_ragged_one(a) for a in args]
