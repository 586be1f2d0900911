"""Ligand topology and the ``.pqrs`` file format.

Host-side data layout of MMO's ``Mol.t`` (src/mol.ml:17-35): SoA coordinates,
partial charges, atomic numbers, the topological distance matrix, the
``interacting`` matrix (topological distance >= 3, src/mol.ml:203-208), the
rotatable bonds as (left, right) pairs and their rotation groups (right end
excluded, src/pqrs.ml:80-87).

Topology is derived from a bond list the way src/mol_graph.ml does it:
all-pairs shortest paths in bonds (mol_graph.ml:53-70), rotatable bond =
single, non-ring, both ends of degree > 1 (mol_graph.ml:126-138), rotation
group = the smaller side of the bond (mol_graph.ml:155-192).
"""
from __future__ import annotations

from collections import deque
from dataclasses import dataclass, field

import numpy as np

# src/ptable.ml: the elements the UFF table supports (UFF.ml:10-22)
SYMBOL_TO_ANUM = {"H": 1, "C": 6, "N": 7, "O": 8, "F": 9, "Mg": 12, "P": 15, "S": 16,
                  "Cl": 17, "Br": 35, "I": 53}
ANUM_TO_SYMBOL = {v: k for k, v in SYMBOL_TO_ANUM.items()}
ANUM_TO_SYMBOL[0] = "X"


@dataclass
class Mol:
    """One molecule; ``rbonds`` and the matrices are empty for a protein."""

    name: str
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    q: np.ndarray
    anum: np.ndarray
    radius: np.ndarray | None = None
    dists: np.ndarray | None = None          # (n, n) int32
    rbonds: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    rgroups: list = field(default_factory=list)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @property
    def nrb(self) -> int:
        return int(self.rbonds.shape[0])

    @property
    def interacting(self) -> np.ndarray:
        """uint8 (n, n): 1 where UFF counts the non-bonded pair (mol.ml:203-208)."""
        if self.dists is None:
            raise ValueError("protein molecules carry no topology")
        return (self.dists >= 3).astype(np.uint8)

    def xyz(self) -> np.ndarray:
        return np.stack([self.x, self.y, self.z], axis=1)

    def with_xyz(self, xyz: np.ndarray) -> "Mol":
        xyz = np.asarray(xyz, dtype=np.float64)
        return Mol(self.name, xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy(), self.q,
                   self.anum, self.radius, self.dists, self.rbonds, self.rgroups)

    def centered(self) -> "Mol":
        """Mol.center (mol.ml:699-702): translate the centroid to the origin."""
        xyz = self.xyz()
        return self.with_xyz(xyz - xyz.mean(axis=0))

    def group_arrays(self) -> tuple[np.ndarray, np.ndarray]:
        """Rotation groups as CSR (offsets[nrb+1], atoms[])."""
        off = np.zeros(self.nrb + 1, np.int32)
        for t, g in enumerate(self.rgroups):
            off[t + 1] = off[t] + len(g)
        atoms = (np.concatenate([np.asarray(g, np.int32) for g in self.rgroups])
                 if self.rgroups else np.zeros(0, np.int32))
        return off, atoms.astype(np.int32)


def adjacency(n: int, bonds) -> list[list[int]]:
    adj: list[list[int]] = [[] for _ in range(n)]
    for a, b in bonds:
        adj[a].append(b)
        adj[b].append(a)
    return adj


def dist_matrix(n: int, bonds) -> np.ndarray:
    """Topological distances in bonds (mol_graph.ml:53-70); disconnected -> error."""
    adj = adjacency(n, bonds)
    d = np.full((n, n), -1, np.int32)
    for s in range(n):
        d[s, s] = 0
        dq = deque([s])
        while dq:
            u = dq.popleft()
            for v in adj[u]:
                if d[s, v] < 0:
                    d[s, v] = d[s, u] + 1
                    dq.append(v)
    if (d < 0).any():
        raise ValueError("disconnected atom")  # Mol_graph.Disconnected_atom
    return d


def _side(n: int, adj, start: int, cut: tuple[int, int]) -> set[int]:
    a, b = cut
    seen = {start}
    dq = deque([start])
    while dq:
        u = dq.popleft()
        for v in adj[u]:
            if (u, v) in ((a, b), (b, a)):
                continue
            if v not in seen:
                seen.add(v)
                dq.append(v)
    return seen


def is_ring_bond(n: int, adj, a: int, b: int) -> bool:
    """mol_graph.ml:110-118: still connected once the bond is removed."""
    return b in _side(n, adj, a, (a, b))


def rotatable_bonds(n: int, bonds, orders) -> list[tuple[int, int]]:
    """mol_graph.ml:126-138, in bond order."""
    adj = adjacency(n, bonds)
    deg = [len(a) for a in adj]
    out = []
    for (a, b), bo in zip(bonds, orders):
        if bo == 1.0 and deg[a] > 1 and deg[b] > 1 and not is_ring_bond(n, adj, a, b):
            out.append((a, b))
    return out


def rot_group(n: int, bonds, bond: tuple[int, int]) -> set[int]:
    """mol_graph.ml:155-192: the smaller side of the bond (ties: the src side)."""
    adj = adjacency(n, bonds)
    a, b = bond
    side_a = _side(n, adj, a, bond)
    side_b = set(range(n)) - side_a
    return side_a if len(side_a) <= len(side_b) else side_b


def axis_and_group(bond: tuple[int, int], group: set[int]) -> tuple[tuple[int, int], list[int]]:
    """pqrs.ml:311-319 and 343-351: orient the axis so that the right end is in
    the group, then drop the right end from the group."""
    beg, end = bond
    left, right = (beg, end) if end in group else (end, beg)
    return (left, right), sorted(i for i in group if i != right)


def build_ligand(name, xyz, q, anum, bonds, orders=None, rbonds=None) -> Mol:
    """Ligand Mol from coordinates and a bond list.  ``rbonds`` (list of bonds)
    overrides the automatic rotatable-bond list when given."""
    xyz = np.asarray(xyz, np.float64)
    n = xyz.shape[0]
    if orders is None:
        orders = [1.0] * len(bonds)
    if rbonds is None:
        rbonds = rotatable_bonds(n, bonds, orders)
    axes, groups = [], []
    for bnd in rbonds:
        ax, g = axis_and_group(bnd, rot_group(n, bonds, bnd))
        axes.append(ax)
        groups.append(np.asarray(g, np.int32))
    return Mol(name, xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy(),
               np.asarray(q, np.float64), np.asarray(anum, np.int32), None,
               dist_matrix(n, bonds), np.asarray(axes, np.int32).reshape(-1, 2), groups)


# ---------------------------------------------------------------------------
# .pqrs format (src/pqrs.ml:17-87, writer src/mol2pqrs.ml:10-43)
# ---------------------------------------------------------------------------

def _fmt(v: float) -> str:
    return "%g" % v


def write_pqrs(path, mols, receptor=False) -> None:
    with open(path, "w") as f:
        for m in mols:
            if receptor:
                f.write("%d:%s\n" % (m.n, m.name))
            else:
                f.write("%d:%d:%s\n" % (m.n, m.nrb, m.name))
            rad = m.radius if m.radius is not None else np.zeros(m.n)
            for i in range(m.n):
                f.write("%s %s %s %s %s %s\n" % (_fmt(m.x[i]), _fmt(m.y[i]), _fmt(m.z[i]),
                                                 _fmt(m.q[i]), _fmt(rad[i]),
                                                 ANUM_TO_SYMBOL[int(m.anum[i])]))
            if receptor:
                continue
            for t in range(m.nrb):
                left, right = (int(v) for v in m.rbonds[t])
                grp = set(int(v) for v in m.rgroups[t]) | {right}
                f.write("%d-%d=%s\n" % (left, right,
                                        "".join(" 1" if i in grp else " 0" for i in range(m.n))))
            for i in range(m.n):
                f.write(" ".join(str(int(v)) for v in m.dists[i]) + "\n")


def read_pqrs(path) -> list[Mol]:
    """All molecules of a .pqrs file (ligands, or one receptor)."""
    out = []
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f]
    k = 0
    while k < len(lines):
        if not lines[k].strip():
            k += 1
            continue
        head = lines[k].split(":")
        k += 1
        if len(head) >= 3 and head[1].lstrip("-").isdigit():
            n, nrb, name = int(head[0]), int(head[1]), ":".join(head[2:])
        else:
            n, nrb, name = int(head[0]), -1, ":".join(head[1:])
        rows = [lines[k + i].split() for i in range(n)]
        k += n
        x = np.array([float(r[0]) for r in rows])
        y = np.array([float(r[1]) for r in rows])
        z = np.array([float(r[2]) for r in rows])
        q = np.array([float(r[3]) for r in rows])
        rad = np.array([float(r[4]) for r in rows])
        anum = np.array([SYMBOL_TO_ANUM[r[5]] for r in rows], np.int32)
        if nrb < 0:
            out.append(Mol(name, x, y, z, q, anum, rad))
            continue
        axes, groups = [], []
        for _ in range(nrb):
            ln = lines[k]
            k += 1
            pair, bits = ln.split("=", 1)
            beg, end = (int(v) for v in pair.split("-"))
            flags = [b == "1" for b in bits.split()]
            if len(flags) != n or flags[beg] == flags[end]:
                raise ValueError("bad rotatable bond line: " + ln)
            left, right = (beg, end) if flags[end] else (end, beg)
            axes.append((left, right))
            groups.append(np.array([i for i in range(n) if flags[i] and i != right], np.int32))
        dists = np.array([[int(v) for v in lines[k + i].split()] for i in range(n)], np.int32)
        k += n
        # pqrs.ml:326-341 stores line i, column j at res.(i + j*n), which
        # get_topo_dist m i j reads back: dists[i, j] here
        out.append(Mol(name, x, y, z, q, anum, rad, dists,
                       np.asarray(axes, np.int32).reshape(-1, 2), groups))
    return out
