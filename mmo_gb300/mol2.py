"""The .mol2 -> .pqrs converter of the reference (src/mol2pqrs.ml), for real inputs.

A .pqrs file carries what the scorer needs of a molecule (src/pqrs.ml): per
atom x y z charge radius element, and for a ligand its rotatable bonds with
their rotation groups and the topological distance matrix.  This module
restates, on the host:

* the .mol2 reader (Mol2.parse_one_mol2_block, src/mol2.ml:243-305): the
  MOLECULE / ATOM / BOND sections, lone pairs ("LP" atoms and their bonds)
  dropped, the UNITY_ATOM_ATTR section skipped, bond orders of
  Mol2.bond_order (src/mol2.ml:141-151: "ar" 1.5, "am" 1);
* the SYBYL type -> element map (Ptable.anum_of_mol2_type,
  src/ptable.ml:169-225) and the vdW radius of the element
  (Ptable.vdW_radii, src/ptable.ml:41-53);
* the molecular graph work of Mol_graph (src/mol_graph.ml): the all-pairs
  topological distances, the rotatable bonds (single, not in a ring, between
  two non-terminal atoms) and each bond's rotation group (the smaller side),
  through mmo_gb300.topology;
* the writers of Mol2pqrs.process_ligand / process_receptor
  (src/mol2pqrs.ml:10-55): a ligand with an atom disconnected from the rest is
  skipped (an error in the reference's log).
"""
from __future__ import annotations

import numpy as np

from .topology import Mol, build_ligand

MOLECULE = "@<TRIPOS>MOLECULE"
ATOM = "@<TRIPOS>ATOM"
BOND = "@<TRIPOS>BOND"
UNITY = "@<TRIPOS>UNITY_ATOM_ATTR"

_TYPE_ANUM = {}
for _anum, _types in (
        (1, "H H.t3p H.spc"), (3, "Li"), (6, "C.3 C.2 C.1 C.ar C.cat"),
        (7, "N.3 N.2 N.1 N.ar N.am N.pl3 N.4"), (8, "O.3 O.2 O.co2 O.spc O.t3p"), (9, "F"),
        (11, "Na"), (12, "Mg"), (13, "Al"), (14, "Si"), (15, "P.3"),
        (16, "S.3 S.2 S.O S.o S.O2 S.o2"), (17, "Cl"), (19, "K"), (20, "Ca"),
        (24, "Cr.th Cr.oh"), (25, "Mn"), (26, "Fe"), (27, "Co.oh"), (29, "Cu"), (30, "Zn"),
        (34, "Se"), (35, "Br"), (42, "Mo"), (50, "Sn"), (53, "I")):
    for _t in _types.split():
        _TYPE_ANUM[_t] = _anum

VDW_RADII = {1: 1.2, 6: 1.7, 7: 1.6, 8: 1.55, 9: 1.5, 12: 2.2, 15: 1.95, 16: 1.8, 17: 1.8,
             35: 1.9, 53: 2.1}

_BOND_ORDER = {"1": 1.0, "2": 2.0, "3": 3.0, "ar": 1.5, "am": 1.0}


class UnsupportedAtom(ValueError):
    pass


def anum_of_mol2_type(typ: str) -> int:
    """Ptable.anum_of_mol2_type."""
    try:
        return _TYPE_ANUM[typ]
    except KeyError:
        raise UnsupportedAtom(typ) from None


def bond_order(typ: str) -> float:
    """Mol2.bond_order ("du", "un", "nc" and others are errors)."""
    try:
        return _BOND_ORDER[typ]
    except KeyError:
        raise ValueError("Mol2.bond_order: %s" % typ) from None


def _blocks(lines):
    cur = None
    for line in lines:
        line = line.rstrip("\n")
        if line.strip() == MOLECULE:
            if cur:
                yield cur
            cur = [line.strip()]
        elif cur is not None:
            cur.append(line)
    if cur:
        yield cur


def parse_block(block):
    """(name, atoms [(name, x, y, z, type, q)], bonds [(src, dst, type)]) of one
    molecule, 0-based bond ends, lone pairs removed."""
    name = block[1].strip()
    n_atoms, n_bonds = (int(v) for v in block[2].split()[:2])
    i = 3
    while block[i].strip() != ATOM:
        i += 1
    i += 1
    atoms = []
    for _ in range(n_atoms):
        f = block[i].split()
        atoms.append((f[1], float(f[2]), float(f[3]), float(f[4]), f[5], float(f[8])))
        i += 1
    if block[i].strip() == UNITY:
        while block[i].strip() != BOND:
            i += 1
    if block[i].strip() != BOND:
        raise ValueError("no bonds section in %s" % name)
    i += 1
    bonds = []
    for _ in range(n_bonds):
        f = block[i].split()
        bonds.append((int(f[1]) - 1, int(f[2]) - 1, f[3]))
        i += 1
    # Mol2.remove_lone_pairs
    lp = [a[4] == "LP" for a in atoms]
    if any(lp):
        new = np.cumsum([0] + [0 if x else 1 for x in lp])[:-1]
        bonds = [(int(new[s]), int(new[d]), t) for s, d, t in bonds if not (lp[s] or lp[d])]
        atoms = [a for a, x in zip(atoms, lp) if not x]
    return name, atoms, bonds


def read_mol2(path):
    with open(path) as f:
        return [parse_block(b) for b in _blocks(f)]


def _connected(n, bonds) -> bool:
    adj = [[] for _ in range(n)]
    for s, d, _ in bonds:
        adj[s].append(d)
        adj[d].append(s)
    seen = {0} if n else set()
    stack = [0] if n else []
    while stack:
        for v in adj[stack.pop()]:
            if v not in seen:
                seen.add(v)
                stack.append(v)
    return len(seen) == n


def to_mol(name, atoms, bonds, receptor=False) -> Mol:
    xyz = np.array([[a[1], a[2], a[3]] for a in atoms], np.float64)
    q = np.array([a[5] for a in atoms], np.float64)
    anum = np.array([anum_of_mol2_type(a[4]) for a in atoms], np.int32)
    radius = np.array([VDW_RADII.get(int(z), np.nan) for z in anum])
    if receptor:
        m = Mol(name, xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy(), q, anum, radius)
        return m
    pairs = [(s, d) for s, d, _ in bonds]
    orders = [bond_order(t) for _, _, t in bonds]
    m = build_ligand(name, xyz, q, anum, pairs, orders)
    m.radius = radius
    return m


SYMBOLS = {1: "H", 3: "Li", 6: "C", 7: "N", 8: "O", 9: "F", 11: "Na", 12: "Mg", 13: "Al",
           14: "Si", 15: "P", 16: "S", 17: "Cl", 19: "K", 20: "Ca", 24: "Cr", 25: "Mn", 26: "Fe",
           27: "Co", 29: "Cu", 30: "Zn", 34: "Se", 35: "Br", 42: "Mo", 50: "Sn", 53: "I"}


def _atom_line(a) -> str:
    """Mol2.pqrs_line_of_atom (src/mol2.ml:67-69): x y z q r element (the radius
    NaN for elements without a vdW radius, as Ptable prints it)."""
    anum = anum_of_mol2_type(a[4])
    r = VDW_RADII.get(anum, float("nan"))
    return "%g %g %g %g %g %s" % (a[1], a[2], a[3], a[5], r, SYMBOLS[anum])


def ligand_pqrs_text(name, atoms, bonds) -> str:
    """Mol2pqrs.process_ligand (src/mol2pqrs.ml:10-43): the header n:nrb:name,
    the atom lines, one "src-dst= 0 1 ..." line per rotatable bond (its rotation
    group, the smaller side; on a tie the side of src), the distance matrix."""
    from .topology import dist_matrix, rot_group, rotatable_bonds

    n = len(atoms)
    pairs = [(s, d) for s, d, _ in bonds]
    orders = [bond_order(t) for _, _, t in bonds]
    rb = rotatable_bonds(n, pairs, orders)
    out = ["%d:%d:%s" % (n, len(rb), name)]
    out += [_atom_line(a) for a in atoms]
    for bnd in rb:
        g = rot_group(n, pairs, bnd)
        out.append("%d-%d=%s" % (bnd[0], bnd[1], "".join(" 1" if i in g else " 0"
                                                          for i in range(n))))
    dm = dist_matrix(n, pairs)
    out += [" ".join(str(int(v)) for v in dm[i]) for i in range(n)]
    return "\n".join(out) + "\n"


def receptor_pqrs_text(name, atoms) -> str:
    """Mol2pqrs.process_receptor (src/mol2pqrs.ml:45-58)."""
    if all(a[5] == 0.0 for a in atoms):
        raise ValueError("all null charges: %s" % name)
    return "\n".join(["%d:%s" % (len(atoms), name)] + [_atom_line(a) for a in atoms]) + "\n"


def mol2_to_pqrs(src: str, dst: str, receptor=False) -> list[str]:
    """Convert every molecule of src (mol2pqrs -lig / -rec); returns the names
    of the ligands skipped for a disconnected atom."""
    texts, skipped = [], []
    for name, atoms, bonds in read_mol2(src):
        if receptor:
            texts.append(receptor_pqrs_text(name, atoms))
        elif not _connected(len(atoms), bonds):
            skipped.append(name)
        else:
            texts.append(ligand_pqrs_text(name, atoms, bonds))
    with open(dst, "w") as f:
        f.write("".join(texts))
    return skipped
