"""The .mol2 -> .pqrs converter (mmo_gb300/mol2.py) on hand-made molecules:
the reference's rules for elements, bond orders, lone pairs, rotatable bonds,
rotation groups and topological distances, and the .pqrs reader reading the
result back."""
import numpy as np
import pytest

from mmo_gb300 import mol2 as M
from mmo_gb300.topology import read_pqrs

# 2-methylpropan-1-ol-like chain with a 3-ring and a lone pair:
# C1-C2(-C3)-C4-O5-H6, ring C7-C8-C9 on C1 via an amide-typed bond, LP on O5
LIG = """@<TRIPOS>MOLECULE
test_lig
 11 11 0 0 0
SMALL
USER_CHARGES

@<TRIPOS>ATOM
      1 C1  0.0000  0.0000  0.0000 C.3   1 LIG  -0.1000
      2 C2  1.5000  0.0000  0.0000 C.3   1 LIG   0.0500
      3 C3  2.0000  1.4000  0.0000 C.3   1 LIG  -0.0200
      4 C4  2.0000 -1.4000  0.0000 C.3   1 LIG   0.1000
      5 O5  3.4000 -1.4000  0.0000 O.3   1 LIG  -0.4000
      6 H6  3.8000 -2.3000  0.0000 H     1 LIG   0.3000
      7 C7 -0.7000  1.2000  0.3000 C.3   1 LIG   0.0100
      8 C8 -1.4000  0.1000  1.0000 C.3   1 LIG   0.0200
      9 C9 -1.0000  1.4000  1.8000 C.3   1 LIG   0.0300
     10 LP1 3.6000 -0.9000  0.5000 LP    1 LIG   0.0000
     11 Cl1 -2.8000  0.0000  1.0000 Cl    1 LIG   0.0400
@<TRIPOS>UNITY_ATOM_ATTR
5 1
charge -1
@<TRIPOS>BOND
     1     1     2    1
     2     2     3    1
     3     2     4    1
     4     4     5    1
     5     5     6    1
     6     1     7   am
     7     7     8    1
     8     8     9    1
     9     9     7    1
    10     5    10    1
    11     8    11    1
"""

REC = """@<TRIPOS>MOLECULE
rec
 2 1 0 0 0
SMALL
USER_CHARGES

@<TRIPOS>ATOM
      1 N1  0.0000  0.0000  0.0000 N.am  1 ALA  -0.4000
      2 S1  1.8000  0.0000  0.0000 S.3   1 CYS   0.1000
@<TRIPOS>BOND
     1     1     2    1
"""


def test_ligand_conversion(tmp_path):
    src = tmp_path / "lig.mol2"
    src.write_text(LIG)
    dst = tmp_path / "lig.pqrs"
    assert M.mol2_to_pqrs(str(src), str(dst)) == []
    lines = dst.read_text().splitlines()
    n = 10  # the lone pair and its bond are dropped
    # rotatable: single, not in the ring, both ends non-terminal:
    # C1-C2, C2-C4, C4-O5, and the amide-typed C1-C7 (bond order 1); not C2-C3
    # (C3 terminal), not O5-H6, not the ring bonds, not C8-Cl (Cl terminal)
    assert lines[0] == "%d:4:test_lig" % n
    assert lines[1] == "0 0 0 -0.1 1.7 C"
    assert lines[6] == "3.8 -2.3 0 0.3 1.2 H"
    assert lines[10] == "-2.8 0 1 0.04 1.8 Cl"
    rb = lines[1 + n:1 + n + 4]
    heads = [r.split("=")[0] for r in rb]
    assert heads == ["0-1", "1-3", "3-4", "0-6"]  # in the file's bond order
    # C1-C2: the C2 side {C2, C3, C4, O5, H6} is the smaller (5 of 10)... the
    # C1 side {C1, C7, C8, C9, Cl} has 5 as well: the tie goes to the src side
    bits = [int(v) for v in rb[0].split("=")[1].split()]
    assert bits == [1, 0, 0, 0, 0, 0, 1, 1, 1, 1]
    # C4-O5: the O5 side {O5, H6}; C1-C7: the ring side {C7, C8, C9, Cl}
    bits = [int(v) for v in rb[2].split("=")[1].split()]
    assert bits == [0, 0, 0, 0, 1, 1, 0, 0, 0, 0]
    bits = [int(v) for v in rb[3].split("=")[1].split()]
    assert bits == [0, 0, 0, 0, 0, 0, 1, 1, 1, 1]
    dm = np.array([[int(v) for v in ln.split()] for ln in lines[1 + n + 4:]])
    assert dm.shape == (n, n) and np.array_equal(dm, dm.T)
    assert dm[0, 5] == 4 and dm[2, 9] == 5 and dm[6, 8] == 1
    (mol,) = read_pqrs(str(dst))
    assert mol.n == n and mol.nrb == 4
    assert mol.anum.tolist() == [6, 6, 6, 6, 8, 1, 6, 6, 6, 17]
    assert np.allclose(mol.q, [-0.1, 0.05, -0.02, 0.1, -0.4, 0.3, 0.01, 0.02, 0.03, 0.04])
    # the in-memory ligand has the same topology
    name, atoms, bonds = M.read_mol2(str(src))[0]
    m = M.to_mol(name, atoms, bonds)
    assert m.nrb == 4 and np.array_equal(m.dists, dm)


def test_receptor_and_errors(tmp_path):
    src = tmp_path / "rec.mol2"
    src.write_text(REC)
    dst = tmp_path / "rec.pqrs"
    M.mol2_to_pqrs(str(src), str(dst), receptor=True)
    assert dst.read_text().splitlines() == ["2:rec", "0 0 0 -0.4 1.6 N", "1.8 0 0 0.1 1.8 S"]
    (rec,) = read_pqrs(str(dst))
    assert rec.n == 2 and rec.anum.tolist() == [7, 16]
    src.write_text(REC.replace("-0.4000", "0.0000").replace(" 0.1000", " 0.0000"))
    with pytest.raises(ValueError):
        M.mol2_to_pqrs(str(src), str(dst), receptor=True)
    with pytest.raises(M.UnsupportedAtom):
        M.anum_of_mol2_type("Du")
    with pytest.raises(ValueError):
        M.bond_order("nc")
    # a disconnected atom: the ligand is skipped
    src.write_text(LIG.replace("    11     8    11    1\n", "").replace(" 11 11 0", " 11 10 0"))
    assert M.mol2_to_pqrs(str(src), str(dst)) == ["test_lig"]


def test_ff_score_reads_mol2_like_pqrs(tmp_path):
    """mmo_gb300.ff_score's input: a .mol2 file gives the same ligands as its
    .pqrs conversion (topology, charges, coordinates), and a ligand with a
    disconnected atom is skipped as mol2pqrs skips it."""
    from mmo_gb300.ff_score import load_ligands

    src = tmp_path / "lig.mol2"
    src.write_text(LIG)
    dst = tmp_path / "lig.pqrs"
    M.mol2_to_pqrs(str(src), str(dst))
    (a,) = load_ligands(str(src))
    (b,) = load_ligands(str(dst))
    assert a.n == b.n and a.nrb == b.nrb
    assert np.array_equal(a.dists, b.dists) and np.array_equal(a.anum, b.anum)
    assert np.allclose(a.q, b.q) and np.allclose(a.xyz(), b.xyz())
    assert [sorted(g) for g in a.rgroups] == [sorted(g) for g in b.rgroups]
    lone = LIG.replace("     11     8    11    1\n", "").replace(" 11 11 0 0 0", " 11 10 0 0 0")
    src2 = tmp_path / "lone.mol2"
    src2.write_text(lone)
    assert load_ligands(str(src2)) == []
