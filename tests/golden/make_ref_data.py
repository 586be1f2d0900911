"""Fixtures from the reference's own data directory (data/ of UnixJunkie/MMO,
BSD 3-Clause License, Copyright (c) 2024, Francois Berenger):

* ref_ligands.pqrs: the 48-atom ligand of data/docked.mol2, data/minimized.mol2
  and data/ligdecs.mol2 (one molecule in three poses), each converted to
  .pqrs by mmo_gb300.mol2, this repository's restatement of the reference's
  mol2pqrs (src/mol2pqrs.ml:10-43): atoms, charges, vdW radii, rotatable bonds
  with their rotation groups, topological distances.
* ref_receptor.pqrs: the protein of data/xtal.pdb (PDB entry 3A2J, the vitamin D
  receptor ligand-binding domain): its ATOM records (no waters, no bound
  ligand), element from columns 77-78.  The PDB file holds no partial
  charges, so the charges here follow a fixed rule (RULE below: a neutral
  backbone, charged side-chain ends) to give the Coulomb term something to sum.

    python tests/golden/make_ref_data.py <MMO checkout>
    (or MMO_REFERENCE_ROOT=<MMO checkout> python tests/golden/make_ref_data.py)

The outputs are committed; the tests read them and never the reference.  The
two CPU tests that regenerate them and run the reference's own .pqrs reader
need MMO_REFERENCE_ROOT and are skipped without it.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mmo_gb300 import mol2 as M2  # noqa: E402
from mmo_gb300.topology import Mol, write_pqrs  # noqa: E402

LIGANDS = ("docked.mol2", "minimized.mol2", "ligdecs.mol2")

# (residue or "*", atom name) -> charge; anything else 0
RULE = {("*", "N"): -0.3, ("*", "CA"): 0.3, ("*", "C"): 0.5, ("*", "O"): -0.5,
        ("*", "OXT"): -0.5, ("ASP", "OD1"): -0.5, ("ASP", "OD2"): -0.5,
        ("GLU", "OE1"): -0.5, ("GLU", "OE2"): -0.5, ("LYS", "NZ"): 1.0,
        ("ARG", "NH1"): 0.5, ("ARG", "NH2"): 0.5}
ELEMENTS = {"C": 6, "N": 7, "O": 8, "S": 16}


def receptor_from_pdb(path) -> Mol:
    xyz, anum, q = [], [], []
    with open(path) as f:
        for ln in f:
            if not ln.startswith("ATOM"):
                continue
            name, res = ln[12:16].strip(), ln[17:20].strip()
            el = ln[76:78].strip()
            xyz.append((float(ln[30:38]), float(ln[38:46]), float(ln[46:54])))
            anum.append(ELEMENTS[el])
            q.append(RULE.get((res, name), RULE.get(("*", name), 0.0)))
    xyz = np.array(xyz)
    anum = np.array(anum, np.int32)
    rad = np.array([M2.VDW_RADII[int(z)] for z in anum])
    return Mol("3A2J", xyz[:, 0].copy(), xyz[:, 1].copy(), xyz[:, 2].copy(), np.array(q), anum,
               rad)


ENV = "MMO_REFERENCE_ROOT"


def reference_root():
    """The MMO checkout to read the molecules from: the MMO_REFERENCE_ROOT
    environment variable, or None when it is not set."""
    return os.environ.get(ENV) or None


def main(ref, out=HERE):
    data = os.path.join(ref, "data")
    texts = []
    for fn in LIGANDS:
        for name, atoms, bonds in M2.read_mol2(os.path.join(data, fn)):
            texts.append(M2.ligand_pqrs_text(fn.split(".")[0] + "|" + name, atoms, bonds))
    with open(os.path.join(out, "ref_ligands.pqrs"), "w") as f:
        f.write("".join(texts))
    write_pqrs(os.path.join(out, "ref_receptor.pqrs"),
               [receptor_from_pdb(os.path.join(data, "xtal.pdb"))], receptor=True)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else reference_root()
    if not root:
        sys.exit("usage: make_ref_data.py <MMO checkout> (or set %s)" % ENV)
    main(root)
