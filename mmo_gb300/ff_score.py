"""The reference's ff_score (src/ff_score.ml:8-15) on the GPU: each ligand of a
.pqrs file (or of a .mol2 file, converted as mol2pqrs does) and its UFF
non-bonded intra-molecular energy, Mol.ene_intra_UFFNB_brute at the
coordinates read, without prior minimisation, printed as "name<TAB>energy"
(%g) like the reference; the rate on stderr.

    python -m mmo_gb300.ff_score ligands.pqrs
"""
from __future__ import annotations

import argparse
import sys
import time

from . import mol2 as M2
from .ff import Physics, UFFScorer
from .topology import read_pqrs


def load_ligands(path):
    """Ligands of a .pqrs file, or of a .mol2 file through the .pqrs converter
    (a ligand with an atom disconnected from the rest is skipped, as
    Mol2pqrs.process_ligand skips it)."""
    if not path.endswith(".mol2"):
        return read_pqrs(path)
    out = []
    for name, atoms, bonds in M2.read_mol2(path):
        if M2._connected(len(atoms), bonds):
            out.append(M2.to_mol(name, atoms, bonds))
        else:
            print("skipped %s: disconnected atom" % name, file=sys.stderr)
    return out


def ff_score(ligands, device=0, physics=Physics()):
    """[(name, E_intra)] of the ligands at their coordinates."""
    s = UFFScorer(device, physics)
    try:
        res = []
        for lig in ligands:
            s.set_ligand(lig)
            res.append((lig.name, s.ene_intra(lig)))
        return res
    finally:
        s.close()


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="UFF non-bonded E_intra of each ligand of a "
                                             ".pqrs or .mol2 file, without minimisation")
    ap.add_argument("input", help="ligands (.pqrs, or .mol2 with partial charges)")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    t0 = time.time()
    res = ff_score(load_ligands(args.input), args.device)
    for name, e in res:
        print("%s\t%g" % (name, e))
    dt = time.time() - t0
    print("%d molecules @ %.2fHz" % (len(res), len(res) / max(dt, 1e-9)), file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
