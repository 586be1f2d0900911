"""Conformer minimisation on the GPU, the role of the reference's ff_opt
(src/ff_opt.py: minimise each ligand's conformer, print it in .xyz format with
"name:energy" as its second line): here the energy is the scoring path's UFF
non-bonded one (the intra-ligand term, plus the inter term against a receptor
when one is given), minimised over the torsions (and, with a receptor, the six
rigid-body DOFs of the optimiser layout, src/optim.ml:19-22) by L-BFGS on the
gradient of the hand-written adjoint, through the torch.autograd.Function of
mmo_gb300.torch_ops.  The reference's script calls RDKit's full UFF instead.

    python -m mmo_gb300.ff_opt ligands.pqrs [--receptor receptor.pqrs]
"""
from __future__ import annotations

import argparse
import sys
import time

import numpy as np

from .ff_score import load_ligands
from .topology import ANUM_TO_SYMBOL, read_pqrs


def minimize(scorer, lig, receptor=False, iters=100):
    """(E, xyz float64 [L, 3]) of the minimised conformer of lig (the scorer's
    ligand); the starting conformer is lig's coordinates (zero DOFs)."""
    import torch

    from .torch_ops import uff_score

    nd = 6 + lig.nrb
    dev = torch.device("cuda", scorer.device)
    # the MC pose map (rotation about the centroid, translation to it), so that
    # the rigid-body DOFs move the ligand about where it is
    d0 = np.zeros((1, nd), np.float32)
    d0[0, :3] = lig.xyz().mean(axis=0)
    base = torch.from_numpy(d0).to(dev)
    d = torch.zeros((1, nd), dtype=torch.float32, device=dev, requires_grad=True)
    mask = torch.ones((1, nd), dtype=torch.float32, device=dev)
    if not receptor:
        mask[:, :6] = 0.0  # E_intra does not depend on the rigid-body DOFs
    opt = torch.optim.LBFGS([d], max_iter=iters, line_search_fn="strong_wolfe")
    best = [float("inf"), d0]

    def closure():
        opt.zero_grad()
        x = base + d * mask
        E = uff_score(x, scorer, inter=receptor, intra=True, recenter=True)
        e = float(E[0].detach())
        if e < best[0]:
            best[0], best[1] = e, x.detach().cpu().numpy()
        E.sum().backward()
        return E.sum()

    opt.step(closure)
    xyz, _ = scorer.posed_coords(best[1], recenter=True)
    return best[0], xyz[0]


def xyz_text(lig, e, xyz) -> str:
    """The reference's xyz_dump layout: atom count, "name:energy", one
    "element x y z" line per atom."""
    lines = ["%d" % lig.n, "%s:%g" % (lig.name, e)]
    lines += ["%s %g %g %g" % (ANUM_TO_SYMBOL[int(a)], *p) for a, p in zip(lig.anum, xyz)]
    return "\n".join(lines) + "\n"


def main(argv=None) -> int:
    from .ff import UFFScorer

    ap = argparse.ArgumentParser(description="minimise each ligand's conformer (UFF non-bonded)")
    ap.add_argument("input", help="ligands (.pqrs, or .mol2 with partial charges)")
    ap.add_argument("--receptor", help="receptor .pqrs: minimise E_inter + E_intra")
    ap.add_argument("--iters", type=int, default=100)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    t0 = time.time()
    ligs = load_ligands(args.input)
    s = UFFScorer(args.device)
    if args.receptor:
        (rec,) = read_pqrs(args.receptor)
        s.set_protein(rec)
    for lig in ligs:
        s.set_ligand(lig)
        e, xyz = minimize(s, lig, receptor=bool(args.receptor), iters=args.iters)
        sys.stdout.write(xyz_text(lig, e, xyz))
    s.close()
    dt = time.time() - t0
    print("%d molecules @ %.2fHz" % (len(ligs), len(ligs) / max(dt, 1e-9)), file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
