"""Score the synthetic pose-batch workload a few times with a fixed launch plan.

A small driver for profilers and quick checks: no tuning, no timing loop, one
line of output.  Example (4,096 poses of the 48-atom ligand against the
6,000-atom pocket, energy and gradient, cut-off sweep with 2 entries per lane):

    python -m mmo_gb300.run_workload --poses 4096 --repeat 4 --sweep cut-off \\
        --per-lane 2 --threads 768 --piece 256 --row-spacing 2.0
"""
from __future__ import annotations

import argparse

import numpy as np

from . import synth
from .ff import Physics, UFFScorer


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--poses", type=int, default=4096)
    ap.add_argument("--repeat", type=int, default=4)
    ap.add_argument("--sweep", choices=["cut-off", "full"], default="cut-off")
    ap.add_argument("--per-lane", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--piece", type=int, default=0)
    ap.add_argument("--chunks", type=int, default=0)
    ap.add_argument("--row-spacing", type=float, default=0.0)
    ap.add_argument("--dielectric", type=int, default=0)
    ap.add_argument("--energy-only", action="store_true")
    ap.add_argument("--grid-margin", type=float, default=None,
                    help="build the per-type grids (0.5 A lattice over the protein's box plus "
                         "this margin, mask sphere of 34 A) --repeat times, then score the poses "
                         "from them")
    ap.add_argument("--grid-kp", type=int, default=0, help="lattice points per lane (1, 2)")
    ap.add_argument("--plain", type=int, default=0,
                    help="score the first N poses one per call (the one-pose kernel), "
                         "--repeat times")
    ap.add_argument("--dock", action="store_true",
                    help="exhaustive docking of the 24-atom ligand in the 6,000-atom cavity site "
                         "(grids over the site's box + 6 A, masks, ROI r = 4 A at 0.5 A, 2,000 "
                         "rotations, top 64), --repeat times")
    args = ap.parse_args(argv)
    if args.dock:
        return _dock(args)

    s = synth.pose_batch(n_poses=args.poses, seed=1)
    sc = UFFScorer(0, Physics(args.dielectric, 0, 0, 0))
    sc.set_protein(s.pocket)
    sc.set_ligand(s.ligand)
    if args.grid_margin is not None:
        from . import grids as GR

        types, _ = GR.type2id([s.ligand])
        sc.set_grid_build(args.grid_kp)
        p = s.pocket.xyz()
        origin, dims = GR.lattice_from_box(GR.GRID_STEP, p.min(axis=0) - args.grid_margin,
                                           p.max(axis=0) + args.grid_margin)
        ms = [sc.build_grids(GR.GRID_STEP, dims, origin, types, mask_center=(0.0, 0.0, 0.0),
                             mask_radius=GR.roi_mask_radius(10.0)) for _ in range(args.repeat)]
        E, G, st = sc.score_poses(s.poses, grad=not args.energy_only, grid=True)
        print("grids %s x %d types  build ms %s  E[0] %.6e  status bits %d" %
              (dims, len(types), " ".join("%.3f" % m for m in ms), E[0],
               int(np.count_nonzero(st))))
        sc.close()
        return 0
    if args.plain:
        for _ in range(args.repeat):
            for b in range(args.plain):
                E, G, st = sc.score_poses(s.poses[b:b + 1], grad=not args.energy_only)
        print("plain: %d poses x %d, %d launch(es) per pose, E %.6e  status bits %d" %
              (args.plain, args.repeat, sc.last_launches(), E[0], int(np.count_nonzero(st))))
        sc.close()
        return 0
    if args.sweep == "cut-off":
        sc.set_cull(0, args.row_spacing, args.piece, args.per_lane)
        sc.set_tiles(0, args.threads, 0)
    else:
        sc.set_cull(1)
        sc.set_tiles(args.per_lane, args.threads, args.chunks)
    for _ in range(args.repeat):
        E, G, st = sc.score_poses(s.poses, grad=not args.energy_only)
    ev, al = sc.pair_count()
    print("poses %d  plan %s  pairs %.0f of %.0f  E[0] %.6e  status bits %d" %
          (len(E), sc.plan(), ev, al, E[0], int(np.count_nonzero(st))))
    sc.close()
    return 0


def _dock(args) -> int:
    from . import grids as GR

    site = synth.docking_site(seed=21, n_pocket=6000, r_in=8.0, r_out=20.0, n_atoms=24, n_rot=4)
    sc = UFFScorer(0)
    sc.set_protein(site.pocket)
    sc.set_ligand(site.ligand)
    types, _ = GR.type2id([site.ligand])
    p = site.pocket.xyz()
    origin, dims = GR.lattice_from_box(GR.GRID_STEP, p.min(axis=0) - 6.0, p.max(axis=0) + 6.0)
    sc.build_grids(GR.GRID_STEP, dims, origin, types)
    sc.build_masks(site.pocket.radius)
    for _ in range(args.repeat):
        r = sc.dock_exhaustive(np.zeros(3), 4.0, 0.5, 2000, topk=64,
                               lig_radius=site.ligand.radius)
    print("dock: %d poses, %d scored, best %.6f at %s rot %d, %.3f ms" %
          (r["poses"], r["scored"], r["best_score"], r["best_pos"], r["best_rot"], r["ms"]))
    sc.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
