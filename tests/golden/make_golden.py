"""Writes tests/golden/golden_small.npz: seeded small systems with their FP64
oracle energies, analytic gradients and statuses.

The reference ships no golden energies (and its OCaml toolchain is absent), so
these vectors come from the oracle; they pin the oracle and the GPU path
against regressions, while the oracle itself is pinned by the known-answer
tests and the reference's dihedral vectors in tests/test_oracle.py.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mmo_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402


def pack(prefix, s, out, physics=(0, 0, 0, 0), flags=3):
    lig, p = s.ligand, s.pocket
    off, atoms = lig.group_arrays()
    out[prefix + "pocket"] = np.stack([p.x, p.y, p.z, p.q], axis=1)
    out[prefix + "pocket_anum"] = p.anum
    out[prefix + "lig"] = np.stack([lig.x, lig.y, lig.z, lig.q], axis=1)
    out[prefix + "lig_anum"] = lig.anum
    out[prefix + "lig_dists"] = lig.dists
    out[prefix + "rbonds"] = lig.rbonds
    out[prefix + "grp_off"] = off
    out[prefix + "grp_atoms"] = atoms
    out[prefix + "poses"] = s.poses
    out[prefix + "physics"] = np.array(physics, np.int32)
    out[prefix + "flags"] = np.array(flags, np.int32)
    E, G, st = O.score_batch(p, lig, s.poses, flags=flags, mode=1, ph=O.physics(*physics))
    out[prefix + "E"] = E
    out[prefix + "G"] = G
    out[prefix + "status"] = st


def main():
    out = {}
    s0 = synth.single_pose(seed=0)
    pack("single_", s0, out)
    s1 = synth.pose_batch(n_poses=24, seed=21, n_atoms=30, n_rot=6, n_pocket=1000, radius=11.0)
    pack("batch_", s1, out)
    pack("mc_", s1, out, flags=3 | O.F_RECENTER)
    pack("variant_", s1, out, physics=(1, 1, 1, 1))
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)


if __name__ == "__main__":
    main()
