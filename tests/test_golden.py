"""Committed golden vectors (tests/golden/golden_small.npz, made by
tests/golden/make_golden.py): the oracle reproduces them on this host, and the
GPU path matches them within the scoring tolerances."""
import os

import numpy as np
import pytest

from mmo_gb300.topology import Mol

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_small.npz")
CASES = ["single_", "batch_", "mc_", "variant_"]


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN))


def case(g, prefix):
    p = g[prefix + "pocket"]
    pocket = Mol("pocket", p[:, 0], p[:, 1], p[:, 2], p[:, 3], g[prefix + "pocket_anum"])
    l = g[prefix + "lig"]
    off, atoms = g[prefix + "grp_off"], g[prefix + "grp_atoms"]
    groups = [atoms[off[t]:off[t + 1]] for t in range(len(off) - 1)]
    lig = Mol("lig", l[:, 0], l[:, 1], l[:, 2], l[:, 3], g[prefix + "lig_anum"], None,
              g[prefix + "lig_dists"], g[prefix + "rbonds"].reshape(-1, 2), groups)
    return pocket, lig


@pytest.mark.parametrize("prefix", CASES)
def test_oracle_reproduces_golden(oracle, golden, prefix):
    pocket, lig = case(golden, prefix)
    ph = oracle.physics(*golden[prefix + "physics"].tolist())
    E, G, st = oracle.score_batch(pocket, lig, golden[prefix + "poses"],
                                  flags=int(golden[prefix + "flags"]), mode=1, ph=ph)
    assert np.allclose(E, golden[prefix + "E"], rtol=1e-12, atol=0)
    assert np.allclose(G, golden[prefix + "G"], rtol=1e-9, atol=1e-9 * np.abs(G).max())
    assert np.array_equal(st, golden[prefix + "status"])


@pytest.mark.gpu
@pytest.mark.parametrize("prefix", CASES)
def test_gpu_matches_golden(scorer_factory, golden, prefix):
    from mmo_gb300.ff import Physics

    pocket, lig = case(golden, prefix)
    s = scorer_factory(pocket, lig, Physics(*golden[prefix + "physics"].tolist()))
    flags = int(golden[prefix + "flags"])
    E, G, st = s.score_poses(golden[prefix + "poses"], grad=True, recenter=bool(flags & 8))
    E64, G64 = golden[prefix + "E"], golden[prefix + "G"]
    assert (np.abs(E - E64) / np.abs(E64)).max() <= 1e-5
    gerr = np.abs(G - G64).max(axis=1) / np.abs(G64).max(axis=1)
    assert gerr.max() <= 1e-4
    assert np.array_equal(st, golden[prefix + "status"])
