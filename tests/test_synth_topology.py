"""Synthetic workload generators and the .pqrs topology (CPU only)."""
import numpy as np
import pytest

from mmo_gb300 import synth
from mmo_gb300.topology import (build_ligand, dist_matrix, read_pqrs, rot_group, rotatable_bonds,
                                write_pqrs)


def test_ligand_generator_spec():
    rng = np.random.default_rng(0)
    lig = synth.random_ligand(rng, 48, 8)
    assert lig.n == 48 and lig.nrb == 8
    xyz = lig.xyz()
    assert np.abs(xyz.mean(axis=0)).max() < 1e-12           # centred
    assert abs(lig.q.sum()) < 1e-12                           # net charge 0
    d = np.linalg.norm(xyz[:, None] - xyz[None], axis=2)
    assert (d[np.triu_indices(48, 1)] >= synth.MIN_SEP - 1e-9).all()
    for a, b in lig.bonds:
        assert abs(d[a, b] - synth.BOND) < 1e-9
    assert set(np.unique(lig.anum)) <= {1, 6, 7, 8, 16}
    deg = np.zeros(48, int)
    for a, b in lig.bonds:
        deg[a] += 1
        deg[b] += 1
    for t, (left, right) in enumerate(lig.rbonds):
        assert deg[left] > 1 and deg[right] > 1             # internal bonds only
        grp = set(lig.rgroups[t].tolist())
        assert right not in grp and left not in grp
        assert len(grp) + 1 <= 48 - len(grp) - 1             # smaller side


def test_pocket_generator_spec():
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(1)
    p = synth.random_pocket(rng, 3000, 15.0)
    xyz = p.xyz()
    assert p.n == 3000
    assert np.linalg.norm(xyz, axis=1).max() <= 15.0
    dmin, _ = cKDTree(xyz).query(xyz, k=2)
    assert dmin[:, 1].min() >= 1.2


def test_poses_layout():
    rng = np.random.default_rng(2)
    d = synth.random_poses(rng, 1000, 8, 4.0)
    assert d.dtype == np.float32 and d.shape == (1000, 14)
    assert np.abs(d[:, :3]).max() <= 4.0
    assert np.abs(d[:, 6:]).max() <= np.pi
    # Euler angles of rot.ml decompose reproduce the sampled rotation
    from oracle import np_twin as T

    q = synth.shoemake_quats(np.random.default_rng(3), 5)
    R = synth.quat_to_matrix(q)
    a, b, g = synth.decompose(R)
    for k in range(5):
        assert np.abs(T.rot_xyz(a[k], b[k], g[k]) - R[k]).max() < 1e-12


def test_generators_are_seeded():
    a = synth.pose_batch(n_poses=8, seed=5, n_pocket=500, radius=10.0)
    b = synth.pose_batch(n_poses=8, seed=5, n_pocket=500, radius=10.0)
    assert np.array_equal(a.poses, b.poses) and np.array_equal(a.pocket.x, b.pocket.x)
    assert np.array_equal(a.ligand.rbonds, b.ligand.rbonds)


def test_rotatable_bond_rules():
    # ring of 6 with a 3-atom tail: ring bonds and terminal bonds are not rotatable
    bonds = [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5), (5, 0), (0, 6), (6, 7), (7, 8)]
    rb = rotatable_bonds(9, bonds, [1.0] * len(bonds))
    assert rb == [(0, 6), (6, 7)]
    assert rotatable_bonds(9, bonds, [1.0] * 6 + [2.0, 1.0, 1.0]) == [(6, 7)]
    assert rot_group(9, bonds, (0, 6)) == {6, 7, 8}
    d = dist_matrix(9, bonds)
    assert d[0, 3] == 3 and d[8, 3] == 6 and d[1, 5] == 2


def test_disconnected_atom():
    with pytest.raises(ValueError):
        dist_matrix(3, [(0, 1)])


def test_pqrs_round_trip(tmp_path):
    rng = np.random.default_rng(6)
    lig = synth.random_ligand(rng, 20, 4)
    f = tmp_path / "lig.pqrs"
    write_pqrs(f, [lig])
    (back,) = read_pqrs(f)
    assert back.n == 20 and back.nrb == 4
    assert np.array_equal(back.rbonds, lig.rbonds)
    for g0, g1 in zip(lig.rgroups, back.rgroups):
        assert np.array_equal(np.sort(g0), np.sort(g1))
    assert np.array_equal(back.dists, lig.dists)
    assert np.array_equal(back.anum, lig.anum)
    assert np.abs(back.xyz() - lig.xyz()).max() < 1e-4  # %g has 6 significant digits
    p = synth.random_pocket(rng, 50, 6.0)
    write_pqrs(tmp_path / "rec.pqrs", [p], receptor=True)
    (rec,) = read_pqrs(tmp_path / "rec.pqrs")
    assert rec.n == 50 and rec.nrb == 0


def test_build_ligand_axis_orientation():
    xyz = np.array([[0, 0, 0], [1.5, 0, 0], [3.0, 0.5, 0], [4.5, 0, 0], [6, 0.5, 0.]])
    lig = build_ligand("c5", xyz, np.zeros(5), np.full(5, 6, np.int32),
                       [(0, 1), (1, 2), (2, 3), (3, 4)])
    # bonds (1,2) and (2,3) rotate; the right end is the group side's axis atom
    assert lig.rbonds.tolist() == [[2, 1], [2, 3]]
    assert [g.tolist() for g in lig.rgroups] == [[0], [4]]
