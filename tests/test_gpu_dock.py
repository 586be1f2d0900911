"""Binding-site clients on the GPU (include/mmo_dock.h) against the oracle.

Masks (Lds.vdW_volume, Lds.first_solvent_shell): equal to the oracle's point
for point.  Clash filters: the same bits as the oracle's tests per pose.
Exhaustive docking: the k best scores within 1e-6 (relative to the sum of
|per-atom terms|) of the oracle's, the same frames where the oracle's
scores are separated by more than that.  Placement: every placement inside the
ROI and free of heavy-atom clashes per the oracle, reproducible from the seed.
Desolvation: protein contributions within 1e-5 of the oracle's, per-pose
penalties within 1e-9 (FP64 on the same shell points)."""
import numpy as np
import pytest

from mmo_gb300 import grids as GR
from mmo_gb300 import synth

pytestmark = pytest.mark.gpu

STEP = 0.5


@pytest.fixture(scope="module")
def site():
    return synth.docking_site(seed=11, n_pocket=2500, r_in=7.5, r_out=15.0, n_atoms=14, n_rot=3)


@pytest.fixture(scope="module")
def lattice():
    return GR.lattice_from_box(STEP, (-18.0, -18.0, -18.0), (18.0, 18.0, 18.0))


def _lat(oracle, lattice):
    origin, dims = lattice
    return oracle.lattice(STEP, dims, origin)


def _scorer(scorer_factory, site, lattice):
    s = scorer_factory(site.pocket, site.ligand)
    types, (lt,) = GR.type2id([site.ligand])
    origin, dims = lattice
    s.build_grids(STEP, dims, origin, types)
    s.build_masks(site.pocket.radius)
    return s, types, lt


def test_masks_match_oracle(oracle, scorer_factory, site, lattice):
    s, _, _ = _scorer(scorer_factory, site, lattice)
    vdw, shell = s.mask_values()
    ov, osh = oracle.masks(_lat(oracle, lattice), site.pocket.xyz(), site.pocket.radius, 1.4)
    assert vdw.sum() > 0 and shell.sum() > 0
    assert np.array_equal(vdw, ov)
    assert np.array_equal(shell, osh)
    # loading them back gives the same state
    s.load_masks(ov, osh)
    v2, s2 = s.mask_values()
    assert np.array_equal(v2, ov) and np.array_equal(s2, osh)


def test_clash_bits_match_oracle(oracle, scorer_factory, site, lattice):
    from mmo_gb300 import lib as L

    s, _, _ = _scorer(scorer_factory, site, lattice)
    vdw, _ = s.mask_values()
    g = _lat(oracle, lattice)
    rng = np.random.default_rng(5)
    B = 96
    d = np.zeros((B, 6 + site.ligand.nrb), np.float32)
    d[:, :3] = rng.uniform(-6.0, 6.0, size=(B, 3))
    d[:, 3:6] = rng.uniform(-np.pi, np.pi, size=(B, 3))
    d[:, 6:] = rng.uniform(-np.pi, np.pi, size=(B, site.ligand.nrb))
    bits = s.clash_poses(d, recenter=True)
    seen = set()
    for b in range(B):
        xyz, _ = oracle.apply_config(site.ligand, d[b].astype(np.float64), oracle.F_RECENTER)
        want = ((L.CLASH_INTRA if oracle.intra_clash(xyz, site.ligand.anum,
                                                     site.ligand.interacting) else 0) |
                (L.CLASH_HEAVY if oracle.heavy_atom_clash(site.pocket, xyz, site.ligand.anum)
                 else 0) |
                (L.CLASH_GRID if oracle.protein_ligand_clash(g, vdw, xyz) else 0))
        assert bits[b] == want, (b, bits[b], want)
        seen.add(want)
    assert len(seen) >= 3  # clashing and free poses both occur
    only = s.clash_poses(d, tests=L.CLASH_HEAVY, recenter=True)
    assert np.array_equal(only, bits & L.CLASH_HEAVY)


def test_so3_rotations_match_oracle(oracle, gpu_lib):
    from mmo_gb300.ff import so3_rotations

    R = so3_rotations(37)
    for i in (0, 5, 36):
        assert np.allclose(R[i], oracle.so3_rotation(37, i), atol=1e-15)


def test_exhaustive_docking_matches_oracle(oracle, scorer_factory, site, lattice):
    s, types, lt = _scorer(scorer_factory, site, lattice)
    g = s.grid_values()
    vdw, _ = s.mask_values()
    center, radius, step, nrot, k = np.array([0.3, -0.2, 0.1]), 2.0, 0.5, 64, 24
    res = s.dock_exhaustive(center, radius, step, nrot, topk=k, const_intra=1.25,
                            lig_radius=site.ligand.radius)
    R = np.stack([oracle.so3_rotation(nrot, i) for i in range(nrot)])
    sc, dims = oracle.dock_scores(_lat(oracle, lattice), g, vdw, site.ligand, lt,
                                  site.ligand.radius, center, radius, step, R, const_intra=1.25)
    ok = np.isfinite(sc)
    assert res["scored"] == ok.sum() and res["poses"] == res["positions"] * nrot
    assert res["scored"] + res["clashed"] <= res["poses"]
    order = np.lexsort((np.arange(len(sc)), sc))[:min(k, ok.sum())]
    want_s, want_f = sc[order], order
    got_s, got_f = res["scores"], res["frames"]
    assert len(got_s) == len(want_s)
    tol = 1e-6 * max(1.0, np.abs(want_s).max())
    assert np.allclose(got_s, want_s, rtol=0, atol=tol)
    for t in range(len(want_s)):
        gap = min(abs(want_s[t] - want_s[t - 1]) if t else np.inf,
                  abs(want_s[t + 1] - want_s[t]) if t + 1 < len(want_s) else np.inf)
        if gap > 4 * tol:
            assert got_f[t] == want_f[t], t
    # the best pose decodes to the oracle's position and rotation
    p, r = divmod(int(want_f[0]), nrot)
    dim = dims[0]
    pos = center - radius + step * np.array([p % dim, (p // dim) % dim, p // dim ** 2])
    assert res["best_rot"] == r and np.allclose(res["best_pos"], pos)


def test_placement_is_clash_free_and_reproducible(oracle, scorer_factory, site, lattice):
    s, _, _ = _scorer(scorer_factory, site, lattice)
    c, r = np.array([0.5, 0.0, -0.5]), 3.0
    d, trials = s.place_in_roi(c, r, 40, seed=7)
    assert trials >= 40
    for b in range(len(d)):
        assert np.linalg.norm(d[b, :3] - c) < r + 1e-5
        xyz, _ = oracle.apply_config(site.ligand, d[b].astype(np.float64), oracle.F_RECENTER)
        assert not oracle.heavy_atom_clash(site.pocket, xyz, site.ligand.anum)
    d2, t2 = s.place_in_roi(c, r, 40, seed=7)
    assert np.array_equal(d, d2) and t2 == trials
    d3, _ = s.place_in_roi(c, r, 40, seed=8)
    assert not np.array_equal(d, d3)
    # the first 10 placements do not depend on how many are asked for
    d4, _ = s.place_in_roi(c, r, 10, seed=7)
    assert np.array_equal(d4, d[:10])


def test_desolvation_matches_oracle(oracle, scorer_factory, site, lattice):
    s, _, _ = _scorer(scorer_factory, site, lattice)
    _, shell = s.mask_values()
    g = _lat(oracle, lattice)
    c, r = np.array([0.0, 0.0, 0.0]), 10.0
    got = s.protein_desolv(c, r)
    want = oracle.protein_desolv(g, site.pocket, shell, c, r)
    assert np.array_equal(got > 0, want > 0)
    assert np.allclose(got, want, rtol=1e-5, atol=1e-12)
    s.set_ligand_radii(site.ligand.radius)
    rng = np.random.default_rng(2)
    B = 8
    d = np.zeros((B, 6 + site.ligand.nrb), np.float32)
    d[:, :3] = rng.uniform(-2.0, 2.0, size=(B, 3))
    d[:, 3:6] = rng.uniform(-np.pi, np.pi, size=(B, 3))
    prot, lig, st = s.desolvation_poses(d, recenter=True)
    assert np.all(st == 0)
    for b in range(B):
        xyz, _ = oracle.apply_config(site.ligand, d[b].astype(np.float64), oracle.F_RECENTER)
        wp, wl = oracle.desolvation_penalty(g, got, shell, xyz, site.ligand.q, site.ligand.radius)
        assert prot[b] == pytest.approx(wp, rel=1e-9, abs=1e-12)
        assert lig[b] == pytest.approx(wl, rel=1e-6, abs=1e-12)
    assert np.any(prot > 0) and np.any(lig > 0)
