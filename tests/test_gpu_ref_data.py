"""The reference's own molecules on the GPU against the FP64 oracle: the
48-atom ligand of data/docked.mol2, data/minimized.mol2 and data/ligdecs.mol2
(one molecule in three poses) in the 3A2J receptor of data/xtal.pdb, as
committed by tests/golden/make_ref_data.py.

* the batched energy and gradient of each pose and of poses perturbed about
  it (rigid moves, torsions), with the reference's physics and its variants,
  both pose maps, and the one-pose path;
* the closures ``ff0 prot`` (ene_inter_builder) and ``ene_intra``
  (ene_intra_builder; ff_score's per-ligand intra energy);
* interpolated scoring on grids built about the binding site;
* exhaustive rigid docking about the docked pose's centre;
* Monte Carlo chains from the docked pose;
* the pose map's coordinates (mmo_posed_coords), and the ff_score / ff_opt
  scripts on these molecules.

Tolerances are the scoring contract's: energies within 1e-5 of
max(|E64|, sum |pair energies|), gradients within 1e-4 of the largest
component; the poses here are mostly clash-free, so the first term counts."""
import os

import numpy as np
import pytest

from mmo_gb300 import grids as GR
from mmo_gb300 import synth
from contract import assert_energy, assert_grad, assert_ref, ref_batch
from test_ref_data import ref_molecules

pytestmark = pytest.mark.gpu

STEP = 0.5


@pytest.fixture(scope="module")
def ref():
    return ref_molecules()


def _poses(lig, n, seed, recenter):
    """n poses about the conformer as it is (pose 0 leaves it in place)."""
    rng = np.random.default_rng(seed)
    d = np.zeros((n, 6 + lig.nrb), np.float32)
    if recenter:
        d[:, :3] = lig.xyz().mean(axis=0)
    d[1:, :3] += rng.uniform(-0.4, 0.4, size=(n - 1, 3)).astype(np.float32)
    if recenter:  # rotations about the centroid
        d[1:, 3:6] = rng.uniform(-0.2, 0.2, size=(n - 1, 3))
    d[1:, 6:] = rng.uniform(-0.5, 0.5, size=(n - 1, lig.nrb))
    return d


@pytest.mark.parametrize("phys", [(0, 0, 0, 0), (1, 0, 0, 0), (0, 0, 1, 0), (0, 1, 0, 0)],
                         ids=["reference", "eps4r", "global", "lorentz-berthelot"])
@pytest.mark.parametrize("recenter", [False, True])
def test_ref_poses_match_oracle(oracle, scorer_factory, ref, phys, recenter):
    from mmo_gb300.ff import Physics

    rec, ligs = ref
    for k, lig in enumerate(ligs):
        s = scorer_factory(rec, lig, Physics(*phys))
        d = _poses(lig, 24, 10 + k, recenter)
        E, G, st = s.score_poses(d, grad=True, recenter=recenter)
        assert np.all(st == 0)
        system = synth.System(lig.name, rec, lig, d)
        r = ref_batch(oracle, system, d, grad=True, recenter=recenter, ph=oracle.physics(*phys))
        assert_ref(E, G, r, st)
        # one pose per call: the plain path
        E1, G1, _ = s.score_poses(d[:1], grad=True, recenter=recenter)
        assert_energy(E1, r.E[:1], r.S[:1])
        assert_grad(G1, r.G[:1], r.GA[:1])
    if phys == (0, 0, 0, 0) and not recenter:
        # the docked pose binds: its inter energy is favourable
        s = scorer_factory(rec, ligs[0])
        e, _, _ = s.score_poses(_poses(ligs[0], 1, 0, False), intra=False)
        assert e[0] < -5.0


def test_ref_closures_match_oracle(oracle, gpu_lib, ref):
    from oracle import np_twin as T

    from mmo_gb300.ff import ene_inter_builder, ene_intra_builder

    rec, ligs = ref
    ff0 = ene_inter_builder(rec)
    for lig in ligs:
        e64 = oracle.ene_inter(rec, lig)
        scale = T.ene_inter(rec.xyz(), rec.q, rec.anum, lig.xyz(), lig.q, lig.anum, absolute=True)
        assert_energy([ff0(lig)], [e64], [scale])
        intra = ene_intra_builder(lig.centered())
        ei64 = oracle.ene_intra(lig)
        si = T.ene_intra(lig.xyz(), lig.q, lig.anum, lig.interacting, absolute=True)
        assert_energy([intra(lig)], [ei64], [si])
        intra.scorer.close()
    ff0.scorer.close()


def _site_lattice(lig, margin=6.0):
    lo, hi = lig.xyz().min(axis=0) - margin, lig.xyz().max(axis=0) + margin
    return GR.lattice_from_box(STEP, lo, hi)


def test_ref_interpolated_scoring_matches_oracle(oracle, scorer_factory, ref):
    from test_gpu_grid import _corner_scale

    rec, ligs = ref
    types, per = GR.type2id(ligs)
    for lig, lt in zip(ligs, per):
        # about each pose: only data/docked.mol2 sits in the pocket, the other
        # two poses of the molecule lie near the origin
        origin, dims = _site_lattice(lig)
        s = scorer_factory(rec, lig)
        s.build_grids(STEP, dims, origin, types)
        g = s.grid_values()
        d = _poses(lig, 8, 3, False)
        E, _, st = s.score_poses(d, intra=False, grid=True)
        assert np.all(st == 0)
        for b in range(len(d)):
            xyz, _ = oracle.apply_config(lig, d[b].astype(np.float64), 0)
            e, off = oracle.ene_inter_interp(STEP, dims, g, xyz - origin, lt)
            assert not off
            sc = _corner_scale(g, lt, (xyz - origin) / STEP)
            assert abs(E[b] - e) <= 1e-6 * max(sc, 1e-300), (b, E[b], e)


def test_ref_exhaustive_docking_matches_oracle(oracle, scorer_factory, ref):
    rec, ligs = ref
    lig = ligs[0]
    origin, dims = _site_lattice(lig, margin=9.0)
    types, (lt,) = GR.type2id([lig])
    s = scorer_factory(rec, lig)
    s.build_grids(STEP, dims, origin, types)
    s.build_masks(rec.radius)
    g = s.grid_values()
    vdw, _ = s.mask_values()
    center, radius, step, nrot, k = lig.xyz().mean(axis=0), 1.0, 0.5, 48, 16
    res = s.dock_exhaustive(center, radius, step, nrot, topk=k, const_intra=0.0,
                            lig_radius=lig.radius)
    R = np.stack([oracle.so3_rotation(nrot, i) for i in range(nrot)])
    sc, _ = oracle.dock_scores(oracle.lattice(STEP, dims, origin), g, vdw, lig, lt, lig.radius,
                               center, radius, step, R, const_intra=0.0)
    ok = np.isfinite(sc)
    assert res["scored"] == ok.sum() > 0
    order = np.lexsort((np.arange(len(sc)), sc))[:min(k, ok.sum())]
    tol = 1e-6 * max(1.0, np.abs(sc[order]).max())
    assert np.allclose(res["scores"], sc[order], rtol=0, atol=tol)
    for t in range(len(order)):
        gap = min(abs(sc[order[t]] - sc[order[t - 1]]) if t else np.inf,
                  abs(sc[order[t + 1]] - sc[order[t]]) if t + 1 < len(order) else np.inf)
        if gap > 4 * tol:
            assert res["frames"][t] == order[t], t


@pytest.mark.parametrize("recenter", [False, True])
def test_ref_gradient_against_central_differences(oracle, scorer_factory, ref, recenter):
    """On the reference's complex, the GPU gradient against FP64 central
    differences with h = 1e-4 A / rad (the step of the benchmark's gradient
    check), Richardson-extrapolated with h / 2, on every component where the
    differences are accurate (tests/contract.py fd_check): most of them on
    these poses, which clash far less than random ones."""
    from contract import G_TOL, fd_check

    rec, ligs = ref
    for k, lig in enumerate(ligs):
        s = scorer_factory(rec, lig)
        d = _poses(lig, 24, 30 + k, recenter)
        _, G, st = s.score_poses(d, grad=True, recenter=recenter)
        assert np.all(st == 0)
        system = synth.System(lig.name, rec, lig, d)
        r = ref_batch(oracle, system, d, grad=True, recenter=recenter)
        flags = oracle.F_INTER | oracle.F_INTRA | (oracle.F_RECENTER if recenter else 0)
        _, F1, _ = oracle.score_batch(rec, lig, d, flags=flags, mode=2, eps=1e-4, nthreads=16)
        _, F2, _ = oracle.score_batch(rec, lig, d, flags=flags, mode=2, eps=5e-5, nthreads=16)
        err, trusted = fd_check(G, F1, F2, r.S, r.GA, 1e-4)
        assert trusted.mean() >= 0.8, (k, trusted.mean())
        assert err.max() <= G_TOL, (k, err.max())


@pytest.mark.parametrize("recenter", [False, True])
def test_posed_coordinates_match_oracle(oracle, scorer_factory, ref, recenter):
    """mmo_posed_coords: the pose map's atoms (double-float on the GPU)
    against Optim.apply_config / the MC map in FP64, to 1e-9 A."""
    rec, ligs = ref
    lig = ligs[0]
    s = scorer_factory(rec, lig)
    d = _poses(lig, 32, 7, recenter)
    d[16:, 3:6] = np.random.default_rng(1).uniform(-np.pi, np.pi, size=(16, 3))
    xyz, st = s.posed_coords(d, recenter=recenter)
    for b in range(len(d)):
        want, st64 = oracle.apply_config(lig, d[b].astype(np.float64),
                                         oracle.F_RECENTER if recenter else 0)
        assert st[b] == st64
        assert np.abs(xyz[b] - want).max() <= 1e-9, (b, np.abs(xyz[b] - want).max())
    if not recenter:
        assert np.abs(xyz[0] - lig.xyz()).max() <= 1e-12  # zero DOFs: the conformer as read


def test_ff_score_matches_oracle(oracle, gpu_lib, ref, tmp_path, capsys):
    """mmo_gb300.ff_score (src/ff_score.ml): E_intra of each ligand as read."""
    from oracle import np_twin as T

    from mmo_gb300 import ff_score as F
    from test_ref_data import GOLD

    _, ligs = ref
    res = F.ff_score(ligs)
    assert [n for n, _ in res] == [m.name for m in ligs]
    for (_, e), m in zip(res, ligs):
        e64 = oracle.ene_intra(m)
        sc = T.ene_intra(m.xyz(), m.q, m.anum, m.interacting, absolute=True)
        assert_energy([e], [e64], [sc])
    assert F.main([os.path.join(GOLD, "ref_ligands.pqrs")]) == 0
    out = capsys.readouterr().out.splitlines()
    assert len(out) == 3 and all(len(ln.split("\t")) == 2 for ln in out)


def test_ff_opt_lowers_the_energy(oracle, gpu_lib, ref, capsys):
    """mmo_gb300.ff_opt: L-BFGS on the adjoint's gradient lowers E_intra (and,
    against the receptor, E_inter + E_intra); the written conformer scores, in
    the oracle, the energy reported for it."""
    from mmo_gb300 import ff_opt as O
    from mmo_gb300.ff import UFFScorer
    from test_ref_data import GOLD

    rec, ligs = ref
    s = UFFScorer(0)
    try:
        for lig in ligs:
            s.set_ligand(lig)
            e, xyz = O.minimize(s, lig, iters=40)
            e0 = oracle.ene_intra(lig)
            assert e < e0 - 1e-3
            assert abs(oracle.ene_intra(lig.with_xyz(xyz)) - e) <= 1e-4 * max(1.0, abs(e))
        s.set_protein(rec)
        s.set_ligand(ligs[0])
        e, xyz = O.minimize(s, ligs[0], receptor=True, iters=40)
        e0 = oracle.ene_inter(rec, ligs[0]) + oracle.ene_intra(ligs[0])
        moved = ligs[0].with_xyz(xyz)
        assert e < e0 - 1e-3
        assert abs(oracle.ene_inter(rec, moved) + oracle.ene_intra(moved) - e) <= \
            1e-4 * max(1.0, abs(e))
    finally:
        s.close()
    assert O.main([os.path.join(GOLD, "ref_ligands.pqrs"), "--iters", "5"]) == 0
    out = capsys.readouterr().out.splitlines()
    assert len(out) == 3 * (2 + 48) and out[1].split(":")[-1]


def test_mc_chains_on_the_real_complex(oracle, scorer_factory, ref):
    """Monte Carlo chains (mmo_mc_run, CUDA graph, gradient-descent
    minimisation every 40 steps) from the docked pose of data/docked.mol2 in
    the 3A2J receptor: the best energies never exceed the start, the returned
    energies are the scorer's of the returned poses, and the final poses
    re-scored in FP64 agree within the scoring contract."""
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L
    from test_gpu_mc import _run

    rec, ligs = ref
    lig = ligs[0]
    sc = scorer_factory(rec, lig)
    d0 = _poses(lig, 32, 5, True)
    E_start, _, _ = sc.score_poses(d0, recenter=True)
    d, E, bd, bE, acc, st = _run(torch, sc, L, d0, 160, minimize_every=40, minimize_iters=8)
    assert np.all(np.isfinite(E)) and np.all(acc > 0)
    assert np.all(bE <= E_start)
    Er, _, _ = sc.score_poses(d, recenter=True)
    assert np.array_equal(Er, E)
    system = synth.System(lig.name, rec, lig, d)
    assert_ref(E, None, ref_batch(oracle, system, d, recenter=True))
