"""Parity of the CUDA path (through the C ABI) with the FP64 oracle, under the
scoring contract of tests/contract.py: energies within 1e-5 relative (outside
cancellation cases, and within 1e-5 of max(|E64|, S) everywhere), gradient
components within 1e-4 relative (with the floor at 1% of each component's own
terms)."""
import numpy as np
import pytest

from contract import E_TOL, assert_energy, assert_grad, assert_ref, ref_batch
from mmo_gb300 import synth
from mmo_gb300.topology import Mol

pytestmark = pytest.mark.gpu


def _posed(oracle, lig, conf, recenter=False):
    xyz, st = oracle.apply_config(lig, np.asarray(conf, np.float64),
                                  oracle.F_RECENTER if recenter else 0)
    return xyz, st


@pytest.fixture(scope="module")
def small():
    return synth.single_pose(seed=0)


@pytest.fixture(scope="module")
def batch():
    return synth.pose_batch(n_poses=256, seed=1)


# -- plain drop-ins (Mol.t -> float) ----------------------------------------------

@pytest.mark.parametrize("phys", [(0, 0, 0, 0), (0, 0, 1, 0), (1, 0, 0, 0), (0, 1, 0, 1),
                                  (1, 1, 1, 1)])
def test_plain_ene_inter_and_intra(oracle, scorer_factory, small, phys):
    from mmo_gb300.ff import Physics
    from oracle import np_twin as T

    ph = oracle.physics(*phys)
    s = scorer_factory(small.pocket, small.ligand, Physics(*phys))
    xyz, _ = _posed(oracle, small.ligand, small.poses[0])
    lig = small.ligand.with_xyz(xyz)
    e = s.ene_inter(lig)
    assert s.last_launches() == 1  # the pair partials and their total in one launch
    e64 = oracle.ene_inter(small.pocket, small.ligand, xyz, ph=ph)
    scale = T.ene_inter(small.pocket.xyz(), small.pocket.q, small.pocket.anum, xyz, lig.q,
                        lig.anum, shifted=phys[2] == 0, dielectric=phys[0], absolute=True)
    assert_energy(np.array([e]), np.array([e64]), np.array([scale]))
    ei = s.ene_intra(lig)
    assert s.last_launches() == 1
    ei64 = oracle.ene_intra(small.ligand, xyz, ph=ph)
    si = T.ene_intra(xyz, lig.q, lig.anum, lig.interacting, dielectric=phys[0], absolute=True)
    assert_energy(np.array([ei]), np.array([ei64]), np.array([si]))


@pytest.mark.parametrize("phys", [(0, 0, 0, 0), (1, 0, 1, 0), (0, 1, 0, 1)])
def test_plain_ene_inter_parts(oracle, scorer_factory, small, phys):
    """The electrostatic and van der Waals parts (ene_inter_UFF_shifted_bst_
    components) against the oracle's, each within 1e-5 of its own sum of
    |terms|; their sum is the energy of mmo_ene_inter; one launch."""
    from mmo_gb300.ff import Physics
    from oracle import np_twin as T

    ph = oracle.physics(*phys)
    s = scorer_factory(small.pocket, small.ligand, Physics(*phys))
    for k in range(3):
        xyz, _ = _posed(oracle, small.ligand, small.poses[0] if k == 0 else
                        np.concatenate([np.full(3, 0.7 * k), small.poses[0][3:]]))
        lig = small.ligand.with_xyz(xyz)
        el, lj = s.ene_inter_parts(lig)
        assert s.last_launches() == 1
        el64, lj64 = oracle.ene_inter_parts(small.pocket, small.ligand, xyz, ph=ph)
        scale = T.ene_inter(small.pocket.xyz(), small.pocket.q, small.pocket.anum, xyz, lig.q,
                            lig.anum, shifted=phys[2] == 0, dielectric=phys[0], absolute=True)
        assert abs(el - el64) <= E_TOL * scale and abs(lj - lj64) <= E_TOL * scale
        e = s.ene_inter(lig)
        assert abs((el + lj) - e) <= 1e-6 * scale


def test_plain_closures_match_reference_call_shape(oracle, gpu_lib, small):
    from mmo_gb300.ff import ene_inter_builder, ene_intra_builder

    xyz, _ = _posed(oracle, small.ligand, small.poses[0])
    lig = small.ligand.with_xyz(xyz)
    ene_inter = ene_inter_builder(small.pocket, "Bst")
    ene_intra = ene_intra_builder(small.ligand)
    e = ene_inter(lig) + ene_intra(lig)
    e64 = oracle.ene_inter(small.pocket, small.ligand, xyz) + oracle.ene_intra(small.ligand, xyz)
    assert abs(e - e64) <= E_TOL * abs(e64)
    rigid = ene_intra_builder(small.ligand, tweak_rbonds=False)
    assert rigid(lig) == pytest.approx(oracle.ene_intra(small.ligand), rel=1e-5)
    ene_inter.scorer.close()
    ene_intra.scorer.close()
    rigid.scorer.close()


# -- one pose per launch (plain path of mmo_score_poses) ---------------------------

@pytest.mark.parametrize("recenter", [False, True])
def test_single_pose_energy_gradient(oracle, scorer_factory, small, recenter):
    s = scorer_factory(small.pocket, small.ligand)
    E, G, st = s.score_poses(small.poses, grad=True, recenter=recenter)
    ref = ref_batch(oracle, small, small.poses, grad=True, recenter=recenter)
    assert_ref(E, G, ref, st)


@pytest.mark.parametrize("grad,recenter,phys", [(True, False, (0, 0, 0, 0)),
                                                 (True, True, (1, 1, 1, 1)),
                                                 (False, False, (0, 0, 1, 0)),
                                                 (True, False, (1, 0, 0, 0)),
                                                 (False, True, (0, 1, 1, 1))])
def test_one_pose_is_one_launch(oracle, scorer_factory, batch, grad, recenter, phys):
    """One pose with the pair terms is a single launch (k_one_pose: every CTA
    rebuilds the pose and sums its protein atoms' pair terms, the last CTA to
    arrive adds the partials in CTA order and finishes the pose).  Twenty-four
    calls in a row, each held to the contract: every launch leaves the
    arrival count at zero for the next."""
    from mmo_gb300.ff import Physics

    s = scorer_factory(batch.pocket, batch.ligand, Physics(*phys))
    d = batch.poses[:24]
    ref = ref_batch(oracle, batch, d, grad=grad, recenter=recenter, ph=oracle.physics(*phys))
    E, G, st = [], [], []
    for b in range(len(d)):
        e, g, t = s.score_poses(d[b:b + 1], grad=grad, recenter=recenter)
        assert s.last_launches() == 1
        E.append(e[0])
        st.append(t[0])
        if grad:
            G.append(g[0])
    assert_ref(np.array(E), np.array(G) if grad else None, ref, np.array(st))


def _nested(lig) -> bool:
    """The nested-group rule of mmo_set_ligand: every two groups nested or
    disjoint; an inner group's axis inside its outer group or on the outer
    axis; no axis atom of one of two disjoint groups inside the other."""
    G = [set(int(a) for a in g) for g in lig.rgroups]
    B = [tuple(int(v) for v in b) for b in lig.rbonds]
    for t in range(lig.nrb):
        for u in range(lig.nrb):
            if t == u:
                continue
            (tl, tr), (ul, ur) = B[t], B[u]
            if not (G[t] & G[u]):
                if ul in G[t] or ur in G[t]:
                    return False
            elif G[u] <= G[t]:
                if not all(a in G[t] or a in (tl, tr) for a in (ul, ur)):
                    return False
            elif not G[t] <= G[u]:
                return False
    return True


def _crossing_ligand(lig):
    """The ligand with one rotatable bond's group moved to the bond's other
    side (axis reversed): a valid MMO group assignment whose groups are no
    longer nested, so the pose map takes the torsions in bond order and the
    gradient the reverse pass."""
    import dataclasses

    n = lig.n
    for t in sorted(range(lig.nrb), key=lambda k: len(lig.rgroups[k])):
        left, right = (int(v) for v in lig.rbonds[t])
        side = set(int(a) for a in lig.rgroups[t]) | {right}
        rb = lig.rbonds.copy()
        rb[t] = (right, left)
        groups = list(lig.rgroups)
        groups[t] = np.asarray(sorted(set(range(n)) - side - {left}), np.int32)
        flipped = dataclasses.replace(lig, rbonds=rb, rgroups=groups)
        if not _nested(flipped):
            return flipped
    raise AssertionError("no flip makes the groups cross")


@pytest.mark.parametrize("recenter", [False, True])
def test_groups_not_nested(oracle, scorer_factory, batch, recenter):
    """A ligand whose rotation groups cross (one group moved to its bond's other
    side): the batched path (bond-order rebuild with records, reverse pass) and
    the one-pose kernel (finishing through the work buffers) against the oracle."""
    assert _nested(batch.ligand)
    lig = _crossing_ligand(batch.ligand)
    d = batch.poses[:64]
    sysm = synth.System("crossing", batch.pocket, lig, d)
    s = scorer_factory(batch.pocket, lig)
    ref = ref_batch(oracle, sysm, d, grad=True, recenter=recenter)
    E, G, st = s.score_poses(d, grad=True, recenter=recenter)
    assert_ref(E, G, ref, st)
    for b in range(0, 64, 9):
        E1, G1, st1 = s.score_poses(d[b:b + 1], grad=True, recenter=recenter)
        assert s.last_launches() == 1
        assert_energy(E1, ref.E[b:b + 1], ref.S[b:b + 1])
        assert_grad(G1, ref.G[b:b + 1], ref.GA[b:b + 1])
        assert st1[0] == ref.st[b]


# -- batched ------------------------------------------------------------------------

def test_batched_energy(oracle, scorer_factory, batch):
    s = scorer_factory(batch.pocket, batch.ligand)
    E, _, st = s.score_poses(batch.poses)
    assert_ref(E, None, ref_batch(oracle, batch, batch.poses), st)


@pytest.mark.parametrize("recenter", [False, True])
def test_batched_energy_gradient(oracle, scorer_factory, batch, recenter):
    s = scorer_factory(batch.pocket, batch.ligand)
    d = batch.poses[:128]
    E, G, st = s.score_poses(d, grad=True, recenter=recenter)
    assert_ref(E, G, ref_batch(oracle, batch, d, grad=True, recenter=recenter), st)


@pytest.mark.parametrize("inter,intra", [(True, False), (False, True)])
def test_batched_terms_separately(oracle, scorer_factory, batch, inter, intra):
    s = scorer_factory(batch.pocket, batch.ligand)
    d = batch.poses[:64]
    E, G, _ = s.score_poses(d, inter=inter, intra=intra, grad=True)
    assert_ref(E, G, ref_batch(oracle, batch, d, grad=True, inter=inter, intra=intra))


def test_pairs_within_cutoff_count(oracle, scorer_factory, batch):
    """mmo_diag_pairs_within (the roofline's pairs within 12 A) against a count
    from the oracle's FP64 posed coordinates; the sweep's counted pairs are at
    least as many (every pair within 12 A passes the box test)."""
    s = scorer_factory(batch.pocket, batch.ligand)
    d = batch.poses[:16]
    s.score_poses(d, grad=True)
    n12 = s.pairs_within(12.0)
    p = batch.pocket.xyz()
    want = 0
    for conf in d:
        xyz, _ = _posed(oracle, batch.ligand, conf)
        d2 = ((xyz[:, None, :] - p[None, :, :]) ** 2).sum(-1)
        want += int(np.count_nonzero(d2 < 144.0))
    assert abs(n12 - want) <= 1e-6 * want + 2  # a pair at 12 A to within rounding
    ev, al = s.pair_count()
    assert n12 <= ev <= al


@pytest.mark.parametrize("phys", [(1, 0, 0, 0), (0, 1, 1, 1), (1, 1, 1, 0)])
def test_batched_physics_variants(oracle, scorer_factory, batch, phys):
    from mmo_gb300.ff import Physics

    s = scorer_factory(batch.pocket, batch.ligand, Physics(*phys))
    d = batch.poses[:64]
    E, G, _ = s.score_poses(d, grad=True)
    assert_ref(E, G, ref_batch(oracle, batch, d, grad=True, ph=oracle.physics(*phys)))


@pytest.mark.parametrize("kp,threads,chunks", [(1, 256, 0), (2, 512, 3), (4, 512, 1),
                                               (4, 256, 17), (2, 256, 64)])
def test_tile_shapes_agree(scorer_factory, batch, kp, threads, chunks):
    s = scorer_factory(batch.pocket, batch.ligand)
    s.set_cull(mode=1)  # the full sweep, whose tiles these are
    d = batch.poses[:200]
    E0, G0, _ = s.score_poses(d, grad=True)
    s.set_tiles(kp, threads, chunks)
    E1, G1, _ = s.score_poses(d, grad=True)
    assert np.abs(E1 - E0).max() <= 1e-6 * np.abs(E0).max()
    assert np.abs(G1 - G0).max() <= 1e-5 * np.abs(G0).max()


# -- cut-off sweep of the shifted form ----------------------------------------------

@pytest.mark.parametrize("diel", [0, 1])
def test_cull_matches_full_sweep(scorer_factory, batch, diel):
    from mmo_gb300.ff import Physics

    s = scorer_factory(batch.pocket, batch.ligand, Physics(diel, 0, 0, 0))
    d = batch.poses
    E0, G0, st0 = s.score_poses(d, grad=True)
    s.set_cull(mode=1)
    E1, G1, st1 = s.score_poses(d, grad=True)
    assert np.array_equal(st0, st1)
    assert np.abs(E1 - E0).max() <= 1e-6 * np.abs(E0).max()
    err = np.abs(G1 - G0).max(axis=1) / np.abs(G0).max(axis=1)
    assert err.max() <= 1e-5


@pytest.mark.parametrize("h,piece,kp", [(1.0, 256, 4), (2.0, 1024, 2), (3.0, 0, 1),
                                        (0.5, 64, 4), (1.5, 100000, 2)])
def test_cull_parameters_agree(oracle, scorer_factory, batch, h, piece, kp):
    s = scorer_factory(batch.pocket, batch.ligand)
    d = batch.poses[:96]
    E0, G0, _ = s.score_poses(d, grad=True)
    s.set_cull(0, h, piece, kp)
    E1, G1, _ = s.score_poses(d, grad=True)
    assert np.abs(E1 - E0).max() <= 1e-6 * np.abs(E0).max()
    assert (np.abs(G1 - G0).max(axis=1) / np.abs(G0).max(axis=1)).max() <= 1e-5
    assert_ref(E1[:24], G1[:24], ref_batch(oracle, batch, d[:24], grad=True))


def test_cull_result_independent_of_grouping(scorer_factory, batch):
    """A pose's energy and gradient do not depend on the other poses of the
    batch: the cut-off sweep groups entries by position, and a reordered or
    smaller batch forms other groups, but skipped pairs add exact zeros and the
    partial sums break at fixed protein rows."""
    s = scorer_factory(batch.pocket, batch.ligand)
    d = batch.poses
    E, G, _ = s.score_poses(d, grad=True)
    perm = np.random.default_rng(5).permutation(len(d))
    Ep, Gp, _ = s.score_poses(d[perm], grad=True)
    assert np.array_equal(Ep, E[perm]) and np.array_equal(Gp, G[perm])
    Es, Gs, _ = s.score_poses(d[17:50], grad=True)
    assert np.array_equal(Es, E[17:50]) and np.array_equal(Gs, G[17:50])


@pytest.mark.parametrize("P", [9000, 13000])
def test_cull_large_pocket_against_oracle(oracle, scorer_factory, P):
    """Pockets beyond the shared-memory copy (about 6,500 atoms) run the
    cut-off sweep with the protein read from global memory: every pose under
    the scoring contract, and the full sweep agrees."""
    rng = np.random.default_rng(P)
    lig = synth.random_ligand(rng, 48, 8)
    pocket = synth.random_pocket(rng, P, 18.0 * (P / 6000.0) ** (1.0 / 3.0))
    d = synth.random_poses(rng, 384, lig.nrb, 4.0)
    sysm = synth.System("big", pocket, lig, d)
    s = scorer_factory(pocket, lig)
    E, G, st = s.score_poses(d, grad=True)
    plan = s.plan()
    assert plan["sweep"] == "cut-off" and plan["protein"] == "global memory", plan
    assert_ref(E, G, ref_batch(oracle, sysm, d, grad=True), st)
    s.set_cull(mode=1)
    E1, G1, st1 = s.score_poses(d, grad=True)
    assert np.array_equal(st, st1)
    assert np.abs(E1 - E).max() <= 1e-6 * np.abs(E).max()


def test_cull_protein_in_global_memory_same_bits(scorer_factory, batch):
    """The cut-off sweep reading the protein from global memory (mode 2) gives
    the bits of the sweep staging it in shared memory."""
    s = scorer_factory(batch.pocket, batch.ligand)
    E0, G0, st0 = s.score_poses(batch.poses, grad=True)
    assert s.plan()["protein"] == "shared memory"
    s.set_cull(mode=2)
    E1, G1, st1 = s.score_poses(batch.poses, grad=True)
    assert s.plan()["protein"] == "global memory"
    assert np.array_equal(E0, E1) and np.array_equal(G0, G1) and np.array_equal(st0, st1)


def test_cull_groups_out_of_reach(scorer_factory, batch):
    """Poses far from the pocket: the broad phase lists no protein piece for
    their entry groups, whose inter energies and forces are exact zeros; in a
    batch mixed with near poses the near ones keep their bits."""
    s = scorer_factory(batch.pocket, batch.ligand)
    far = batch.poses[:200].copy()
    far[:, :3] += 200.0
    E, G, st = s.score_poses(far, grad=True)
    Ei, Gi, _ = s.score_poses(far, inter=False, grad=True)
    assert np.array_equal(E, Ei) and np.array_equal(G, Gi)
    mixed = np.concatenate([far[:100], batch.poses[:100]])
    Em, Gm, _ = s.score_poses(mixed, grad=True)
    En, Gn, _ = s.score_poses(batch.poses[:100], grad=True)
    assert np.array_equal(Em[100:], En) and np.array_equal(Gm[100:], Gn)
    assert np.array_equal(Em[:100], E[:100])


def test_cull_non_finite_pose(scorer_factory, batch):
    s = scorer_factory(batch.pocket, batch.ligand)
    d = batch.poses[:64].copy()
    E0, G0, _ = s.score_poses(d, grad=True)
    d[5, 0] = np.nan
    E, G, st = s.score_poses(d, grad=True, inter=True, intra=False)
    assert np.isnan(E[5]) and (st[5] & 2)
    E1, _, _ = s.score_poses(batch.poses[:64], grad=True, inter=True, intra=False)
    keep = np.arange(64) != 5
    assert np.array_equal(E[keep], E1[keep])


@pytest.mark.parametrize("sweep", ["cut-off", "full"])
def test_energy_same_with_and_without_gradient(scorer_factory, batch, sweep):
    """Asking for the gradient does not change the energies, bit for bit, in
    the batched and the one-pose paths, with either pose map."""
    s = scorer_factory(batch.pocket, batch.ligand)
    if sweep == "full":
        s.set_cull(mode=1)
    for rc in (False, True):
        for d in (batch.poses[:100], batch.poses[:1]):
            E0, _, st0 = s.score_poses(d, recenter=rc)
            E1, _, st1 = s.score_poses(d, grad=True, recenter=rc)
            assert np.array_equal(E0, E1) and np.array_equal(st0, st1)


def test_deterministic(scorer_factory, batch):
    s = scorer_factory(batch.pocket, batch.ligand)
    a = s.score_poses(batch.poses, grad=True)
    b = s.score_poses(batch.poses, grad=True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_page_locked_buffers_give_the_same_results(scorer_factory, batch):
    """mmo_score_poses copies page-locked caller buffers by DMA directly, and
    other host memory through its staging buffers: the same bits either way,
    for inputs and outputs page-locked or not, with and without the gradient."""
    torch = pytest.importorskip("torch")
    s = scorer_factory(batch.pocket, batch.ligand)
    d = batch.poses[:300]
    B, nd = d.shape
    E0, G0, st0 = s.score_poses(d, grad=True)
    pin_d = torch.from_numpy(np.ascontiguousarray(d)).pin_memory().numpy()
    out = (torch.zeros(B, dtype=torch.float64).pin_memory().numpy(),
           torch.zeros((B, nd), dtype=torch.float32).pin_memory().numpy(),
           torch.zeros(B, dtype=torch.int32).pin_memory().numpy())
    for dofs in (d, pin_d):
        E, G, st = s.score_poses(dofs, grad=True, out=out)
        assert E is out[0] and G is out[1] and st is out[2]
        assert np.array_equal(E, E0) and np.array_equal(G, G0) and np.array_equal(st, st0)
        E1, _, st1 = s.score_poses(dofs, out=(np.zeros(B), None, np.zeros(B, np.int32)))
        assert np.array_equal(E1, E0) and np.array_equal(st1, st0)


def test_plain_and_batched_agree(scorer_factory, batch):
    s = scorer_factory(batch.pocket, batch.ligand)
    d = batch.poses[:40]
    Eb, Gb, _ = s.score_poses(d, grad=True)
    for b in range(0, 40, 7):
        E1, G1, _ = s.score_poses(d[b:b + 1], grad=True)
        assert abs(E1[0] - Eb[b]) <= 1e-6 * abs(Eb[b])
        assert np.abs(G1[0] - Gb[b]).max() <= 1e-5 * np.abs(Gb[b]).max()


# -- edge cases ---------------------------------------------------------------------

def test_edge_single_atom_ligand(oracle, scorer_factory, small):
    lig = Mol("one", np.zeros(1), np.zeros(1), np.zeros(1), np.array([0.4]),
              np.array([8], np.int32), None, np.zeros((1, 1), np.int32))
    s = scorer_factory(small.pocket, lig)
    d = np.array([[0.5, -1.0, 2.0, 0.1, 0.2, 0.3], [30.0, 0, 0, 0, 0, 0]], np.float32)
    E, G, st = s.score_poses(d, grad=True)
    sysm = synth.System("one", small.pocket, lig, d)
    ref = ref_batch(oracle, sysm, d, grad=True)
    assert_energy(E[:1], ref.E[:1], ref.S[:1])
    assert_grad(G[:1], ref.G[:1], ref.GA[:1])
    assert E[1] == 0.0 and np.all(G[1] == 0.0)  # beyond the 12 A cutoff


@pytest.mark.parametrize("case", ["one-atom ligand", "rigid ligand", "one-atom pocket"])
def test_one_pose_edges(oracle, scorer_factory, small, case):
    """The one-pose kernel at its edges, one pose per call against the oracle:
    L = 1 (every thread of a CTA on one ligand atom), nrb = 0 (no torsions, no
    intra terms to straddle), P = 1 (a single pair CTA)."""
    rng = np.random.default_rng(12)
    if case == "one-atom ligand":
        lig = Mol("one", np.zeros(1), np.zeros(1), np.zeros(1), np.array([0.4]),
                  np.array([8], np.int32), None, np.zeros((1, 1), np.int32))
        pocket = small.pocket
        d = np.array([[0.5, -1.0, 2.0, 0.1, 0.2, 0.3], [3.0, 2.0, -1.0, 1.0, 0.5, -2.0]],
                     np.float32)
    elif case == "rigid ligand":
        lig = synth.random_ligand(rng, 20, 0)
        pocket = small.pocket
        d = synth.random_poses(rng, 6, 0, 2.0)
    else:
        lig = small.ligand
        pocket = synth.random_pocket(rng, 1, 1.0)
        d = small.poses[:1].repeat(3, axis=0)
        d[1, :3] += 1.5
        d[2, :3] -= 2.0
    sysm = synth.System(case, pocket, lig, d)
    s = scorer_factory(pocket, lig)
    ref = ref_batch(oracle, sysm, d, grad=True)
    for b in range(len(d)):
        E1, G1, st1 = s.score_poses(d[b:b + 1], grad=True)
        assert s.last_launches() == 1
        assert_energy(E1, ref.E[b:b + 1], ref.S[b:b + 1])
        assert_grad(G1, ref.G[b:b + 1], ref.GA[b:b + 1])
        assert st1[0] == ref.st[b]


def test_edge_max_ligand_and_two_slices(oracle, scorer_factory):
    rng = np.random.default_rng(4)
    lig = synth.random_ligand(rng, 128, 32)
    pocket = synth.random_pocket(rng, 13000, 23.0)  # above one shared-memory slice
    d = synth.random_poses(rng, 40, lig.nrb, 4.0)
    sysm = synth.System("big", pocket, lig, d)
    s = scorer_factory(pocket, lig)
    E, G, st = s.score_poses(d, grad=True)
    ref = ref_batch(oracle, sysm, d, grad=True)
    assert_ref(E, G, ref, st)
    # one pose per call: the one-pose finishing CTA at its largest shared memory
    for b in (0, 7):
        E1, G1, st1 = s.score_poses(d[b:b + 1], grad=True)
        assert_energy(E1, ref.E[b:b + 1], ref.S[b:b + 1])
        assert_grad(G1, ref.G[b:b + 1], ref.GA[b:b + 1])
        assert st1[0] == ref.st[b]


def test_edge_rigid_ligand_and_tiny_pocket(oracle, scorer_factory):
    rng = np.random.default_rng(5)
    lig = synth.random_ligand(rng, 20, 0)
    pocket = synth.random_pocket(rng, 1, 1.0)
    d = synth.random_poses(rng, 33, 0, 2.0)
    sysm = synth.System("rigid", pocket, lig, d)
    s = scorer_factory(pocket, lig)
    E, G, _ = s.score_poses(d, grad=True)
    assert_ref(E, G, ref_batch(oracle, sysm, d, grad=True))


def test_edge_too_long_status(oracle, scorer_factory, small):
    from mmo_gb300.ff import TooLong

    n = 22
    xyz = np.array([[i * 1.22, 0.8 * (i % 2), 0.0] for i in range(n)])
    from mmo_gb300.topology import build_ligand

    lig = build_ligand("chain", xyz - xyz.mean(0), np.zeros(n), np.full(n, 6, np.int32),
                       [(i, i + 1) for i in range(n - 1)])
    s = scorer_factory(small.pocket, lig)
    d = np.zeros((3, 6 + lig.nrb), np.float32)
    d[1, 6:] = np.pi / 2  # folded: not too long
    E, _, st = s.score_poses(d)
    _, st64 = oracle.apply_config(lig, d[0].astype(np.float64))
    assert st[0] == st64 == 1
    assert [int(v) for v in st] == [int(oracle.apply_config(lig, c.astype(np.float64))[1])
                                    for c in d]
    with pytest.raises(TooLong):
        s.score_config(d[0])


def test_edge_close_contact_clamp(oracle, scorer_factory):
    # a ligand atom on top of a protein atom: r clamped to 0.01 A, finite energy
    prot = Mol("p", np.array([0.0, 5.0]), np.zeros(2), np.zeros(2), np.array([0.3, -0.2]),
               np.array([6, 8], np.int32))
    lig = Mol("l", np.zeros(1), np.zeros(1), np.zeros(1), np.array([0.1]),
              np.array([7], np.int32), None, np.zeros((1, 1), np.int32))
    s = scorer_factory(prot, lig)
    d = np.array([[0.0, 0.0, 0.004, 0, 0, 0], [0.0, 0.0, 0.5, 0, 0, 0]], np.float32)
    E, G, st = s.score_poses(d, grad=True)
    sysm = synth.System("clamp", prot, lig, d)
    ref = ref_batch(oracle, sysm, d, grad=True)
    assert np.all(np.isfinite(E)) and not np.any(st & 2)
    assert_ref(E, G, ref)


def test_ragged_batch_sizes(oracle, scorer_factory, batch):
    s = scorer_factory(batch.pocket, batch.ligand)
    for B in (2, 31, 33, 129, 255):
        d = batch.poses[:B]
        E, _, _ = s.score_poses(d)
        if B <= 33:
            assert_ref(E, None, ref_batch(oracle, batch, d))
        Efull, _, _ = s.score_poses(batch.poses)
        assert np.abs(E - Efull[:B]).max() <= 1e-6 * np.abs(Efull[:B]).max()


# -- full-size workload through size-independent properties ------------------------

def test_full_size_energy_batch(oracle, scorer_factory):
    """65,536 poses: 4,096 of them against the oracle under the energy
    contract, and the batch against its own poses in another order."""
    big = synth.pose_batch(n_poses=65536, seed=1)
    s = scorer_factory(big.pocket, big.ligand)
    E, _, st = s.score_poses(big.poses)
    assert np.all(np.isfinite(E))
    idx = np.random.default_rng(0).choice(len(E), 4096, replace=False)
    ref = ref_batch(oracle, big, big.poses[idx])
    assert_ref(E[idx], None, ref, st[idx])
    perm = np.random.default_rng(1).permutation(len(E))
    Ep, _, _ = s.score_poses(big.poses[perm])
    assert np.abs(Ep - E[perm]).max() <= 1e-6 * np.abs(E).max()
